/*
 * lywell_mlfma.h — C ABI of the GB300 (sm_103a) MLFMA iterative solve.
 *
 * A drop-in for MLFMAxwell's solve path (gabsantamaria/lywell, Fortran 90):
 * the MLFMA matvec of modMLFMA, CGS + ILU0 of modIterativo and the RCS
 * far-field sum of modRCS.  Every entry point takes plain pointers and sizes
 * (no torch or CUDA types), returns an int status (MLF_OK = 0) and never
 * prints.  A Fortran host binds these with ISO_C_BINDING; the interface
 * module is shipped as lywell_gb300/fortran/lywell_mlfma_cabi.f90.
 *
 * Conventions
 *  - Complex numbers are interleaved (re, im) doubles: a complex(8) array of
 *    length n is `double[2n]`, exactly Fortran's complex(kind=8) layout.
 *  - Geometry arrays are Fortran column-major, e.g. e_centro(3, N) is
 *    `double[3*N]` with the three coordinates of edge i at [3i .. 3i+2].
 *  - Index arrays are 1-based int32, matching Fortran integer(4).
 *  - Multi-RHS blocks are column-major (n x nrhs) with leading dimension ld.
 *  - A context is bound to the CUDA device that was current at mlf_init and
 *    owns one CUDA stream; calls on one context must not overlap.
 */
#ifndef LYWELL_MLFMA_H
#define LYWELL_MLFMA_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mlf_ctx mlf_ctx;

enum {
    MLF_OK = 0,
    MLF_E_ARG = -1,        /* invalid argument */
    MLF_E_TOO_SMALL = -2,  /* nivel_max <= 3: the reference stops here (modMLFMA.f90:195-198) */
    MLF_E_CUDA = -3,       /* CUDA runtime error (message in mlf_last_error) */
    MLF_E_NOMEM = -4,
    MLF_E_TABLE = -5,      /* more than 316 distinct translation vectors on a level */
    MLF_E_STATE = -6,      /* e.g. ILU0 apply before a successful mlf_ilu0 */
    MLF_E_NOT_FINITE = -7, /* NaN/Inf met in the solver */
    MLF_E_NO_DEVICE = -8
};

/* mlf_cgs outcome codes (written to *status_out) */
enum {
    MLF_CGS_CONVERGED = 0,
    MLF_CGS_MAXIT = 1,
    MLF_CGS_BREAKDOWN = 2,   /* rho == 0: the reference exits silently (modIterativo.f90:392-395) */
    MLF_CGS_NOT_FINITE = 3,
    MLF_CGS_STAGNATED = 4    /* no progress over the stagnation window */
};

/* mlf_cgs preconditioners */
enum {
    MLF_PRECOND_NONE = 0,
    MLF_PRECOND_ILU0 = 1,     /* ilu0C + lusol0C, as the reference */
    MLF_PRECOND_NEARINV = 2   /* neighbourhood inverse (mlf_nearinv); no counterpart in the reference */
};

/* mlf_init flags */
enum {
    MLF_FLAG_LEGENDRE_RECURRENCE = 1, /* P_l by the three-term recurrence instead of the
                                         reference's explicit binomial sum */
    MLF_FLAG_DENSE_MOM = 2            /* dense MoM operator (MoM + MatxVec_MoM, modMoM.f90:85-128,
                                         273-277): the N x N matrix in FP64 on the device, no
                                         octree (ladomax ignored); matvec, CGS without
                                         preconditioner, excitation, RCS and the FP64 monostatic
                                         modes work, octree-based calls return MLF_E_STATE */,
    MLF_FLAG_FMM = 4                  /* single-level FMM (inicializar_FMM + MatxVec_FMM,
                                         modFMM.f90:170-268, 904-963) instead of MLFMA: one grid
                                         level of boxes of side <= ladomax * lambda (the
                                         reference uses ladomax = 0.5), far pairs translated
                                         directly, near field and preconditioners as MLFMA's */
};

/* Build the RWG basis from a triangle soup, reproducing the reference's
 * edge order (modRWG.f90:8-174, modReadStl.f90:1444-1533) and triangle
 * geometry (modRWG.f90:270-328).  Call once with all outputs NULL to get
 * *N_out and *P_out, then again with arrays of these sizes:
 *   p_coord(3,P) t_p(3,T) e_p(2,N) e_t(2,N) e_po(2,N) e_long(N) e_centro(3,N)
 *   t_area(T) t_baric(3,T) t_baric_sub(3,9,T)        (index arrays 1-based)
 * tris: double[T*9], triangle-major, vertex, xyz (the order of an STL file).
 * Replaces: cap_geom (main.f90:1430-1468) -> obtener_p_t, parametros_rwg,
 * hallar_geometria_rwg. */
int mlf_rwg_build(const double* tris, int T, int* N_out, int* P_out,
                  double* p_coord, int* t_p, int* e_p, int* e_t, int* e_po,
                  double* e_long, double* e_centro, double* t_area,
                  double* t_baric, double* t_baric_sub);

/* Set up the octree, sampling, interpolation and translation tables,
 * radiation patterns and the complex(4) near-field CSR on the current CUDA
 * device.  Copies what it needs; the caller keeps ownership of the arrays.
 * lambda: wavelength in metres (global `lambda`, setlambda in
 * modGlobalParam.f90:52-61); ladomax: conf%criterio_ladomax.
 * t_area, t_p, e_p and t_normal are accepted for signature parity and not
 * needed (t_normal only enters the reference through (1-alphaCFIE) = 0).
 * Replaces: inicializar_MLFMA (modMLFMA.f90:113-275). */
int mlf_init(mlf_ctx** ctx, const double* e_centro, int N, const int* e_t, const int* e_po,
             const double* e_long, const double* t_area, const double* t_baric,
             const double* t_baric_sub, const double* p_coord, const int* t_p, const int* e_p,
             int P, int T, const double* t_normal, double lambda, double ladomax, int flags);

/* Release the context.  Replaces: destruir_MLFMA (modMLFMA.f90:85-110). */
void mlf_free(mlf_ctx* ctx);

/* Last error message of the context (or of the last failed mlf_init when
 * ctx is NULL). */
const char* mlf_last_error(const mlf_ctx* ctx);

/* y = Z_MLFMA x for nrhs columns, host arrays (complex(8), n x nrhs, ld >= N).
 * Includes the host<->device copies.
 * Replaces: MatxVec_MLFMA (modMLFMA.f90:1901-1946). */
int mlf_matvec(mlf_ctx* ctx, const double* x, double* y, int nrhs, int ld);

/* Same on device-resident arrays; stream NULL = the context's stream. */
int mlf_matvec_device(mlf_ctx* ctx, const void* x_dev, void* y_dev, int nrhs, int ld,
                      void* stream);

/* Allocation-free variant of mlf_matvec_device for one right-hand side
 * (x, y: device arrays of N complex(8)).  It has no counterpart in the
 * reference.  It is for callers that must not allocate device memory
 * while they solve: hosts that record their iteration into a CUDA graph,
 * or hosts whose device memory belongs to another runtime or a fixed
 * pool.  It issues the same FP64-operator launches as mlf_matvec_device,
 * with bit-identical results, but keeps the multipole fields in one fixed
 * 64 MiB device array inside the library (held by every GPU that loads it,
 * until exit) and never calls cudaMalloc/cudaFree.  Octrees whose C, B and
 * A fields together exceed 4,194,304 complex values are rejected with
 * MLF_E_ARG.  The first call on a device looks up the array's address and
 * keeps it for the process; make it before any stream capture.  All calls
 * share the array: calls that overlap on the GPU race.  The caller's
 * current device is restored on return.  stream NULL = the context's
 * stream. */
int mlf_matvec_device_noalloc(mlf_ctx* ctx, const void* x_dev, void* y_dev, void* stream);

/* Near-field block in CSR (1-based), values complex(4) interleaved floats.
 * Call with a/ja/ia NULL to get *nnz.  Replaces the public module data
 * Zesparcida_MLFMA, ja_MLFMA, ia_MLFMA, n_esparcida_MLFMA (modMLFMA.f90:12, 30-32). */
int mlf_near_csr(mlf_ctx* ctx, long long* nnz, float* a, int* ja, int* ia);

/* ILU(0) of the near-field block, complex(4) factors kept on the device.
 * *ierr_row = 0 on success, k > 0 when a zero pivot was met at row k.
 * Replaces: crear_precond ILU0 branch (main.f90:851-902) -> ilu0C
 * (modIterativo.f90:1805-1976). */
int mlf_ilu0(mlf_ctx* ctx, int* ierr_row);

/* ILU(0) of a host CSR matrix with the reference routine's own arguments:
 * ilu0C(n, a, ja, ia, alu, jlu, ju, iw, ierr) (modIterativo.f90:1805-1976),
 * the work array iw kept inside.  a: nnz complex(4) values (interleaved
 * floats); ja, ia: 1-based CSR, columns strictly ascending in each row.
 * Outputs in ilu0C's MSR layout: alu (nnz+1 complex(4)), jlu (nnz+1), ju (n).
 * *ierr = 0, or k > 0 when a zero pivot was met at row k (a row without a
 * diagonal entry counts as one).  A malformed CSR (ia(1) != 1, ia
 * decreasing, a column outside 1..n or out of order) returns MLF_E_ARG and
 * names the row in mlf_last_error(NULL); the reference checks none of this.
 * Host code only: no CUDA device is needed. */
int mlf_ilu0_csr(int n, const float* a, const int* ja, const int* ia, float* alu, int* jlu, int* ju, int* ierr);

/* Overwrite the context's complex(4) near-field values (nnz, in the order of
 * mlf_near_csr), as the reference's host may overwrite its public
 * Zesparcida_MLFMA (modMLFMA.f90:12) before crear_precond.  ILU and
 * neighbourhood preconditioners built earlier are dropped: build them again. */
int mlf_set_near_values(mlf_ctx* ctx, const float* a);

/* ILUT (dual threshold) of the near-field block, the reference's default
 * preconditioner: lfil = ceiling(0.01 fill_in_prc N), drop tolerance
 * droptol (ilut.fillin / ilut.droptol; defaults 5 and 1e-3).  The factors
 * replace any ILU0 factors and are applied by mlf_ilu0_solve / precond kind
 * MLF_PRECOND_ILU0.  *ierr as ilutC: 0, zero-pivot row k > 0, or -1..-5.
 * Replaces: crear_precond ILUT branch (main.f90:904-960) -> ilutC
 * (modIterativo.f90:2432-2883). */
int mlf_ilut(mlf_ctx* ctx, double fill_in_prc, double droptol, int* ierr);

/* Export the ILU0 / ILUT factors in the reference's MSR layout (alu:
 * complex(4) interleaved, jlu: same length = jlu(N+1)-1 entries, nnz+1 for
 * ILU0; ju: N; 1-based).  mlf_ilu_size gives that length. */
int mlf_ilu_size(mlf_ctx* ctx, long long* len);
int mlf_ilu0_factors(mlf_ctx* ctx, float* alu, int* jlu, int* ju);

/* x = (LU)^-1 y for nrhs host columns.  Replaces: lusol0C
 * (modIterativo.f90:504-560). */
int mlf_ilu0_solve(mlf_ctx* ctx, const double* y, double* x, int nrhs);

/* Right-preconditioned CGS on the MLFMA operator, one or more right-hand
 * sides (each solved with its own scalars; converged columns retire).
 * b, x0, x: host complex(8) n x nrhs (ld = N).  x0 may be NULL (zero guess).
 * precond_kind: MLF_PRECOND_NONE, MLF_PRECOND_ILU0 (mlf_ilu0 must have
 * succeeded) or MLF_PRECOND_NEARINV (mlf_nearinv must have succeeded).
 * maxit: iteration cap (the reference has none).  Per column outputs:
 * iters[nrhs], relres[nrhs] (true-recursion residual ||r||/||b||),
 * status_out[nrhs] (MLF_CGS_*).
 * Replaces: CGSold (modIterativo.f90:331-493). */
int mlf_cgs(mlf_ctx* ctx, const double* b, const double* x0, double tol, int maxit, int nrhs,
            double* x, int* iters, double* relres, int precond_kind, int* status_out);

/* Stagnation detector of mlf_cgs, mlf_solve and mlf_monostatic: a column
 * whose relative residual has set no new minimum within `window` iterations
 * stops with status MLF_CGS_STAGNATED (mlf_solve mode 1: the FP64 residual
 * of each refinement step, the window counted in inner steps).  0, the
 * default, turns it off, as in the reference, whose CGSold iterates until
 * it converges (modIterativo.f90:384-490). */
int mlf_set_stagnation(mlf_ctx* ctx, int window);

/* Solve Z_MLFMA x = b for nrhs columns.  mode 0: CGS on the FP64 operator
 * (exactly mlf_cgs).  mode 1: mixed precision — iterative refinement whose
 * residual r = b - Z x is formed with the FP64 operator and whose
 * corrections come from one right-preconditioned GMRES(m) cycle (m set by
 * mlf_set_gmres_restart, or by default 1600 while the basis fits in 16 GB,
 * down to 800 for wide blocks) on the FP32
 * operator (patterns, translations, interpolation and fields in float;
 * complex(4) near field), stopped when its residual estimate drops below
 * inner_tol ||b|| (<= 0: 0.9 tol).  Stops when the FP64 residual satisfies
 * ||b - Z x|| < tol ||b||, the same test as CGSold (modIterativo.f90:472).
 * The first cycle's right-hand side needs no FP64 operator: it is b itself
 * without x0, and b - Z32 x0 (FP32 operator) with x0, on which no column is
 * declared converged.  iters: inner GMRES steps (FP32 matvecs) per column;
 * *outer: refinement cycles.  No counterpart in the reference for mode 1. */
int mlf_solve(mlf_ctx* ctx, const double* b, const double* x0, double tol, int maxit, int nrhs,
              int precond_kind, int mode, double inner_tol, double* x, int* iters, double* relres,
              int* status_out, int* outer);

/* Restart length m of mode 1's GMRES cycles (4..2000, or 0 = automatic:
 * 1600 while the basis fits in 16 GB, down to 800; memory (m+1) N nrhs
 * FP32 complex values). */
int mlf_set_gmres_restart(mlf_ctx* ctx, int m);

/* Classical Gram-Schmidt passes per Arnoldi step of mode 1 (1, the default:
 * one pass, FP32 orthogonality losses left to the FP64 refinement; 2 = CGS2,
 * twice the basis traffic). */
int mlf_set_gs_passes(mlf_ctx* ctx, int passes);

/* Krylov basis storage of mode 1: 32 (FP32, the default) or 16 (FP16, each
 * unit basis column stored scaled by sqrt(N), so entries stay within FP16's
 * range).  FP16 halves the Gram-Schmidt traffic, which streams the basis
 * twice per step; the arithmetic stays FP32 with FP64 reductions, and the
 * FP64 refinement keeps the same stopping test.  No counterpart in the
 * reference. */
int mlf_set_basis_precision(mlf_ctx* ctx, int bits);

/* FP32 translation stage (mode 1 and mlf_matvec32*): boxes = 2 or 4 = one
 * thread per sample for that many consecutive boxes over the merged list of
 * their far boxes, each source value read once for all of them; 1 = one box
 * at a time; 0 (the default) = 2 for one column, 4 for blocks of columns.
 * cols = columns per thread with grouped boxes (1, 2 or 4; 0, the default:
 * 2 with 4 boxes, else 4).  The same sums in another order.  No counterpart
 * in the reference. */
int mlf_set_translation_group(mlf_ctx* ctx, int boxes, int cols);

/* Phase times (ms) of the last mixed-precision solve run while profiling was
 * on (mlf_set_profiling): out4 = {preconditioner, FP32 operator,
 * orthogonalisation, wall total}.  No counterpart in the reference. */
int mlf_solve_times(mlf_ctx* ctx, double* out4);

/* The same phases and more, out[0..n-1] of {preconditioner, FP32 operator,
 * orthogonalisation, wall total, FP64 residuals (the outer checks), the
 * provisional FP32 residual of a warm start (ms), outer steps}; n <= 7.
 * The residual phases are timed on the host between stream
 * synchronisations.  No counterpart in the reference. */
int mlf_solve_phases(mlf_ctx* ctx, double* out, int n);

/* Autotuner for batched solves: times the FP32 operator on each candidate
 * block of right-hand sides (candidates[ncand], 1..4096) with each
 * multi-column engine -- both box-block GEMM engines at the tile widths 8, 32
 * and 64 columns, the warp engine (leaf boxes under 96 bases on average) and
 * the tcgen05 engine (16 bases or more) -- and returns
 * the smallest block whose time per right-hand side is within 5 % of the
 * best, with its tile width (0 for a single column or the warp engine) and
 * engine (best_engine, optional: 1 tensor cores (mma.sync), 0 FP32 FMA, 2 or
 * 3 warp engine, 4 tensor cores (tcgen05)); both are kept for later
 * operator and preconditioner calls.
 * per_rhs_ms (optional, ncand) receives the best time per right-hand side of
 * each candidate.  No counterpart in the reference. */
int mlf_autotune_block(mlf_ctx* ctx, const int* candidates, int ncand, int* best_block, int* best_cols,
                       int* best_engine, float* per_rhs_ms);

/* Multi-column engine of the FP32 operator and of the FP32 preconditioner
 * applies on blocks of columns:
 *   1 = box-block GEMMs on tensor cores (mma.sync m16n8k8 TF32 with the
 *       3xTF32 split, within a few 1e-6 of FP32),
 *   0 = box-block GEMMs on FP32 FMAs,
 *   2 = warp engine: one warp per basis over 8 columns, nothing padded (for
 *       leaf boxes of a few tens of bases), the leaf receive by one CTA per
 *       box with the box's fields in shared memory,
 *   3 = warp engine with the leaf receive also one warp per basis,
 *   4 = box-block GEMMs on the fifth-generation tensor cores (tcgen05.mma,
 *       3xTF32, accumulators in tensor memory, operands staged by TMA): the
 *       near field, the leaf aggregation and receive, and the near-pattern
 *       preconditioner, 64 columns per tile,
 *  -1 = by the mean leaf-box size: 2 below 48 bases per box, else 1 (the
 *       default).
 * cols = box-block tile width 8, 32 or 64 (0: by the block's width).
 * mlf_autotune_block sets both.  No counterpart in the reference. */
int mlf_set_block_engine(mlf_ctx* ctx, int engine, int cols);

/* y = Z_MLFMA x with the FP32 operator of mode 1 (host or device arrays);
 * inputs and outputs complex(8). */
int mlf_matvec32(mlf_ctx* ctx, const double* x, double* y, int nrhs, int ld);
int mlf_matvec32_device(mlf_ctx* ctx, const void* x_dev, void* y_dev, int nrhs, int ld, void* stream);

/* Neighbourhood-inverse preconditioner: for every leaf box, the rows of the
 * inverse of its near-field neighbourhood block (the box's near list x
 * itself, entries from the near CSR) that belong to the box's own bases;
 * M has the near CSR's pattern.  No counterpart in the reference, which
 * offers ILU0/ILUT (modIterativo.f90:1805-1976, 2432-2883); on the bodies
 * measured here ILU0 makes CGS diverge while this one cuts the iteration
 * count several-fold.  *bad_box = 0 on success, b+1 when box b's block is
 * singular. */
int mlf_nearinv(mlf_ctx* ctx, int* bad_box);

/* Arithmetic of mlf_nearinv's elimination: 64 = FP64 Gaussian elimination
 * with partial pivoting, one CTA per box; 32 = blocked FP32 LU with partial
 * pivoting (panels of 32 columns, tiled GEMM trailing updates), for
 * neighbourhoods of thousands of unknowns; 0 (the default) = FP64 up to 768
 * unknowns per neighbourhood, FP32 above.  No counterpart in the reference. */
int mlf_set_nearinv_precision(mlf_ctx* ctx, int bits);

/* The FP32 LU gives each box one CTA, so the largest neighbourhoods would set
 * the set-up time alone.  Boxes of at least min_unknowns unknowns whose work
 * (n^3) exceeds three times the remaining boxes' share per CTA are factorised on many CTAs
 * each instead (panel on one CTA; row swaps, U12 and the trailing update over
 * the GPU), on side streams next to the one-CTA-per-box kernel.
 * min_unknowns = 0 turns this off; the default is 1024.  mlf_get_lu_split
 * reads the setting and how many boxes took the many-CTA path in the last
 * build.  No counterpart in the reference. */
int mlf_set_lu_split(mlf_ctx* ctx, int min_unknowns);
int mlf_get_lu_split(mlf_ctx* ctx, int* min_unknowns, int* last_big_boxes);

/* Same with each box's own bases as the neighbourhood (block Jacobi on the
 * near field): cheaper where leaf boxes hold many bases and near lists run
 * into the thousands.  Replaces any previous mlf_nearinv result. */
int mlf_nearinv_own(mlf_ctx* ctx, int* bad_box);

/* Values of M (complex(8), interleaved) in the order of mlf_near_csr
 * (full-neighbourhood mode only). */
int mlf_nearinv_values(mlf_ctx* ctx, double* vals);

/* x = M^-1 y for nrhs host columns with the preconditioner of kind
 * MLF_PRECOND_ILU0 (lusol0C) or MLF_PRECOND_NEARINV. */
int mlf_precond_apply(mlf_ctx* ctx, int precond_kind, const double* y, double* x, int nrhs);

/* x = M32 y: the FP32 copy of the neighbourhood / own-box (or learned)
 * preconditioner that mode 1 of mlf_solve applies in its inner loop; for
 * nrhs > 1 the own-box blocks run as per-box GEMMs.  Complex(8) in and out.
 * No counterpart in the reference. */
int mlf_precond_apply32(mlf_ctx* ctx, const double* y, double* x, int nrhs);

/* Residual history ||r_i||/||b|| of column col of the last mlf_cgs call
 * (the per-iteration line CGSold prints, modIterativo.f90:446-465).
 * *n = number of iterations recorded; up to cap values are copied. */
int mlf_cgs_history(mlf_ctx* ctx, int col, double* hist, int cap, int* n);

/* Plane-wave excitation b(N) for nrhs waves: dirs(3,nrhs) propagation
 * directions, pols(3,nrhs) complex polarisations, ctte complex amplitude.
 * Replaces: generar_onda (main.f90:1488-1525). */
int mlf_excitation(mlf_ctx* ctx, const double* dirs, const double* pols, double ctte_re,
                   double ctte_im, int nrhs, double* b);

/* sigma(theta_a, phi_a) (linear, m^2) of the current I(N) for nang angles,
 * polarisation pol(3) complex and amplitude ctte as given to
 * inicializar_RCS.  Replaces: inicializar_RCS + sigmaRCS + calc_RCS +
 * calc_E (modRCS.f90:23-153). */
int mlf_rcs(mlf_ctx* ctx, const double* I, const double* pol, double ctte_re, double ctte_im,
            const double* theta, const double* phi, int nang, double* sigma);

/* Monostatic RCS sweep.  Replaces: gen_rcs_monostatica (main.f90:967-1089).
 * nang angles phi_a (radians; phis NULL = the reference's grid
 * (a-1) pi / nang), incidence d = (-cos phi, -sin phi, 0), polarisation VV
 * (hh = 0) or HH (hh = 1), backscatter sigma(pi/2, phi_a) (linear) into
 * sigma[nang]; iters/status_out per angle.
 * mode 0: the reference's sequential sweep, CGS on the FP64 operator,
 *         warm start = previous currents x exp(-j k (d_a - d_{a-1}) . r_edge).
 * mode 1: batched, blocks of `block` angles as one multi-RHS FP64 CGS.
 * mode 2: batched mixed precision (mlf_solve mode 1 per block), zero guesses.
 * mode 3: batched mixed precision with mode 0's warm starts: column q of the
 *         block sweeps the contiguous run of angles [q n, (q + 1) n),
 *         n = ceil(nang / block); block k solves the k-th angle of every run,
 *         each column starting from its previous angle's phase-shifted
 *         currents.
 * mode 4: mode 3 with each column's start extrapolated linearly from its
 *         two previous angles' currents, both phase-shifted to the new
 *         direction (x0 = 2 x_{k-1} - x_{k-2}).
 * block <= 0 (modes 1-4): chosen by mlf_autotune_block among 8..128 (modes
 * 3 and 4: at most nang / 4, so that every column sweeps at least four
 * angles).
 * Modes 1-4 have no counterpart in the reference. */
int mlf_monostatic(mlf_ctx* ctx, int nang, const double* phis, int hh, double ctte_re, double ctte_im,
                   double tol, int maxit, int precond_kind, int mode, int block, double* sigma, int* iters,
                   int* status_out);

/* Octree summary for hosts and tests: out[0] = number of levels, out[1] = N;
 * for level l (1-based) out[5l .. 5l+4] = boxes, multipoles L, samples K,
 * distinct translation vectors, far-interaction pairs.  out must hold
 * 5*(levels+1) ints (160 always suffices). */
int mlf_info(mlf_ctx* ctx, int* out, long long* nnz_near);

/* Per-stage device timings of the last mlf_matvec[_device] in ms:
 * out[0] aggregation, [1] interpolation, [2] translation, [3] anterpolation,
 * [4] receive + near.  Only filled when profiling is on (mlf_set_profiling). */
int mlf_set_profiling(mlf_ctx* ctx, int on);
int mlf_stage_times(mlf_ctx* ctx, float* out5);

/* Copy the C / B / A field of one level (complex(8), K x 2 x boxes,
 * the reference's campoC/campoB/campoA layout) after the last matvec.
 * which: 0 = C, 1 = B, 2 = A.  For parity checks of single stages. */
int mlf_debug_field(mlf_ctx* ctx, int level, int which, double* out);

/* ---- Learned near-field preconditioner: the network ------------------------
 * A 16 -> 128 -> 128 -> 2 MLP (ReLU) with hand-written CUDA forward, backward
 * and Adam kernels: BF16 parameters and activations, FP32 accumulation, FP32
 * master weights.  Parameter vector (mlf_mlp_nparam() floats):
 * W1[16][128] b1[128] W2[128][128] b2[128] W3[128][2] b3[2]; norm = mu[16],
 * sd[16] (inputs enter as (x - mu) / sd).  Loss: mean squared error over
 * tokens and outputs.  X, T, Y are device arrays (row-major [ntok][16],
 * [ntok][2]).  No counterpart in the reference. */
typedef struct mlf_mlp mlf_mlp;
int mlf_mlp_create(mlf_mlp** net, int device, unsigned long long seed);
void mlf_mlp_free(mlf_mlp* net);
const char* mlf_mlp_last_error(mlf_mlp* net);
int mlf_mlp_nparam(void);
int mlf_mlp_set_params(mlf_mlp* net, const float* params, const float* norm);
int mlf_mlp_get_params(mlf_mlp* net, float* params, float* norm);
int mlf_mlp_forward(mlf_mlp* net, const float* X, long long ntok, float* Y, void* stream);
int mlf_mlp_grad(mlf_mlp* net, const float* X, const float* T, long long ntok, float* grad, double* loss);
int mlf_mlp_train(mlf_mlp* net, const float* X, const float* T, long long ntok, int steps, int batch, float lr,
                  unsigned long long seed, float* loss_hist);

/* ---- Learned near-field preconditioner: tokens and installation -----------
 * Base: the exact neighbourhood inverse M1 (mlf_nearinv, 27-box
 * neighbourhoods).  The network predicts, per near-field entry (row m,
 * column j), the correction D = M2 - M1 towards the inverse over the 2-ring
 * (125-box) neighbourhood restricted to the same pattern, in units of
 * s_m s_j, s_m = 1/sqrt(Z_mm).  Token features (16 floats, in the near CSR's
 * entry order): Re, Im of s_m Z_mj s_j; Re, Im, |.| of M1_mj / (s_m s_j);
 * [same leaf box]; [m == j]; (r_j - r_m) / lambda (3) and its length; the
 * leaf-cell distance of the two boxes (max norm, Euclidean); n_own / 100 and
 * near boxes / 27 of m's box; 1.  Target (2 floats): Re, Im of
 * D_mj / (s_m s_j), the 2-ring inverses computed on the device (FP32
 * elimination; bodies up to 55 000 unknowns).
 * mlf_lp_tokens needs mlf_nearinv first; X (16 per token) and T (2 per
 * token, with_target only) are device arrays of capacity cap; X = NULL
 * returns the token count (the near nnz) only; *bad_box: first 2-ring block
 * that was singular, 0 if none.
 * mlf_lp_install: M = M1 + scale * s_m s_j net(tokens), on M1's pattern,
 * applied as MLF_PRECOND_NEARINV; repeated installs start from the exact M1;
 * mlf_nearinv restores it.  *nonfinite counts non-finite network outputs
 * (set to zero).  No counterpart in the reference. */
int mlf_lp_tokens(mlf_ctx* ctx, int with_target, float* X, float* T, long long cap, long long* ntok, int* bad_box);
int mlf_lp_install(mlf_ctx* ctx, mlf_mlp* net, float scale, int* nonfinite);

#ifdef __cplusplus
}
#endif
#endif
