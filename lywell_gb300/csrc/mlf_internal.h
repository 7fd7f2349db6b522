// Internal state of an MLFMA context: host tables built once at set-up and
// their device copies.  Layouts (all device arrays in HBM, box-major):
//   fields  C/B/A of level n : double2[nb_n][2][K_n]   (reference campoC/B/A is
//                                (K,2,nb) column-major: the same bytes)
//   patterns R               : double2[N][2][K_leaf] in leaf-box order
//                                (basis j of the box-sorted list = perm[j])
//   translation tables T     : double2[ntrans_n][K_n]
//   near field               : CSR rows in basis order, float2 values
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/lywell_mlfma.h"

namespace mlf {

struct TcState;   // tensor-core near-field engine (mlf_tc.cu)

// Device allocations of one call, released when the call returns (error
// returns included).
struct DevScope {
    std::vector<void*> ptrs;
    DevScope() = default;
    DevScope(const DevScope&) = delete;
    DevScope& operator=(const DevScope&) = delete;
    template <class T>
    cudaError_t alloc(T** p, size_t bytes) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, bytes);
        *p = static_cast<T*>(q);
        if (e == cudaSuccess) ptrs.push_back(q);
        return e;
    }
    ~DevScope() {
        for (void* q : ptrs) cudaFree(q);
    }
};

constexpr double PI = 3.141592653589793;
constexpr double MU = 1.2566370614E-6;
constexpr double EPSI = 8.8541878176E-12;
constexpr int SEP_SLAB = 8;   // coarse theta rows per CTA in the separable upward pass

struct Phys {
    double lambda, w, kappa, vp, smue;
};
Phys phys_from_lambda(double lambda);

struct Level {
    int nb = 0, L = 0, K = 0, nth = 0, nph = 0;
    double side = 0;
    std::vector<double> centre;   // nb*3
    std::vector<int> parent;      // nb (0-based, -1 at level 1)
    std::vector<int> child_ptr;   // nb+1 (children at level+1 are contiguous)
    std::vector<int> octant;      // nb: 0..7 position relative to the parent centre
    // sampling (level >= 3)
    std::vector<double> kap, ath, aph, ang, wq;
    // far interactions (level >= 3)
    std::vector<int> far_ptr, far_src, far_tid;
    int ntrans = 0;
    std::vector<double> rab;      // ntrans*3
    // interpolation from level+1 (fine) to this level (coarse), 3 <= level < nlev
    std::vector<double> iw;       // K*9
    std::vector<int> iidx;        // K*9 (0-based fine sample)
    // transposed table for anterpolation: for fine sample q, entries
    // [ant_ptr[q], ant_ptr[q+1]) of (coarse sample, weight) in (row, tap) order
    std::vector<int> ant_ptr, ant_row;
    std::vector<double> ant_w;
    // the same stencil in separable form: 3 fine theta rows per coarse theta,
    // 3 fine phi columns per coarse phi, and the transposed lists
    std::vector<int> sth, sph;          // L*3, 2L*3 (0-based fine indices)
    std::vector<double> wth, wph;       // L*3, 2L*3
    std::vector<int> thT_ptr, thT_row;  // per fine theta: coarse rows
    std::vector<double> thT_w;
    std::vector<int> phT_ptr, phT_row;  // per fine phi: coarse columns
    std::vector<double> phT_w;

    // device
    double2 *dC = nullptr, *dB = nullptr, *dA = nullptr;
    double2* dT = nullptr;
    double* dwq = nullptr;
    int *dfar_ptr = nullptr, *dfar_src = nullptr, *dfar_tid = nullptr;
    int *dsth = nullptr, *dsph = nullptr, *dthT_ptr = nullptr, *dthT_row = nullptr, *dphT_ptr = nullptr,
        *dphT_row = nullptr;
    double *dwth = nullptr, *dwph = nullptr, *dthT_w = nullptr, *dphT_w = nullptr;
    double2* dshift = nullptr;    // 8*K: exp(+j k khat . r_oct) for the 8 child octants
    int *dchild_ptr = nullptr, *dparent = nullptr, *doctant = nullptr;
    double *dkap = nullptr, *dath = nullptr, *daph = nullptr, *dcentre = nullptr;
    int fcap = 0;                 // right-hand sides the field buffers hold
};

// FP32 copies of the operator tables and FP32 fields (mixed-precision solve)
struct Mixed32 {
    int ready = 0, fcap = 0;
    float2* R = nullptr;
    float2* xf = nullptr;
    float2* xT = nullptr;             // box-sorted row-major copy of the input block (near blocks)
    struct Lv {
        float2 *T = nullptr, *shift = nullptr, *C = nullptr, *B = nullptr, *A = nullptr;
        float* wq = nullptr;
        float *wth = nullptr, *wph = nullptr, *thT_w = nullptr, *phT_w = nullptr;
        // translation by groups of G = 2 (grp[0]) or 4 (grp[1]) consecutive boxes:
        // merged far lists, sources ascending, tid = the source's translation
        // index for each box of the group (-1: not far)
        struct Grp {
            int *ptr = nullptr, *src = nullptr, *tid = nullptr;
        } grp[2];
    } lv[32];
};

struct Ctx {
    int dev = 0;
    int dense = 0;                    // dense MoM operator instead of the octree (MLF_FLAG_DENSE_MOM)
    double2* dZdense = nullptr;       // N x N row-major, FP64
    int mv_prec = 0;                  // operator precision used by device_matvec: 0 FP64, 1 FP32
    int gmres_m = 0;                  // restart length of the mixed-precision GMRES cycles (0: automatic)
    int gs_passes = 1;                // classical Gram-Schmidt passes per Arnoldi step (1 or 2)
    int tr_group = 0;                 // FP32 translation: boxes per thread (1, 2, 4; 0: 2 for one column, else 4)
    int tr_cols = 0;                  // ... and columns per thread for grouped boxes (1, 2, 4; 0: 2 with 4 boxes, else 4)
    int basis_bits = 32;              // Krylov basis storage of the mixed solve: 32 (FP32) or 16 (FP16)
    int stag_window = 0;              // stagnation window in iterations (0: off): a column whose residual
                                      // sets no new minimum within this many iterations stops as stagnated
    Mixed32 m32;
    cudaStream_t stream = nullptr;
    std::string err;
    Phys ph{};
    double ladomax = 0.5;
    int flags = 0;
    int N = 0, T = 0, P = 0;
    // geometry (host, 0-based indices)
    std::vector<double> p_coord, t_baric, t_baric_sub, e_long, e_centro;
    std::vector<int> e_t, e_po;
    int nlev = 0;
    Level lv[32];
    double root_centre[3]{}, root_side = 0;
    // leaf boxes
    std::vector<int> box_ptr, box_bases, box_of;
    std::vector<int> near_ptr, near_bases;
    std::vector<int> nbox_ptr, nbox_list;   // near leaf boxes of each leaf box, ascending
    // near field as dense box-pair blocks (multi-right-hand-side FP32 operator):
    // block e = (i, nbox_list[e]) holds Z(rows of box i, columns of box j)
    // column-major at Zblk + blk_off[e]; tiles = (box, first row) of each
    // 64-row tile of the leaf boxes
    int blk_ok = 0, nblk_tiles = 0;
    int blk_cols = 0;                 // box-block tile width: 0 = by nrhs, else 8, 32 or 64 (autotuner)
    int blk_engine = -1;              // multi-column engine: 0 box-block FP32 FMA, 1 box-block mma.sync
                                      // 3xTF32, 2 warp per basis with a per-box receive, 3 warp per basis
                                      // throughout, 4 box blocks on tcgen05 (near field, leaf
                                      // aggregation and receive); -1 by mean leaf-box size
    TcState* tc = nullptr;            // engine 4's operand layouts and tensor maps, built on first use
    int lu_big_min = 1024;            // neighbourhood inverse: smallest box for the many-CTA LU (0: none)
    int lu_big_last = 0;              //   boxes that took it in the last build
    void* mix_ws = nullptr;           // workspace of the mixed-precision solve (Krylov basis and vectors),
    size_t mix_ws_bytes = 0;          //   kept between solves, grown on demand
    int* djas = nullptr;              // near CSR columns as box-sorted positions (warp engine)
    float2* dZblk = nullptr;
    long long* dblk_off = nullptr;
    int *dnbox_ptr = nullptr, *dnbox_list = nullptr;
    int2* dblk_tiles = nullptr;
    int* dblk_entry = nullptr;        // leaf box of each block entry
    float2* dMinvblk = nullptr;       // FP32 neighbourhood inverse as near-pattern blocks (batched apply)
    long long nnz = 0;
    std::vector<int> ia, ja;          // 0-based CSR
    // device: leaf
    double2* dR = nullptr;            // patterns, box order
    int *dperm = nullptr, *dbox_ptr = nullptr, *dbox_of_sorted = nullptr;
    int *dia = nullptr, *dja = nullptr;
    float2* dZ = nullptr;
    double2* dZd = nullptr;           // the same near values as complex(8)
    // device geometry for set-up kernels and RCS
    double *dp_coord = nullptr, *dt_baric = nullptr, *dt_baric_sub = nullptr, *de_long = nullptr,
           *de_centro = nullptr;
    int *de_t = nullptr, *de_po = nullptr;
    // ILU0 (MSR layout, 1-based content like the reference)
    int ilu_ok = 0;
    std::vector<float2> alu;
    std::vector<int> jlu, ju;
    float2* dalu = nullptr;
    int *djlu = nullptr, *dju = nullptr;
    // neighbourhood-inverse preconditioner (near CSR pattern)
    double2* dMinv = nullptr;         // CSR values, or compact own-box blocks when nearinv_own
    long long* dboff = nullptr;       // own-box block offsets
    float2* dMinv32 = nullptr;        // FP32 copy for the FP32 inner solves
    double2* dMinv_base = nullptr;    // the exact neighbourhood inverse kept under a learned correction
    long long minv_len = 0;
    float2* dpre_xs = nullptr;        // box-sorted copy of the preconditioner input (blocks of columns)
    size_t pre_xs_cap = 0;
    int nearinv_ok = 0, nearinv_own = 0;
    int nearinv_bits = 0;             // 64: FP64 elimination, 32: blocked FP32 LU, 0: by neighbourhood size
    int learned = 0;                  // own-box blocks installed from the learned network
    // level schedule of the triangular solves
    std::vector<int> lvl_ptr_f, lvl_rows_f, lvl_ptr_b, lvl_rows_b;
    int *dlvl_rows_f = nullptr, *dlvl_rows_b = nullptr;
    // scratch vectors for the solver (grown on demand)
    size_t work_cap = 0;
    double2* dwork = nullptr;
    double* dscal = nullptr;          // device scalars
    size_t scal_cap = 0;
    int* dflags = nullptr;
    size_t io_cap = 0;
    double2 *dx_io = nullptr, *dy_io = nullptr;
    // profiling
    int last_nrhs = 1;
    std::vector<double> cgs_hist;     // ||r||/||b|| per iteration, [it * nrhs + col]
    int cgs_hist_nrhs = 0;
    int profiling = 0;
    cudaEvent_t ev[8]{};
    float stage_ms[5]{};
    // mixed solve phases, accumulated while profiling: preconditioner,
    // FP32 operator, orthogonalisation, total
    cudaEvent_t sev[4]{};
    double solve_ms[7]{};             // last profiled mixed solve: precond, FP32 operator, orthogonalisation,
                                      // wall total, FP64 residuals, provisional FP32 residual (ms), outer steps
};

// host set-up (mlf_setup.cpp)
int fetch_near_values(Ctx* c, std::vector<float2>& out);  // device near values -> host
int build_octree(Ctx* c);          // levels, boxes, lists, interpolation tables
int build_fmm(Ctx* c);             // single-level FMM grid as a one-level tree (nlev = 3)
void sph_bessel(int nmax, double x, double* j, double* y);
void binomial_squares(int nmax, std::vector<double>& out);  // (n!/(i!(n-i)!))^2, [n*(nmax+1)+i]
int ilu0_factor(Ctx* c);           // host ILU(0), fills alu/jlu/ju, returns ierr
// ILU(0) of an n x n CSR matrix (0-based ia/ja, columns ascending in each row)
// into MSR arrays with 1-based content (alu, jlu: nnz + 2 entries, ju: n + 1;
// element 0 unused); returns 0 or the zero-pivot row (1-based)
int ilu0_msr(int n, const int* ia, const int* ja, const float2* a, float2* alu, int* jlu, int* ju);
int ilut_factor(Ctx* c, int lfil, double tol);  // host ILUT, same MSR layout
void ilu_levels(Ctx* c);           // level schedules of the forward/backward sweeps

// device set-up and operators (mlf_device.cu)
int device_setup(Ctx* c);          // uploads tables, computes T, patterns, near field
int device_set_near(Ctx* c, const float2* host_vals);   // replace the near values, drop what derives from them
void device_free(Ctx* c);
int ensure_fields(Ctx* c, int nrhs);
int configure_kernels(Ctx* c);
int ensure_work(Ctx* c, size_t n_double2);
int device_matvec(Ctx* c, const double2* x, double2* y, int nrhs, int ld, cudaStream_t s);
int fp64_matvec_launch(Ctx* c, const double2* x, double2* y, int nrhs, int ld, cudaStream_t s,
                       double2* const* Cf, double2* const* Bf, double2* const* Af, cudaEvent_t* ev);
int device_ilu_upload(Ctx* c);
int device_ilu_solve(Ctx* c, const double2* y, double2* x, cudaStream_t s);
int device_cgs(Ctx* c, const double2* b, const double2* x0, double tol, int maxit, int nrhs,
               double2* x, int* iters, double* relres, int precond, int* status);
int device_nearinv_setup(Ctx* c, int* bad_box, int own_only);
int nbhd_inverse_lu32(Ctx* c, int nownmax, int* bad_box);   // blocked FP32 LU (mlf_nbhd_lu.cu)
// the same over 2-ring lists (dense Z, N x N row-major complex(4)): rows of the
// own bases on the near pattern into M2 (the learned preconditioner's targets)
int ring_inverse_lu32(Ctx* c, const float2* Zd, const long long* off, const int* len, const int* bases,
                      const std::vector<int>& len_host, const std::vector<long long>& off_host, int nownmax,
                      float2* M2, int* bad_box);
int device_matvec32(Ctx* c, const double2* x, double2* y, int nrhs, int ld, cudaStream_t s);
int device_matvec32_from32(Ctx* c, const float2* x32, double2* y, int nrhs, cudaStream_t s);
int device_nearinv_apply32(Ctx* c, const float2* y, float2* x, int nrhs, cudaStream_t s);
void mixed_free(Ctx* c);
int upload_geometry(Ctx* c);
int dense_setup(Ctx* c);
int dense_matvec(Ctx* c, const double2* x, double2* y, int nrhs, int ld, cudaStream_t s);
int need_tree(Ctx* c);
int device_blk_pack(Ctx* c, const double2* x, const float2* x32, int ld, int nrhs, float2* xs, cudaStream_t s);
int device_near_blocks32(Ctx* c, const float2* xs, int ld, int nrhs, double2* y, cudaStream_t s);
int device_agg_blocks32(Ctx* c, const float2* R, int K, const float2* xs, int nrhs, float2* C, cudaStream_t s);
int device_recv_blocks32(Ctx* c, const float2* R, int K, const float2* A, float facy, int nrhs, int ld, double2* y,
                         cudaStream_t s);
int device_own_blocks32(Ctx* c, const long long* boff, const float2* M, const float2* xs, int nrhs, float2* out,
                        cudaStream_t s);
void near_blocks_free(Ctx* c);
// warp engine (mlf_nearwarp.cu): one warp per basis, for small leaf boxes
void warp_engine_free(Ctx* c);
int blk_engine_of(const Ctx* c);   // the engine in force (resolves -1)
inline bool warp_engine(int e) { return e == 2 || e == 3; }
// tensor-core engine (mlf_tc.cu)
int device_blocks_ready(Ctx* c);   // box-pair blocks of the near field built
int device_near_tc(Ctx* c, const float2* xs, int ld, int nrhs, double2* y, cudaStream_t s, bool x_packed = false);
int device_agg_tc(Ctx* c, const float2* R, int K, const float2* xs, int nrhs, float2* C, cudaStream_t s);
int device_recv_tc(Ctx* c, const float2* R, int K, const float2* A, float facy, int nrhs, int ld, double2* y,
                   cudaStream_t s);
int device_near_pattern_tc(Ctx* c, const float2* Mblk, const float2* xs, int nrhs, float2* out, cudaStream_t s);
void tc_drop_precond(Ctx* c);      // drop the preconditioner's tensor-core operand (its blocks changed)
int tc_check(Ctx* c);              // MLF_E_CUDA if a tensor-core CTA gave up a wait since the last check
void tc_free(Ctx* c);
int device_agg_warp32(Ctx* c, const float2* R, int K, const float2* xs, int nrhs, float2* C, cudaStream_t s);
int device_recv_near_warp32(Ctx* c, const float2* R, int K, const float2* A, float facy, const float2* xs, int nrhs,
                            int ld, double2* y, cudaStream_t s);
int device_near_pattern_warp32(Ctx* c, const float2* M, const float2* xs, int nrhs, float2* out, cudaStream_t s);
int device_own_warp32(Ctx* c, const long long* boff, const float2* M, const float2* xs, int nrhs, float2* out,
                      cudaStream_t s);
int device_blocks_from_csr(Ctx* c, const float2* csr, float2** blk);
int device_near_pattern_apply32(Ctx* c, const float2* Mblk, const float2* xs, int nrhs, float2* out, cudaStream_t s);
int lp_tokens(Ctx* c, int with_target, float* X, float* T, long long cap, long long* ntok, int* bad_box);
int autotune_block(Ctx* c, const int* cand, int ncand, int* best_block, int* best_cols, int* best_engine,
                   float* per_rhs_ms);
int device_solve_mixed(Ctx* c, const double2* b, const double2* x0, double tol, int maxit, int nrhs, double2* x,
                       int* iters, double* relres, int precond, int* status, double inner_tol, int* outer);
int device_nearinv_apply(Ctx* c, const double2* y, double2* x, int nrhs, cudaStream_t s);
int device_excitation(Ctx* c, const double* dirs, const double2* pols, double2 ctte, int nrhs,
                      double2* b);
int device_rcs(Ctx* c, const double2* I, const double2* pol, double2 ctte, const double* th,
               const double* ph, int nang, double* sigma);
int device_rcs_cols(Ctx* c, const double2* X, size_t ldx, int ncol, const double2* pols, double2 ctte,
                    const double* th, const double* ph, double* sigma);

bool cuda_ok(Ctx* c, cudaError_t e, const char* what);

}  // namespace mlf

struct mlf_ctx {
    mlf::Ctx c;
};
