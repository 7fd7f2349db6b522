"""Host-side mirror of MLFMAxwell's solve interface over the C ABI.

Names follow the reference so that a driver written against it reads the
same:

==========================  ============================================  =========================
reference (Fortran)          here                                           C ABI
==========================  ============================================  =========================
cap_geom -> parametros_rwg   ``RWG(tris)``                                  mlf_rwg_build
inicializar_MLFMA            ``MLFMA(rwg, lam, ladomax)``                   mlf_init
MatxVec_MLFMA                ``MLFMA.MatxVec_MLFMA(x)`` / ``matvec``        mlf_matvec
Zesparcida_MLFMA, ia, ja     ``MLFMA.near_csr()``                           mlf_near_csr
crear_precond -> ilu0C       ``MLFMA.ilu0C()`` (returns ierr)               mlf_ilu0
ilu0C on a host CSR          ``ilu0C(n, a, ja, ia)``                        mlf_ilu0_csr
lusol0C                      ``MLFMA.lusol0C(y)``                           mlf_ilu0_solve
CGSold                       ``MLFMA.CGSold(b, guess, errmax, ...)``        mlf_cgs
generar_onda                 ``MLFMA.generar_onda(dir, pol, ctte)``         mlf_excitation
inicializar_RCS + sigmaRCS   ``MLFMA.sigmaRCS(I, pol, theta, phi, ctte)``   mlf_rcs
destruir_MLFMA               ``MLFMA.close()``                              mlf_free
==========================  ============================================  =========================

Errors the reference only prints (ILU zero pivot, CGS breakdown) are
returned as values; invalid calls raise :class:`MLFError`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import CGS_STATUS, ENGINES, FLAG_DENSE_MOM, FLAG_FMM, FLAG_LEGENDRE_RECURRENCE, PRECOND, MLFError, load

__all__ = ["RWG", "MLFMA", "MoM", "FMM", "MLFError", "FLAG_LEGENDRE_RECURRENCE", "ajustar_polariz", "direction", "ilu0C"]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _check(code, h=None):
    if code != 0:
        msg = load().mlf_last_error(h)
        raise MLFError(code, msg.decode() if msg else "")


class RWG:
    """RWG basis of a triangle soup ``tris[T, 3, 3]`` in the reference's edge order.

    Arrays are 0-based numpy views for Python users; ``fortran()`` gives the
    1-based arrays the C ABI takes.
    """

    def __init__(self, tris):
        tris = np.ascontiguousarray(tris, dtype=np.float64).reshape(-1, 3, 3)
        L = load()
        T = tris.shape[0]
        # one call with the arrays sized for the bounds (P <= 3T nodes, N <= 3T/2
        # edges: every edge pairs two triangle sides), then trimmed
        Pm, Nm = 3 * T, (3 * T) // 2
        N = C.c_int()
        P = C.c_int()
        p_coord = np.zeros((Pm, 3))
        self.t_p = np.zeros((T, 3), dtype=np.int32)
        e_p = np.zeros((Nm, 2), dtype=np.int32)
        e_t = np.zeros((Nm, 2), dtype=np.int32)
        e_po = np.zeros((Nm, 2), dtype=np.int32)
        e_long = np.zeros(Nm)
        e_centro = np.zeros((Nm, 3))
        self.t_area = np.zeros(T)
        self.t_baric = np.zeros((T, 3))
        self.t_baric_sub = np.zeros((T, 9, 3))
        _check(L.mlf_rwg_build(_p(tris), T, C.byref(N), C.byref(P), _p(p_coord), _p(self.t_p), _p(e_p), _p(e_t),
                               _p(e_po), _p(e_long), _p(e_centro), _p(self.t_area), _p(self.t_baric),
                               _p(self.t_baric_sub)))
        N, P = N.value, P.value
        self.N, self.P, self.T = N, P, T
        self.p_coord = p_coord[:P]
        self.e_p, self.e_t, self.e_po = e_p[:N], e_t[:N], e_po[:N]
        self.e_long, self.e_centro = e_long[:N], e_centro[:N]
        # 0-based views
        self.t_p -= 1
        self.e_p -= 1
        self.e_t -= 1
        self.e_po -= 1

    def fortran(self):
        return dict(e_t=np.ascontiguousarray(self.e_t + 1), e_po=np.ascontiguousarray(self.e_po + 1),
                    t_p=np.ascontiguousarray(self.t_p + 1), e_p=np.ascontiguousarray(self.e_p + 1))


def direction(theta_deg: float, phi_deg: float) -> np.ndarray:
    """Incidence direction as the driver builds it (main.f90:97-99)."""
    f180 = float(np.float32(180.0))
    t = theta_deg * np.pi / f180
    p = phi_deg * np.pi / f180
    return np.array([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)])


def ajustar_polariz(d, kind: str) -> np.ndarray:
    """VV -> z, HH -> d x z normalised (ajustar_polariz, main.f90:828-849)."""
    if kind == "VV":
        return np.array([0, 0, 1], dtype=np.complex128)
    v = np.array([d[1], -d[0], 0.0])
    return (v / np.sqrt(np.sum(v * v))).astype(np.complex128)


def ilu0C(n: int, a, ja, ia):
    """ilu0C (modIterativo.f90:1805-1976) on a host CSR matrix: a complex64
    values, ja / ia 1-based.  Returns (alu, jlu, ju, ierr) in the reference's
    MSR layout; raises MLFError on a malformed CSR."""
    L = load()
    a = np.ascontiguousarray(a, dtype=np.complex64)
    ja = np.ascontiguousarray(ja, dtype=np.int32)
    ia = np.ascontiguousarray(ia, dtype=np.int32)
    if ia.size != n + 1 or a.size != ja.size:
        raise ValueError("ia must hold n + 1 entries and a, ja the same count")
    nnz = int(ia[-1]) - 1 if ia.size else 0
    if nnz != a.size:
        raise ValueError("ia(n+1) - 1 must equal the number of values")
    alu = np.zeros(nnz + 1, dtype=np.complex64)
    jlu = np.zeros(nnz + 1, dtype=np.int32)
    ju = np.zeros(n, dtype=np.int32)
    ierr = C.c_int()
    code = L.mlf_ilu0_csr(int(n), _p(a), _p(ja), _p(ia), _p(alu), _p(jlu), _p(ju), C.byref(ierr))
    if code != 0:
        msg = L.mlf_last_error(None)
        raise MLFError(code, msg.decode() if msg else "")
    return alu, jlu, ju, int(ierr.value)


class MLFMA:
    """One MLFMA operator on the current CUDA device (inicializar_MLFMA)."""

    def __init__(self, rwg: RWG, lam: float = 1.0, ladomax: float = 0.5, flags: int = 0):
        L = load()
        self.rwg = rwg
        self.lam = float(lam)
        self.N = rwg.N
        f = rwg.fortran()
        h = C.c_void_p()
        code = L.mlf_init(C.byref(h), _p(np.ascontiguousarray(rwg.e_centro)), rwg.N, _p(f["e_t"]),
                          _p(f["e_po"]), _p(np.ascontiguousarray(rwg.e_long)),
                          _p(np.ascontiguousarray(rwg.t_area)), _p(np.ascontiguousarray(rwg.t_baric)),
                          _p(np.ascontiguousarray(rwg.t_baric_sub)), _p(np.ascontiguousarray(rwg.p_coord)),
                          _p(f["t_p"]), _p(f["e_p"]), rwg.P, rwg.T, None, self.lam, float(ladomax), int(flags))
        if code != 0:
            msg = L.mlf_last_error(None)
            raise MLFError(code, msg.decode() if msg else "")
        self._h = h
        info = np.zeros(160, dtype=np.int32)
        nnz = C.c_longlong()
        _check(L.mlf_info(self._h, _p(info), C.byref(nnz)), self._h)
        self.nlev = int(info[0])
        self.nnz = int(nnz.value)
        self.levels = {l: dict(nb=int(info[5 * l]), L=int(info[5 * l + 1]), K=int(info[5 * l + 2]),
                               ntrans=int(info[5 * l + 3]), nfar=int(info[5 * l + 4]))
                       for l in range(1, self.nlev + 1)}

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            load().mlf_free(self._h)
            self._h = None

    destruir_MLFMA = close

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- operator
    def matvec(self, x):
        x = np.asarray(x, dtype=np.complex128)
        single = x.ndim == 1
        X = np.asfortranarray(x.reshape(self.N, -1))
        Y = np.zeros_like(X)
        _check(load().mlf_matvec(self._h, _p(X), _p(Y), X.shape[1], self.N), self._h)
        return Y[:, 0] if single else Y

    MatxVec_MLFMA = matvec

    def matvec_device(self, x_ptr: int, y_ptr: int, nrhs: int = 1, stream: int = 0):
        _check(load().mlf_matvec_device(self._h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), nrhs, self.N,
                                        C.c_void_p(stream) if stream else None), self._h)

    def matvec_device_noalloc(self, x_ptr: int, y_ptr: int, stream: int = 0):
        """One-column matvec on device arrays that allocates nothing: the
        multipole fields live in the library's fixed 64 MiB device scratch
        (for hosts that cannot allocate mid-solve); raises MLFError when the
        octree's fields do not fit."""
        _check(load().mlf_matvec_device_noalloc(self._h, C.c_void_p(x_ptr), C.c_void_p(y_ptr),
                                                C.c_void_p(stream) if stream else None), self._h)

    def near_csr(self):
        """(ia, ja, a) with 1-based ia/ja and complex64 values (Zesparcida_MLFMA)."""
        nnz = C.c_longlong()
        _check(load().mlf_near_csr(self._h, C.byref(nnz), None, None, None), self._h)
        a = np.zeros(nnz.value, dtype=np.complex64)
        ja = np.zeros(nnz.value, dtype=np.int32)
        ia = np.zeros(self.N + 1, dtype=np.int32)
        _check(load().mlf_near_csr(self._h, C.byref(nnz), _p(a), _p(ja), _p(ia)), self._h)
        return ia, ja, a

    def set_near_values(self, a):
        """Overwrite the complex(4) near-field values (Zesparcida_MLFMA) in
        near_csr()'s order; preconditioners built before must be built again."""
        a = np.ascontiguousarray(a, dtype=np.complex64)
        if a.size != self.nnz:
            raise ValueError(f"expected {self.nnz} near values, got {a.size}")
        _check(load().mlf_set_near_values(self._h, _p(a)), self._h)

    # -- preconditioner
    def ilu0(self) -> int:
        ierr = C.c_int()
        _check(load().mlf_ilu0(self._h, C.byref(ierr)), self._h)
        return int(ierr.value)

    ilu0C = ilu0

    def ilut(self, fill_in_prc=5.0, droptol=1e-3) -> int:
        """ILUT of the near field (crear_precond ILUT branch); returns ilutC's ierr."""
        ierr = C.c_int()
        _check(load().mlf_ilut(self._h, float(fill_in_prc), float(droptol), C.byref(ierr)), self._h)
        return int(ierr.value)

    ilutC = ilut

    def ilu0_factors(self):
        n = C.c_longlong()
        _check(load().mlf_ilu_size(self._h, C.byref(n)), self._h)
        alu = np.zeros(n.value, dtype=np.complex64)
        jlu = np.zeros(n.value, dtype=np.int32)
        ju = np.zeros(self.N, dtype=np.int32)
        _check(load().mlf_ilu0_factors(self._h, _p(alu), _p(jlu), _p(ju)), self._h)
        return alu, jlu, ju

    def lusol0(self, y):
        y = np.asarray(y, dtype=np.complex128)
        single = y.ndim == 1
        Y = np.asfortranarray(y.reshape(self.N, -1))
        X = np.zeros_like(Y)
        _check(load().mlf_ilu0_solve(self._h, _p(Y), _p(X), Y.shape[1]), self._h)
        return X[:, 0] if single else X

    lusol0C = lusol0

    def nearinv(self, own_only: bool = False) -> int:
        """Build the neighbourhood-inverse preconditioner (own_only: block Jacobi on each
        box's own bases); 0 or (singular box + 1)."""
        bad = C.c_int()
        f = load().mlf_nearinv_own if own_only else load().mlf_nearinv
        _check(f(self._h, C.byref(bad)), self._h)
        return int(bad.value)

    def set_nearinv_precision(self, bits: int):
        """Elimination of nearinv(): 64 FP64, 32 blocked FP32 LU, 0 by size (FP64 up to 768 unknowns)."""
        _check(load().mlf_set_nearinv_precision(self._h, int(bits)), self._h)

    def set_lu_split(self, min_unknowns: int = 1024):
        """mlf_set_lu_split: boxes of at least min_unknowns unknowns that would
        dominate the neighbourhood inverse's set-up are factorised on many CTAs
        each (0: never)."""
        _check(load().mlf_set_lu_split(self._h, int(min_unknowns)), self._h)

    def lu_split(self):
        """(min_unknowns, boxes on the many-CTA path in the last build)."""
        a, b = C.c_int(), C.c_int()
        _check(load().mlf_get_lu_split(self._h, C.byref(a), C.byref(b)), self._h)
        return a.value, b.value

    def precond_apply(self, y, precond="nearinv"):
        if isinstance(precond, str):
            precond = PRECOND[precond]
        y = np.asarray(y, dtype=np.complex128)
        single = y.ndim == 1
        Y = np.asfortranarray(y.reshape(self.N, -1))
        X = np.zeros_like(Y)
        _check(load().mlf_precond_apply(self._h, int(precond), _p(Y), _p(X), Y.shape[1]), self._h)
        return X[:, 0] if single else X

    def nearinv_values(self):
        out = np.zeros(self.nnz, dtype=np.complex128)
        _check(load().mlf_nearinv_values(self._h, _p(out)), self._h)
        return out

    # -- solver
    def cgs(self, b, guess=None, errmax=1e-4, maxit=1000, precond=0):
        """Returns dict(x, iters, relres, status) per column.  precond: 0/'none',
        1/'ilu0', 2/'nearinv'."""
        if isinstance(precond, str):
            precond = PRECOND[precond]
        b = np.asarray(b, dtype=np.complex128)
        single = b.ndim == 1
        B = np.asfortranarray(b.reshape(self.N, -1))
        nrhs = B.shape[1]
        G = None if guess is None else np.asfortranarray(np.asarray(guess, dtype=np.complex128).reshape(self.N, -1))
        X = np.zeros_like(B)
        it = np.zeros(nrhs, dtype=np.int32)
        rr = np.zeros(nrhs)
        st = np.zeros(nrhs, dtype=np.int32)
        _check(load().mlf_cgs(self._h, _p(B), None if G is None else _p(G), float(errmax), int(maxit), nrhs,
                              _p(X), _p(it), _p(rr), int(precond), _p(st)), self._h)
        if single:
            return dict(x=X[:, 0], iters=int(it[0]), relres=float(rr[0]), status=CGS_STATUS[int(st[0])])
        return dict(x=X, iters=it, relres=rr, status=[CGS_STATUS[int(s)] for s in st])

    def set_stagnation(self, window: int):
        """Stop a column as 'stagnated' when its residual has set no new
        minimum within `window` iterations (0: off, the default)."""
        _check(load().mlf_set_stagnation(self._h, int(window)), self._h)

    def cgs_history(self, col: int = 0):
        n = C.c_int()
        _check(load().mlf_cgs_history(self._h, int(col), None, 0, C.byref(n)), self._h)
        h = np.zeros(n.value)
        _check(load().mlf_cgs_history(self._h, int(col), _p(h), n.value, C.byref(n)), self._h)
        return h

    def solve(self, b, guess=None, errmax=1e-4, maxit=1000, precond=0, mixed=False, inner_tol=0.0):
        """mlf_solve: mixed=False is CGS on the FP64 operator; mixed=True is FP64
        iterative refinement around CGS on the FP32 operator."""
        if isinstance(precond, str):
            precond = PRECOND[precond]
        b = np.asarray(b, dtype=np.complex128)
        single = b.ndim == 1
        B = np.asfortranarray(b.reshape(self.N, -1))
        nrhs = B.shape[1]
        G = None if guess is None else np.asfortranarray(np.asarray(guess, dtype=np.complex128).reshape(self.N, -1))
        X = np.zeros_like(B)
        it = np.zeros(nrhs, dtype=np.int32)
        rr = np.zeros(nrhs)
        st = np.zeros(nrhs, dtype=np.int32)
        outer = C.c_int()
        _check(load().mlf_solve(self._h, _p(B), None if G is None else _p(G), float(errmax), int(maxit), nrhs,
                                int(precond), 1 if mixed else 0, float(inner_tol), _p(X), _p(it), _p(rr), _p(st),
                                C.byref(outer)), self._h)
        if single:
            return dict(x=X[:, 0], iters=int(it[0]), relres=float(rr[0]), status=CGS_STATUS[int(st[0])],
                        outer=outer.value)
        return dict(x=X, iters=it, relres=rr, status=[CGS_STATUS[int(s)] for s in st], outer=outer.value)

    def set_block_engine(self, engine: int, cols: int = 0):
        """Multi-column engine of the batched FP32 operator and preconditioner:
        1 box blocks on tensor cores (3xTF32 mma.sync), 0 box blocks on FP32
        FMA, 2 warp per basis (receive per box), 3 warp per basis throughout,
        4 box blocks on tcgen05 (near field, leaf aggregation and receive;
        3xTF32, TMEM accumulators, TMA-staged operands), -1 by leaf-box size; tile width
        cols 8, 32, 64 (0: by block width)."""
        _check(load().mlf_set_block_engine(self._h, int(engine), int(cols)), self._h)

    def autotune_block(self, candidates=(8, 16, 32, 64, 128)):
        """mlf_autotune_block: block size and near-field tile width for batched
        solves, with the measured FP32 operator time per right-hand side."""
        cand = np.ascontiguousarray(candidates, dtype=np.int32)
        per = np.zeros(cand.size, dtype=np.float32)
        best, cols, eng = C.c_int(), C.c_int(), C.c_int()
        _check(load().mlf_autotune_block(self._h, _p(cand), cand.size, C.byref(best), C.byref(cols), C.byref(eng),
                                         _p(per)), self._h)
        return dict(block=best.value, tile_cols=cols.value,
                    engine=ENGINES.get(eng.value, str(eng.value)),
                    per_rhs_ms={int(b): float(t) for b, t in zip(cand, per)})

    def precond_apply32(self, y):
        """mlf_precond_apply32: the FP32 preconditioner of the mixed inner loop."""
        y = np.asarray(y, dtype=np.complex128)
        single = y.ndim == 1
        Y = np.asfortranarray(y.reshape(self.N, -1))
        X = np.zeros_like(Y, order="F")
        _check(load().mlf_precond_apply32(self._h, _p(Y), _p(X), Y.shape[1]), self._h)
        return X[:, 0] if single else X

    def solve_times(self):
        """Phase times (ms) of the last mixed solve run with profiling on:
        preconditioner, FP32 operator, orthogonalisation, total."""
        out = np.zeros(4)
        _check(load().mlf_solve_times(self._h, _p(out)), self._h)
        return dict(zip(("precond", "operator", "orthogonalisation", "total"), out.tolist()))

    def solve_phases(self):
        """mlf_solve_phases: solve_times plus the FP64 residual checks, the
        provisional FP32 residual of a warm start (ms) and the outer steps."""
        out = np.zeros(7)
        _check(load().mlf_solve_phases(self._h, _p(out), 7), self._h)
        return dict(zip(("precond", "operator", "orthogonalisation", "total", "fp64_residual",
                         "provisional_residual", "outer"), out.tolist()))

    def set_gmres_restart(self, m: int):
        _check(load().mlf_set_gmres_restart(self._h, int(m)), self._h)

    def set_gs_passes(self, passes: int):
        _check(load().mlf_set_gs_passes(self._h, int(passes)), self._h)

    def set_basis_precision(self, bits: int):
        """Krylov basis storage of the mixed solve: 32 (FP32) or 16 (FP16)."""
        _check(load().mlf_set_basis_precision(self._h, int(bits)), self._h)

    def set_translation_group(self, boxes: int = 0, cols: int = 0):
        """FP32 translation over the merged far lists of 2 or 4 consecutive
        boxes per thread, 1 box at a time, or 0 (the default): 2 for one
        column, 4 for blocks; cols = columns per thread with grouped boxes
        (0: automatic)."""
        _check(load().mlf_set_translation_group(self._h, int(boxes), int(cols)), self._h)

    def matvec32(self, x):
        x = np.asarray(x, dtype=np.complex128)
        single = x.ndim == 1
        X = np.asfortranarray(x.reshape(self.N, -1))
        Y = np.zeros_like(X)
        _check(load().mlf_matvec32(self._h, _p(X), _p(Y), X.shape[1], self.N), self._h)
        return Y[:, 0] if single else Y

    def CGSold(self, b, guess, errmax, prec=False, maxit=100000):
        return self.cgs(b, guess, errmax, maxit, 1 if prec else 0)

    # -- excitation and RCS
    def excitation(self, dirs, pols, ctte=1.0):
        dirs = np.ascontiguousarray(np.atleast_2d(dirs), dtype=np.float64)
        pols = np.ascontiguousarray(np.atleast_2d(pols), dtype=np.complex128)
        nrhs = dirs.shape[0]
        Bm = np.zeros((nrhs, self.N), dtype=np.complex128)
        _check(load().mlf_excitation(self._h, _p(dirs), _p(pols), float(np.real(ctte)), float(np.imag(ctte)),
                                     nrhs, _p(Bm)), self._h)
        return Bm[0] if nrhs == 1 else Bm.T.copy()

    def generar_onda(self, direccion, polarizacion, ctte=1.0):
        return self.excitation(direccion, polarizacion, ctte)

    def rcs(self, current, pol, theta, phi, ctte=1.0):
        """Linear sigma for each (theta, phi) pair in radians."""
        th, ph = np.broadcast_arrays(np.atleast_1d(np.asarray(theta, dtype=np.float64)),
                                     np.atleast_1d(np.asarray(phi, dtype=np.float64)))
        th = np.ascontiguousarray(th.ravel())
        ph = np.ascontiguousarray(ph.ravel())
        cur = np.ascontiguousarray(current, dtype=np.complex128)
        pol = np.ascontiguousarray(pol, dtype=np.complex128)
        out = np.zeros(th.size)
        _check(load().mlf_rcs(self._h, _p(cur), _p(pol), float(np.real(ctte)), float(np.imag(ctte)), _p(th), _p(ph),
                              th.size, _p(out)), self._h)
        return out

    def sigmaRCS(self, current, pol, theta, phi, ctte=1.0):
        return self.rcs(current, pol, theta, phi, ctte)

    def monostatic(self, nang, phis=None, pol="VV", errmax=1e-3, maxit=5000, precond=0, mode=0, block=32,
                   ctte=1.0):
        """Monostatic sweep (gen_rcs_monostatica).  Returns dict(phi, sigma_db, iters, status).
        mode 0: the reference's warm-started sequential sweep; 1: batched FP64 CGS;
        2: batched mixed precision; 3: batched mixed precision, each block
        column sweeping a contiguous run of angles with mode 0's warm starts;
        4: as 3, starts extrapolated from each column's two previous angles."""
        if isinstance(precond, str):
            precond = PRECOND[precond]
        ph = None if phis is None else np.ascontiguousarray(phis, dtype=np.float64)
        sig = np.zeros(nang)
        it = np.zeros(nang, dtype=np.int32)
        st = np.zeros(nang, dtype=np.int32)
        _check(load().mlf_monostatic(self._h, int(nang), None if ph is None else _p(ph), 1 if pol == "HH" else 0,
                                     float(np.real(ctte)), float(np.imag(ctte)), float(errmax), int(maxit),
                                     int(precond), int(mode), int(block), _p(sig), _p(it), _p(st)), self._h)
        phi = ph if ph is not None else np.arange(nang) * (np.pi / nang)
        return dict(phi=phi, sigma_db=10 * np.log10(sig), iters=it, status=[CGS_STATUS[int(s)] for s in st])

    gen_rcs_monostatica = monostatic

    # -- diagnostics
    def set_profiling(self, on=True):
        _check(load().mlf_set_profiling(self._h, 1 if on else 0), self._h)

    def stage_times(self):
        out = np.zeros(5, dtype=np.float32)
        _check(load().mlf_stage_times(self._h, _p(out)), self._h)
        return out

    def algorithmic_counts(self):
        """Per-matvec algorithmic FLOPs and HBM bytes (1 RHS), by stage.

        FLOPs: complex MAC = 8, real x complex MAC = 4, complex multiply = 6.
        Bytes: patterns read at aggregation and at receive, near CSR
        (complex(4) values + int32 columns + row pointers), each field level
        written/read once per pass (C write+read, B write, A write+read),
        x read twice and y written once.
        """
        nl = self.nlev
        lv = self.levels
        Kl, N = lv[nl]["K"], self.N
        trans = sum(16.0 * lv[n]["nfar"] * lv[n]["K"] for n in range(3, nl + 1))
        rows = sum(lv[n - 1]["K"] * lv[n]["nb"] for n in range(4, nl + 1))
        flops = dict(translation=trans, aggregation=16.0 * Kl * N, receive=16.0 * Kl * N,
                     interpolation=4.0 * 9 * 2 * rows + 6.0 * 2 * rows,
                     anterpolation=4.0 * 9 * 2 * rows + 6.0 * 2 * rows, near=8.0 * self.nnz)
        field = sum(2.0 * lv[n]["K"] * lv[n]["nb"] * 16 for n in range(3, nl + 1))
        byt = dict(patterns=2 * 2.0 * Kl * N * 16, near=self.nnz * 12.0 + (N + 1) * 4.0, fields=5 * field,
                   vectors=3.0 * N * 16)
        trans_bytes = sum(2.0 * 2 * lv[n]["K"] * lv[n]["nb"] * 16 + lv[n]["ntrans"] * lv[n]["K"] * 16.0
                          for n in range(3, nl + 1))
        return dict(flops=flops, bytes=byt, flops_total=sum(flops.values()), bytes_total=sum(byt.values()),
                    translation_bytes=trans_bytes)

    def debug_field(self, level, which):
        lv = self.levels[level]
        out = np.zeros((lv["nb"], 2, lv["K"]), dtype=np.complex128)
        _check(load().mlf_debug_field(self._h, int(level), int(which), _p(out)), self._h)
        return out


class MoM(MLFMA):
    """Dense method-of-moments operator on the GPU (MoM + MatxVec_MoM,
    modMoM.f90:85-128, 273-277): the full impedance matrix in FP64 on the
    device.  matvec, cgs / CGSold without preconditioner, excitation, rcs and
    the FP64 monostatic modes work as for MLFMA; octree-based calls raise."""

    def __init__(self, rwg: RWG, lam: float = 1.0):
        super().__init__(rwg, lam=lam, ladomax=1.0, flags=FLAG_DENSE_MOM)


class FMM(MLFMA):
    """Single-level FMM (inicializar_FMM + MatxVec_FMM, modFMM.f90:170-268,
    904-963): one grid level of boxes of side <= side * lambda (the
    reference's is lambda / 2), far pairs translated directly; matvec,
    ILU0 / ILUT / neighbourhood preconditioners, CGS, mixed solves and RCS as
    for MLFMA."""

    def __init__(self, rwg: RWG, lam: float = 1.0, side: float = 0.5):
        super().__init__(rwg, lam=lam, ladomax=side, flags=FLAG_FMM)
