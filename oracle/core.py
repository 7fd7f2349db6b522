"""ORACLE (test infrastructure): ctypes front-end of oracle/mlfma_oracle.c.

``OracleMLFMA`` mirrors the reference's module state after
``inicializar_MLFMA`` (modMLFMA.f90:113-275): octree, sampling, translation
tables, interpolation tables, radiation patterns and the complex(4) near-field
CSR, and offers ``matvec`` (MatxVec_MLFMA, modMLFMA.f90:1901-1946), ``ilu0`` /
``lusol0`` (ilu0C / lusol0C, modIterativo.f90:1805-1976, 504-560), ``cgs``
(CGSold, modIterativo.f90:331-493) and per-stage field dumps.
Free functions: ``generar_onda`` (main.f90:1488-1525), ``sigma_rcs``
(modRCS.f90:60-153), ``ajustar_polariz`` (main.f90:828-849).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from .rwg import RWG

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None

PI = 3.141592653589793
MU = 1.2566370614E-6
EPSI = 8.8541878176E-12


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
                os.path.join(HERE, "mlfma_oracle.c")):
            build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.ora_create.restype = vp
        L.ora_create.argtypes = [C.c_int, C.c_int, C.c_int] + [vp] * 7 + [C.c_double, C.c_double, C.c_int, vp]
        L.ora_create_fmm.restype = vp
        L.ora_create_fmm.argtypes = [C.c_int, C.c_int, C.c_int] + [vp] * 7 + [C.c_double, C.c_double, C.c_int, vp]
        L.ora_free.argtypes = [vp]
        L.ora_nlev.argtypes = [vp]
        L.ora_nnz.argtypes = [vp]
        L.ora_nnz.restype = C.c_int64
        L.ora_level_info.argtypes = [vp, C.c_int, vp, vp]
        for f in ("ora_level_centres", "ora_level_parents", "ora_patterns", "ora_leaf_boxes"):
            getattr(L, f).argtypes = None
        L.ora_matvec.argtypes = [vp, vp, vp]
        L.ora_ilu0.argtypes = [vp]
        L.ora_lusol0.argtypes = [vp, vp, vp]
        L.ora_cgs.argtypes = [vp, vp, vp, C.c_double, C.c_int, C.c_int, vp, vp, vp, vp]
        L.ora_generar_onda.argtypes = [C.c_int, vp, vp, vp, vp, vp, C.c_double, vp, vp, C.c_double, C.c_double, vp]
        L.ora_rcs.argtypes = [C.c_int, vp, vp, vp, vp, C.c_double, vp, vp, C.c_double, C.c_double, vp, vp, C.c_int, vp]
        L.ora_zmn_block.argtypes = [vp, C.c_int, C.c_int, vp]
        L.ora_root.restype = C.c_double
        L.ora_root.argtypes = [vp, vp]
        L.ora_ilu0_raw.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp]
        L.ora_lusol0_raw.argtypes = [C.c_int, vp, vp, vp, vp, vp]
        L.ora_interp_table.argtypes = [C.c_int, C.c_int, vp, vp]
        L.ora_sph_bessel.argtypes = [C.c_int, C.c_double, vp, vp]
        L.ora_legendre.argtypes = [C.c_int, C.c_double, C.c_int, vp]
        L.ora_set_threads.argtypes = [C.c_int]
        L.ora_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _c2(z):
    return float(np.real(z)), float(np.imag(z))


def set_threads(n: int):
    lib().ora_set_threads(int(n))


def get_threads() -> int:
    return int(lib().ora_get_threads())


class OracleError(RuntimeError):
    pass


class OracleMLFMA:
    def __init__(self, rwg: RWG, lam: float = 1.0, ladomax: float = 0.5, legendre_mode: int = 0,
                 fmm: bool = False):
        """fmm=True builds the single-level FMM of modFMM.f90 instead, with box
        side ladomax * lambda as the criterion (the reference's is 0.5)."""
        L = lib()
        self.rwg = rwg
        self.lam = float(lam)
        self.N = rwg.N
        # keep contiguous copies alive for the C side
        self._pc = np.ascontiguousarray(rwg.p_coord, dtype=np.float64)
        self._tb = np.ascontiguousarray(rwg.t_baric, dtype=np.float64)
        self._tbs = np.ascontiguousarray(rwg.t_baric_sub, dtype=np.float64)
        self._el = np.ascontiguousarray(rwg.e_long, dtype=np.float64)
        self._ec = np.ascontiguousarray(rwg.e_centro, dtype=np.float64)
        self._et = np.ascontiguousarray(rwg.e_t, dtype=np.int32)
        self._epo = np.ascontiguousarray(rwg.e_po, dtype=np.int32)
        st = C.c_int(0)
        create = L.ora_create_fmm if fmm else L.ora_create
        self._h = create(rwg.N, rwg.T, rwg.P, _p(self._pc), _p(self._tb), _p(self._tbs), _p(self._el),
                               _p(self._ec), _p(self._et), _p(self._epo), self.lam, float(ladomax),
                               int(legendre_mode), C.byref(st))
        self.status = st.value
        if self.status != 0:
            L.ora_free(self._h)
            self._h = None
            raise OracleError(f"ora_create status {self.status}")
        self.nlev = L.ora_nlev(self._h)
        self.nnz = int(L.ora_nnz(self._h))
        self.levels = {}
        for n in range(1, self.nlev + 1):
            info = np.zeros(5, dtype=np.int32)
            side = C.c_double()
            L.ora_level_info(self._h, n, _p(info), C.byref(side))
            self.levels[n] = dict(nb=int(info[0]), L=int(info[1]), K=int(info[2]), ntrans=int(info[3]),
                                  nfar=int(info[4]), side=side.value)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ora_free(self._h)
            self._h = None

    # ---- tables
    def centres(self, n):
        a = np.zeros((self.levels[n]["nb"], 3))
        lib().ora_level_centres(C.c_void_p(self._h), C.c_int(n), _p(a))
        return a

    def parents(self, n):
        a = np.zeros(self.levels[n]["nb"], dtype=np.int32)
        lib().ora_level_parents(C.c_void_p(self._h), C.c_int(n), _p(a))
        return a

    def far(self, n):
        lv = self.levels[n]
        ptr = np.zeros(lv["nb"] + 1, dtype=np.int32)
        src = np.zeros(max(lv["nfar"], 1), dtype=np.int32)
        tid = np.zeros(max(lv["nfar"], 1), dtype=np.int32)
        lib().ora_level_far(C.c_void_p(self._h), C.c_int(n), _p(ptr), _p(src), _p(tid))
        return ptr, src[:lv["nfar"]], tid[:lv["nfar"]]

    def trans(self, n):
        lv = self.levels[n]
        rab = np.zeros((lv["ntrans"], 3))
        T = np.zeros((lv["ntrans"], lv["K"]), dtype=np.complex128)
        lib().ora_level_trans(C.c_void_p(self._h), C.c_int(n), _p(rab), _p(T))
        return rab, T

    def interp(self, n):
        K = self.levels[n]["K"]
        w = np.zeros((K, 9))
        idx = np.zeros((K, 9), dtype=np.int32)
        lib().ora_level_interp(C.c_void_p(self._h), C.c_int(n), _p(w), _p(idx))
        return w, idx

    def fields(self, n):
        lv = self.levels[n]
        shp = (lv["nb"], 2, lv["K"])
        Cf, Bf, Af = (np.zeros(shp, dtype=np.complex128) for _ in range(3))
        lib().ora_level_fields(C.c_void_p(self._h), C.c_int(n), _p(Cf), _p(Bf), _p(Af))
        return Cf, Bf, Af

    def leaf_boxes(self):
        nb = self.levels[self.nlev]["nb"]
        ptr = np.zeros(nb + 1, dtype=np.int32)
        bases = np.zeros(self.N, dtype=np.int32)
        lib().ora_leaf_boxes(C.c_void_p(self._h), _p(ptr), _p(bases))
        return ptr, bases

    def patterns(self):
        K = self.levels[self.nlev]["K"]
        a = np.zeros((self.N, 2, K), dtype=np.complex128)
        lib().ora_patterns(C.c_void_p(self._h), _p(a))
        return a

    def near(self):
        ia = np.zeros(self.N + 1, dtype=np.int32)
        ja = np.zeros(self.nnz, dtype=np.int32)
        z = np.zeros(self.nnz, dtype=np.complex64)
        lib().ora_near(C.c_void_p(self._h), _p(ia), _p(ja), _p(z))
        return ia, ja, z

    def set_near(self, z):
        z = np.ascontiguousarray(z, dtype=np.complex64)
        assert z.size == self.nnz
        self._z_keep = z
        lib().ora_set_near(C.c_void_p(self._h), _p(z))

    def root(self):
        c = np.zeros(3)
        side = lib().ora_root(self._h, _p(c))
        return c, side

    # ---- operators
    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.N, dtype=np.complex128)
        lib().ora_matvec(self._h, _p(x), _p(y))
        return y

    def ilu0(self) -> int:
        return int(lib().ora_ilu0(self._h))

    def ilut(self, fill_in_prc=5.0, droptol=1e-3) -> int:
        lfil = int(np.ceil(0.01 * fill_in_prc * self.N))
        return int(lib().ora_ilut(C.c_void_p(self._h), C.c_int(lfil), C.c_double(droptol)))

    def ilu_factors(self):
        lib().ora_ilu_len.restype = C.c_int64
        n = int(lib().ora_ilu_len(C.c_void_p(self._h)))
        alu = np.zeros(n + 2, dtype=np.complex64)
        jlu = np.zeros(n + 2, dtype=np.int32)
        ju = np.zeros(self.N + 1, dtype=np.int32)
        lib().ora_ilu_factors(C.c_void_p(self._h), _p(alu), _p(jlu), _p(ju))
        return alu, jlu, ju

    def lusol0(self, y):
        y = np.ascontiguousarray(y, dtype=np.complex128)
        x = np.zeros(self.N, dtype=np.complex128)
        lib().ora_lusol0(self._h, _p(y), _p(x))
        return x

    def nearinv(self) -> int:
        return int(lib().ora_nearinv(C.c_void_p(self._h)))

    def nearinv_values(self):
        out = np.zeros(self.nnz, dtype=np.complex128)
        lib().ora_nearinv_values(C.c_void_p(self._h), _p(out))
        return out

    def nearinv_apply(self, y):
        y = np.ascontiguousarray(y, dtype=np.complex128)
        x = np.zeros(self.N, dtype=np.complex128)
        lib().ora_nearinv_apply(C.c_void_p(self._h), _p(y), _p(x))
        return x

    def cgs(self, b, guess=None, tol=1e-4, maxit=1000, prec=False, history=False):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        g = np.zeros(self.N, dtype=np.complex128) if guess is None else np.ascontiguousarray(guess, dtype=np.complex128)
        x = np.zeros(self.N, dtype=np.complex128)
        it = C.c_int()
        rr = C.c_double()
        hist = np.zeros(maxit)
        st = lib().ora_cgs(self._h, _p(b), _p(g), float(tol), int(maxit), int(prec), _p(x),
                           C.byref(it), C.byref(rr), _p(hist))
        out = dict(x=x, status=int(st), iters=it.value, relres=rr.value)
        if history:
            out["history"] = hist[:it.value]
        return out

    def zmn_rows(self, m0, m1):
        Z = np.zeros((m1 - m0, self.N), dtype=np.complex128)
        lib().ora_zmn_block(self._h, int(m0), int(m1), _p(Z))
        return Z


def generar_onda(rwg: RWG, lam: float, direction, pol, ctte=1.0):
    d = np.ascontiguousarray(direction, dtype=np.float64)
    p = np.ascontiguousarray(pol, dtype=np.complex128)
    res = np.zeros(rwg.N, dtype=np.complex128)
    pc = np.ascontiguousarray(rwg.p_coord); tb = np.ascontiguousarray(rwg.t_baric)
    el = np.ascontiguousarray(rwg.e_long)
    et = np.ascontiguousarray(rwg.e_t, dtype=np.int32); epo = np.ascontiguousarray(rwg.e_po, dtype=np.int32)
    lib().ora_generar_onda(rwg.N, _p(pc), _p(tb), _p(el), _p(et), _p(epo), float(lam), _p(d), _p(p),
                           *_c2(ctte), _p(res))
    return res


def sigma_rcs(rwg: RWG, lam: float, current, pol, theta, phi, ctte=1.0):
    """Linear sigma for each (theta, phi) pair (radians)."""
    th = np.ascontiguousarray(np.atleast_1d(theta), dtype=np.float64)
    ph = np.ascontiguousarray(np.atleast_1d(phi), dtype=np.float64)
    th, ph = np.broadcast_arrays(th, ph)
    th = np.ascontiguousarray(th); ph = np.ascontiguousarray(ph)
    cur = np.ascontiguousarray(current, dtype=np.complex128)
    p = np.ascontiguousarray(pol, dtype=np.complex128)
    out = np.zeros(th.size)
    tb = np.ascontiguousarray(rwg.t_baric); el = np.ascontiguousarray(rwg.e_long)
    ec = np.ascontiguousarray(rwg.e_centro); et = np.ascontiguousarray(rwg.e_t, dtype=np.int32)
    lib().ora_rcs(rwg.N, _p(tb), _p(el), _p(ec), _p(et), float(lam), _p(cur), _p(p), *_c2(ctte),
                  _p(th), _p(ph), th.size, _p(out))
    return out


def ajustar_polariz(direction, kind: str):
    """main.f90:828-849: VV -> z; HH -> d x z normalised."""
    if kind == "VV":
        return np.array([0, 0, 1], dtype=np.complex128)
    d = np.asarray(direction, dtype=np.float64)
    v = np.array([d[1] * 1.0 - d[2] * 0.0, d[2] * 0.0 - d[0] * 1.0, d[0] * 0.0 - d[1] * 0.0])
    return (v / np.sqrt(np.sum(v * v))).astype(np.complex128)


def direction_from_angles(theta_deg, phi_deg):
    """main.f90:97-99: dir = (sin t cos p, sin t sin p, cos t), angles in degrees."""
    f180 = float(np.float32(180.0))
    t = theta_deg * PI / f180
    p = phi_deg * PI / f180
    return np.array([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)])


def monostatic_sweep(o: "OracleMLFMA", nang, pol="VV", tol=1e-3, maxit=5000, prec=0):
    """gen_rcs_monostatica (main.f90:967-1089): sequential angles phi = (a-1) pi/nang,
    incidence (-cos, -sin, 0), warm start = previous currents x exp(-j k dR . r_edge),
    backscatter sigma(pi/2, phi).  Returns (phi, sigma_dB, iterations)."""
    r = o.rwg
    kappa = 2. * PI / o.lam
    dephi = 1. * PI / nang
    guess = np.zeros(o.N, dtype=np.complex128)
    prev = np.array([-1., 0., 0.])
    phis, out_db, its = [], [], []
    for a in range(1, nang + 1):
        phi = (a - 1) * dephi
        d = np.array([-np.cos(phi), -np.sin(phi), 0.])
        dR = d - prev
        guess = guess * np.exp((-1j) * kappa * (r.e_centro @ dR))
        pol_v = ajustar_polariz(d, pol)
        b = generar_onda(r, o.lam, d, pol_v)
        res = o.cgs(b, guess=guess, tol=tol, maxit=maxit, prec=prec)
        s = sigma_rcs(r, o.lam, res["x"], pol_v, PI / 2., phi)[0]
        phis.append(phi); out_db.append(10 * np.log10(s)); its.append(res["iters"])
        guess = res["x"]
        prev = d
    return np.array(phis), np.array(out_db), np.array(its)


def ilu0_raw(n, a, ja, ia):
    """ilu0C on a 1-based CSR given as 0-padded arrays (index 0 unused)."""
    a = np.ascontiguousarray(a, dtype=np.complex64)
    ja = np.ascontiguousarray(ja, dtype=np.int32)
    ia = np.ascontiguousarray(ia, dtype=np.int32)
    nnz = len(a) - 1
    alu = np.zeros(nnz + n + 3, dtype=np.complex64)
    jlu = np.zeros(nnz + n + 3, dtype=np.int32)
    ju = np.zeros(n + 1, dtype=np.int32)
    ierr = lib().ora_ilu0_raw(int(n), _p(a), _p(ja), _p(ia), _p(alu), _p(jlu), _p(ju))
    return int(ierr), alu, jlu, ju


def lusol0_raw(n, y, alu, jlu, ju):
    y = np.ascontiguousarray(y, dtype=np.complex128)
    x = np.zeros(n, dtype=np.complex128)
    lib().ora_lusol0_raw(int(n), _p(y), _p(x), _p(alu), _p(jlu), _p(ju))
    return x


def interp_table(L_coarse, L_fine):
    K = L_coarse * 2 * L_coarse
    w = np.zeros((K, 9))
    idx = np.zeros((K, 9), dtype=np.int32)
    lib().ora_interp_table(int(L_coarse), int(L_fine), _p(w), _p(idx))
    return w, idx


def sph_bessel(nmax, x):
    j = np.zeros(nmax + 1)
    y = np.zeros(nmax + 1)
    lib().ora_sph_bessel(int(nmax), float(x), _p(j), _p(y))
    return j, y


def legendre(nmax, x, mode=0):
    P = np.zeros(nmax + 1)
    lib().ora_legendre(int(nmax), float(x), int(mode), _p(P))
    return P
