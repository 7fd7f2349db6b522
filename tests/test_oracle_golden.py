"""Pin the CPU oracle to the reference: known-answer files shipped with the
reference and fixtures produced by running the reference's binary
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest
import scipy.special as sp

from conftest import load_golden
from oracle import core
from oracle.rwg import RWG


def _bistatic_grid(ntheta, nphi):
    # RCS_bi grid (main.f90:1390-1424): midpoints in theta and phi
    th = np.array([(2 * t - 1) * (np.pi / ntheta) / 2. for t in range(1, ntheta + 1)])
    ph = np.array([(2 * p - 1) * (2. * np.pi / nphi) / 2. for p in range(1, nphi + 1)])
    TT, PP = np.meshgrid(th, ph, indexing="ij")
    return TT.ravel(), PP.ravel()


@pytest.fixture(scope="module")
def ico3():
    g = load_golden("bin_ico3_mlfma.npz")
    r = RWG(g["tris"])
    o = core.OracleMLFMA(r, lam=1.0, ladomax=0.3)
    return g, r, o


def test_octree_matches_binary_log(ico3):
    # the binary printed: 4 levels; level 3: 56 boxes, L=15, K=450; level 4:
    # 248 boxes, L=11, K=242; 316 distinct translations; nnz = 1542240/8
    g, r, o = ico3
    assert o.nlev == 4
    assert (o.levels[3]["nb"], o.levels[3]["L"], o.levels[3]["K"]) == (56, 15, 450)
    assert (o.levels[4]["nb"], o.levels[4]["L"], o.levels[4]["K"]) == (248, 11, 242)
    assert o.levels[3]["ntrans"] == 316 and o.levels[4]["ntrans"] == 316
    assert o.nnz == 1542240 // 8


def test_matvec_reproduces_binary_currents(ico3):
    """Z_MLFMA I_ref = b to the print precision of the binary's currents."""
    g, r, o = ico3
    d = core.direction_from_angles(90.0, 180.0)
    pol = core.ajustar_polariz(d, "VV")
    b = core.generar_onda(r, 1.0, d, pol)
    res = np.linalg.norm(o.matvec(g["I"]) - b) / np.linalg.norm(b)
    assert res < 2e-5, res


def test_cgs_iterations_and_currents_match_binary(ico3):
    g, r, o = ico3
    d = core.direction_from_angles(90.0, 180.0)
    b = core.generar_onda(r, 1.0, d, core.ajustar_polariz(d, "VV"))
    out = o.cgs(b, tol=1e-8, maxit=2000, history=True)
    assert out["status"] == 0
    assert out["iters"] == int(g["iterations"])
    assert np.linalg.norm(out["x"] - g["I"]) / np.linalg.norm(g["I"]) < 1e-5
    # residual history printed by the binary (6 significant digits); CGS
    # amplifies last-bit differences of the two builds as it goes, so only
    # the first iterations are compared tightly
    hist = g["res_hist"] / float(g["bnorm"])
    np.testing.assert_allclose(out["history"][:10], hist[:10], rtol=1e-4)


def test_rcs_reproduces_binary_bistatic(ico3):
    g, r, o = ico3
    d = core.direction_from_angles(90.0, 180.0)
    pol = core.ajustar_polariz(d, "VV")
    th, ph = _bistatic_grid(5, 8)
    rcs = 10 * np.log10(core.sigma_rcs(r, 1.0, g["I"], pol, th, ph)).reshape(5, 8)
    assert np.abs(rcs - g["rcsbi"]).max() < 1e-4


def test_interpolation_dump_of_binary_run(ico3):
    """The binary's test_interp dump (L=15 -> 11 here): inter = W orig, anter = W^T inter."""
    g, r, o = ico3
    w, idx = o.interp(3)
    K3, K4 = o.levels[3]["K"], o.levels[4]["K"]
    W = np.zeros((K3, K4))
    np.add.at(W, (np.repeat(np.arange(K3), 9), idx.ravel()), w.ravel())
    Wb = np.zeros(tuple(g["W_shape"]))
    Wb[g["W_rows"], g["W_cols"]] = g["W_vals"]
    assert np.abs(W - Wb).max() < 1e-7          # f16.8 print precision
    orig = np.stack([g["orig_t"].T.ravel(), g["orig_p"].T.ravel()], axis=1)
    inter = np.stack([g["inter_t"].T.ravel(), g["inter_p"].T.ravel()], axis=1)
    # orig and inter are printed in f16.8 (half-ulp 5e-9): the bound is that
    # print error carried through the 9 weights plus the print of inter
    bound = 5e-9 * (np.abs(W).sum(axis=1, keepdims=True) + 1.0) * np.sqrt(2.0) * 1.01
    assert np.all(np.abs(W @ orig - inter) <= bound)


def test_interpolation_kat_reference_files():
    """_Winterp.dat shipped with the reference: L=16 (parent) <- L=11 (child)."""
    k = load_golden("interp_kat_L16_L11.npz")
    w, idx = core.interp_table(16, 11)
    W = np.zeros((512, 242))
    np.add.at(W, (np.repeat(np.arange(512), 9), idx.ravel()), w.ravel())
    Wb = np.zeros(tuple(k["W_shape"]))
    Wb[k["W_rows"], k["W_cols"]] = k["W_vals"]
    assert np.abs(W - Wb).max() < 1e-7
    np.testing.assert_allclose(np.sort(k["thetas_n1"]), np.sort(np.unique(
        np.round([(np.pi / 16 / 2) * (2 * t - 1) for t in range(1, 17)], 8))), atol=1e-7)
    orig = np.stack([k["orig_t"].T.ravel(), k["orig_p"].T.ravel()], axis=1)
    inter = np.stack([k["inter_t"].T.ravel(), k["inter_p"].T.ravel()], axis=1)
    anter = np.stack([k["anter_t"].T.ravel(), k["anter_p"].T.ravel()], axis=1)
    scale = np.abs(orig).max()
    assert np.abs(W @ orig - inter).max() < 1e-3 * scale
    assert np.abs(W.T @ inter - anter).max() < 1e-3 * np.abs(inter).max() * 3


def _ilu_kat_inputs():
    k = load_golden("ilu0_kat.npz")
    n = 10
    rows, cols, vals = k["i"], k["j"], k["s"]
    # coocsrC: stable bucketing by row keeps the input (column-sorted) order
    order = np.argsort(rows, kind="stable")
    a = np.zeros(len(vals) + 1, dtype=np.complex64)
    ja = np.zeros(len(vals) + 1, dtype=np.int32)
    a[1:] = vals[order]
    ja[1:] = cols[order]
    ia = np.zeros(n + 2, dtype=np.int32)
    ia[1] = 1
    for i in range(1, n + 1):
        ia[i + 1] = ia[i] + np.count_nonzero(rows == i)
    return k, n, a, ja, ia


def test_ilu0_kat_reference_files():
    """ilu0C on the 10x10 case of testSAAD (main.f90:719-826) against its dump."""
    k, n, a, ja, ia = _ilu_kat_inputs()
    ierr, alu, jlu, ju = core.ilu0_raw(n, a, ja, ia)
    assert ierr == 0
    # MSR -> (row, col, value) with the inverted diagonal in column position
    trip = []
    for i in range(1, n + 1):
        ent = [(int(jlu[q]), complex(alu[q])) for q in range(jlu[i], jlu[i + 1])]
        ent.append((i, complex(alu[i])))
        for c_, v in sorted(ent):
            trip.append((i, c_, v))
    nz = len(trip)
    assert nz == 47
    assert np.array_equal(k["ir"][:nz], [t[0] for t in trip])
    assert np.array_equal(k["jc"][:nz], [t[1] for t in trip])
    np.testing.assert_allclose(np.array([t[2] for t in trip]), k["ao"][:nz], atol=2e-6, rtol=2e-6)


def test_lusol0_inverts_ilu_product():
    k, n, a, ja, ia = _ilu_kat_inputs()
    ierr, alu, jlu, ju = core.ilu0_raw(n, a, ja, ia)
    # dense L, U from the factors; lusol0 must apply (LU)^-1
    Lm = np.eye(n, dtype=complex)
    Um = np.zeros((n, n), dtype=complex)
    for i in range(1, n + 1):
        Um[i - 1, i - 1] = 1.0 / complex(alu[i])
        for q in range(jlu[i], jlu[i + 1]):
            c_ = int(jlu[q])
            (Lm if c_ < i else Um)[i - 1, c_ - 1] = complex(alu[q])
    y = np.random.default_rng(3).standard_normal(n) + 1j * np.random.default_rng(4).standard_normal(n)
    x = core.lusol0_raw(n, y, alu, jlu, ju)
    np.testing.assert_allclose(Lm @ Um @ x, y, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("x", [0.37, 3.0, 12.5, 47.0, 98.6])
def test_spherical_bessel_against_scipy(x):
    nmax = int(x) + 8
    j, y = core.sph_bessel(nmax, x)
    n = np.arange(nmax + 1)
    jr, yr = sp.spherical_jn(n, x), sp.spherical_yn(n, x)
    np.testing.assert_allclose(j, jr, rtol=1e-11, atol=1e-14 * np.abs(jr).max())
    np.testing.assert_allclose(y, yr, rtol=1e-11)


def test_legendre_explicit_sum_and_recurrence():
    for x in (-0.93, -0.2, 0.0, 0.41, 0.999):
        Pe = core.legendre(20, x, 0)
        Pr = core.legendre(20, x, 1)
        ref = sp.eval_legendre(np.arange(21), x)
        np.testing.assert_allclose(Pr, ref, atol=1e-13)
        np.testing.assert_allclose(Pe, ref, atol=1e-9)


def test_mom_golden_dense_solve():
    """Dense MoM (Zmn_MoM, modMoM.f90:85-128) against the binary's run=mom currents."""
    try:
        g = load_golden("bin_ico3_mom.npz")
    except FileNotFoundError:
        pytest.skip("no dense-MoM fixture")
    if "I" not in g.files:
        pytest.skip("dense-MoM fixture has no currents")
    r = RWG(g["tris"])
    o = core.OracleMLFMA(r, lam=1.0, ladomax=0.3)
    Z = o.zmn_rows(0, r.N)
    d = core.direction_from_angles(90.0, 180.0)
    b = core.generar_onda(r, 1.0, d, core.ajustar_polariz(d, "VV"))
    res = np.linalg.norm(Z @ g["I"] - b) / np.linalg.norm(b)
    assert res < 5e-5, res


def test_ilu0_cgs_against_binary_run():
    """CGS + ILU0 (crear_precond ILU0 + CGSold with lusol0C) against the binary's
    run with precond=ilu0, errsolver=1e-3.  The first iterates agree to the
    printed digits; CGS then amplifies the two builds' rounding differences, so
    the iteration count is compared within 10 % and the currents at the level
    the 1e-3 stopping tolerance allows."""
    g = load_golden("bin_ico3_ilu0.npz")
    r = RWG(g["tris"])
    o = core.OracleMLFMA(r, lam=1.0, ladomax=0.3)
    d = core.direction_from_angles(90.0, 180.0)
    b = core.generar_onda(r, 1.0, d, core.ajustar_polariz(d, "VV"))
    assert o.ilu0() == 0
    out = o.cgs(b, tol=1e-3, maxit=3000, prec=True, history=True)
    assert out["status"] == 0
    assert abs(out["iters"] - int(g["iterations"])) <= 0.1 * int(g["iterations"])
    hist = g["res_hist"] / float(g["bnorm"])
    np.testing.assert_allclose(out["history"][:5], hist[:5], rtol=2e-5)
    assert np.linalg.norm(o.matvec(g["I"]) - b) / np.linalg.norm(b) < 1e-3
    assert np.linalg.norm(out["x"] - g["I"]) / np.linalg.norm(g["I"]) < 1e-2


def test_monostatic_sweep_matches_binary():
    """gen_rcs_monostatica (main.f90:967-1089): 4 angles, VV, warm-started CGS to 1e-8."""
    g = load_golden("bin_ico3_mono.npz")
    r = RWG(g["tris"])
    o = core.OracleMLFMA(r, lam=1.0, ladomax=0.3)
    phi, db, its = core.monostatic_sweep(o, 4, "VV", tol=1e-8)
    np.testing.assert_allclose(np.rad2deg(phi), g["rcsmono"][:, 0], atol=1e-9)
    assert np.abs(db - g["rcsmono"][:, 1]).max() < 1e-6
    assert its[-1] == int(g["iterations"])
    assert abs(int(its.sum()) - len(g["res_hist"])) <= 10


def test_five_level_octree_against_binary():
    """icosphere-4 at lambda = 0.5 (7680 RWG, 5 levels): the binary's converged currents."""
    g = load_golden("bin_ico4_mlfma.npz")
    r = RWG(g["tris"])
    o = core.OracleMLFMA(r, lam=0.5, ladomax=0.3)
    assert o.nlev == 5
    d = core.direction_from_angles(90.0, 180.0)
    pol = core.ajustar_polariz(d, "VV")
    b = core.generar_onda(r, 0.5, d, pol)
    assert np.linalg.norm(o.matvec(g["I"]) - b) / np.linalg.norm(b) < 5e-5
    th, ph = _bistatic_grid(5, 8)
    rcs = 10 * np.log10(core.sigma_rcs(r, 0.5, g["I"], pol, th, ph)).reshape(5, 8)
    assert np.abs(rcs - g["rcsbi"]).max() < 1e-4


def test_ilut_cgs_against_binary_run():
    """crear_precond ILUT (fill-in 5 %, drop 1e-3; ilutC + bsort2C) + CGSold
    against the binary's precond=ilut run: same iteration count, same
    residual history to the printed digits, same currents."""
    g = load_golden("bin_ico3_ilut.npz")
    r = RWG(g["tris"])
    o = core.OracleMLFMA(r, lam=1.0, ladomax=0.3)
    assert o.ilut(5.0, 1e-3) == 0
    d = core.direction_from_angles(90.0, 180.0)
    b = core.generar_onda(r, 1.0, d, core.ajustar_polariz(d, "VV"))
    out = o.cgs(b, tol=1e-6, maxit=3000, prec=True, history=True)
    assert out["status"] == 0 and out["iters"] == int(g["iterations"])
    hist = g["res_hist"] / float(g["bnorm"])
    np.testing.assert_allclose(out["history"][:20], hist[:20], rtol=2e-5)
    assert np.linalg.norm(out["x"] - g["I"]) / np.linalg.norm(g["I"]) < 1e-5
