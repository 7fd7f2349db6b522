"""Parity of the CUDA path (through the C ABI) with the CPU oracle and with
the reference binary's golden fixtures.  Needs a GB300.

Tolerances (FP64 path): stage fields and matvec 1e-12 relative when both
sides use the same complex(4) near-field values (the near-field fill itself
is compared separately: values may differ by one float32 rounding, 2^-23
relative, because the GPU and the host round the double-precision Zmn
differently in the last bit); ILU0 factors bit-exact; RCS 1e-9 dB.
"""
import numpy as np
import pytest

from conftest import load_golden
from lywell_gb300 import MLFMA, RWG, ajustar_polariz, direction, meshes
from oracle import core
from oracle.rwg import RWG as ORWG

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def _vectors(N, seeds=range(8)):
    out = []
    for s in seeds:
        rng = np.random.default_rng(s)
        out.append(rng.standard_normal(N) + 1j * rng.standard_normal(N))
    return out


@pytest.fixture(scope="module")
def ico3(gpu_lib):
    tris = meshes.icosphere(3, 1.0, quantum=2.0 ** -12)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=0.3)
    o = core.OracleMLFMA(ORWG(tris), lam=1.0, ladomax=0.3)
    yield tris, m, o
    m.close()


@pytest.fixture(scope="module")
def ico4(gpu_lib):
    tris = meshes.icosphere(4, 1.0, quantum=2.0 ** -12)
    m = MLFMA(RWG(tris), lam=0.5, ladomax=0.3)
    o = core.OracleMLFMA(ORWG(tris), lam=0.5, ladomax=0.3)
    yield tris, m, o
    m.close()


def test_octree_structure(ico3):
    _, m, o = ico3
    assert m.nlev == o.nlev and m.nnz == o.nnz
    for l in range(3, m.nlev + 1):
        for k in ("nb", "L", "K", "ntrans"):
            assert m.levels[l][k] == o.levels[l][k], (l, k)


def test_near_field_values(ico3):
    _, m, o = ico3
    ia, ja, a = m.near_csr()
    oia, oja, oa = o.near()
    assert np.array_equal(ia - 1, oia) and np.array_equal(ja - 1, oja)
    d = np.abs(a.astype(np.complex128) - oa.astype(np.complex128))
    rel = d / np.abs(oa.astype(np.complex128))
    worst = int(np.argmax(rel))
    row = int(np.searchsorted(oia, worst, side="right") - 1)
    print(f"near: {np.count_nonzero(d)} of {d.size} differ; max rel {rel.max():.3e} at row {row} "
          f"col {oja[worst]}: gpu {a[worst]} oracle {oa[worst]}")
    # one float32 rounding of either component: |dz| <= 2^-23 (|re| + |im|)
    one_ulp = 2.0 ** -23 * (np.abs(oa.real) + np.abs(oa.imag)) * 1.0001
    assert np.count_nonzero(d > one_ulp) <= d.size // 1000
    assert rel.max() < 1e-5


@pytest.mark.parametrize("case", ["ico3", "ico4"])
def test_matvec_parity_seeded(case, request):
    _, m, o = request.getfixturevalue(case)
    _, _, a = m.near_csr()
    o.set_near(a)
    for x in _vectors(m.N):
        y = m.matvec(x)
        yo = o.matvec(x)
        assert _rel(y, yo) < 1e-12


def test_stage_fields(ico4):
    _, m, o = ico4
    _, _, a = m.near_csr()
    o.set_near(a)
    x = _vectors(m.N, [11])[0]
    m.matvec(x)
    o.matvec(x)
    for l in range(3, m.nlev + 1):
        Co, Bo, Ao = o.fields(l)
        assert _rel(m.debug_field(l, 0), Co) < 1e-12, ("C", l)
        assert _rel(m.debug_field(l, 1), Bo) < 1e-12, ("B", l)
        if l >= 4:
            assert _rel(m.debug_field(l, 2), Ao) < 1e-12, ("A", l)


def test_matvec_multi_rhs_columns(ico3):
    _, m, _ = ico3
    X = np.stack(_vectors(m.N, [1, 2, 3]), axis=1)
    Y = m.matvec(X)
    for k in range(3):
        np.testing.assert_array_equal(Y[:, k], m.matvec(X[:, k]))


def test_matvec_linearity(ico4):
    _, m, _ = ico4
    x, y = _vectors(m.N, [5, 6])
    a, b = 0.3 - 1.1j, -2.0 + 0.25j
    lhs = m.matvec(a * x + b * y)
    rhs = a * m.matvec(x) + b * m.matvec(y)
    assert _rel(lhs, rhs) < 1e-13


def test_excitation_and_rcs(ico3):
    tris, m, o = ico3
    r = ORWG(tris)
    d = direction(90.0, 180.0)
    pol = ajustar_polariz(d, "VV")
    b = m.excitation(d, pol)
    bo = core.generar_onda(r, 1.0, d, pol)
    assert _rel(b, bo) < 1e-13
    d2 = direction(60.0, 30.0)
    pol2 = ajustar_polariz(d2, "HH")
    assert _rel(m.excitation(d2, pol2), core.generar_onda(r, 1.0, d2, pol2)) < 1e-13
    I = _vectors(m.N, [9])[0] * 1e-3
    th = np.linspace(0.01, np.pi - 0.01, 37)
    ph = np.linspace(0.0, 2 * np.pi, 37)
    s = m.rcs(I, pol, th, ph)
    so = core.sigma_rcs(r, 1.0, I, pol, th, ph)
    assert np.abs(10 * np.log10(s) - 10 * np.log10(so)).max() < 1e-9


def test_ilu0_bitexact_and_solve(ico3):
    _, m, o = ico3
    _, _, a = m.near_csr()
    o.set_near(a)
    assert m.ilu0() == 0
    assert o.ilu0() == 0
    alu, jlu, ju = m.ilu0_factors()
    oalu, ojlu, oju = o.ilu_factors()
    n1 = m.nnz + 1
    assert np.array_equal(jlu, ojlu[1:n1 + 1]) and np.array_equal(ju, oju[1:m.N + 1])
    assert np.array_equal(alu.view(np.uint32), oalu[1:n1 + 1].view(np.uint32))
    for y in _vectors(m.N, [21, 22]):
        assert _rel(m.lusol0(y), o.lusol0(y)) < 1e-12


def test_cgs_matches_oracle_and_binary(ico3):
    tris, m, o = ico3
    _, _, a = m.near_csr()
    o.set_near(a)
    d = direction(90.0, 180.0)
    b = m.excitation(d, ajustar_polariz(d, "VV"))
    out = m.cgs(b, errmax=1e-8, maxit=2000)
    ref = o.cgs(b, tol=1e-8, maxit=2000)
    assert out["status"] == "converged"
    assert abs(out["iters"] - ref["iters"]) <= 2
    assert _rel(out["x"], ref["x"]) < 1e-6
    g = load_golden("bin_ico3_mlfma.npz")
    assert abs(out["iters"] - int(g["iterations"])) <= 2
    assert _rel(out["x"], g["I"]) < 1e-5
    assert np.linalg.norm(m.matvec(g["I"]) - b) / np.linalg.norm(b) < 2e-5


def test_cgs_ilu0_matches_oracle(ico3):
    _, m, o = ico3
    _, _, a = m.near_csr()
    o.set_near(a)
    assert m.ilu0() == 0 and o.ilu0() == 0
    d = direction(90.0, 180.0)
    b = m.excitation(d, ajustar_polariz(d, "VV"))
    # ILU0-preconditioned CGS is erratic on this body (as in the reference), so
    # rounding differences grow along the iteration: compare the first steps
    # (measured growth: ~1e-16 at k = 1, ~1e-7 at k = 4)
    for k, tol in ((1, 1e-10), (2, 1e-9), (4, 1e-6)):
        out = m.cgs(b, errmax=1e-12, maxit=k, precond=1)
        ref = o.cgs(b, tol=1e-12, maxit=k, prec=True)
        assert out["iters"] == ref["iters"] == k
        assert _rel(out["x"], ref["x"]) < tol, k
        assert abs(out["relres"] - ref["relres"]) < tol * ref["relres"], k


def test_cgs_ilu0_against_binary_run(ico3):
    """The binary's precond=ilu0, errsolver=1e-3 run on the same mesh."""
    _, m, _ = ico3
    g = load_golden("bin_ico3_ilu0.npz")
    assert m.ilu0() == 0
    d = direction(90.0, 180.0)
    b = m.excitation(d, ajustar_polariz(d, "VV"))
    out = m.cgs(b, errmax=1e-3, maxit=3000, precond=1)
    assert out["status"] == "converged"
    assert abs(out["iters"] - int(g["iterations"])) <= 0.1 * int(g["iterations"])
    assert np.linalg.norm(m.matvec(g["I"]) - b) / np.linalg.norm(b) < 1e-3
    assert _rel(out["x"], g["I"]) < 1e-2


def test_cgs_multi_rhs_per_column(ico3):
    _, m, _ = ico3
    dirs = np.stack([direction(90.0, 180.0), direction(90.0, 90.0)])
    pols = np.stack([ajustar_polariz(dd, "VV") for dd in dirs])
    B = m.excitation(dirs, pols)
    out = m.cgs(B, errmax=1e-6, maxit=1000)
    for k in range(2):
        one = m.cgs(B[:, k], errmax=1e-6, maxit=1000)
        assert int(out["iters"][k]) == one["iters"]
        np.testing.assert_allclose(out["x"][:, k], one["x"], rtol=1e-10, atol=1e-16)


def test_monostatic_reference_sweep(ico3):
    """mlf_monostatic mode 0 against the oracle's sweep and the binary's RCSMONO file."""
    tris, m, o = ico3
    _, _, a = m.near_csr()
    o.set_near(a)
    out = m.monostatic(4, pol="VV", errmax=1e-8, maxit=3000, mode=0)
    phi, db, its = core.monostatic_sweep(o, 4, "VV", tol=1e-8)
    assert all(s == "converged" for s in out["status"])
    assert np.abs(out["sigma_db"] - db).max() < 1e-6
    # warm-started CGS to 1e-8: rounding differences shift the stopping iteration slightly
    assert np.all(np.abs(out["iters"] - its) <= np.maximum(3, 0.05 * its))
    g = load_golden("bin_ico3_mono.npz")
    assert np.abs(out["sigma_db"] - g["rcsmono"][:, 1]).max() < 1e-5


def test_monostatic_batched_modes(ico3):
    _, m, _ = ico3
    ref = m.monostatic(12, pol="HH", errmax=1e-6, maxit=3000, mode=0)
    b1 = m.monostatic(12, pol="HH", errmax=1e-6, maxit=3000, mode=1, block=5)
    b2 = m.monostatic(12, pol="HH", errmax=1e-6, maxit=3000, mode=2, block=5)
    # mode 3, block 5: runs of 3 angles (the last column has none), a ragged
    # last block; warm-started columns
    b3 = m.monostatic(12, pol="HH", errmax=1e-6, maxit=3000, mode=3, block=5)
    b4 = m.monostatic(12, pol="HH", errmax=1e-6, maxit=3000, mode=4, block=5)
    for out in (b1, b2, b3, b4):
        assert all(s == "converged" for s in out["status"])
        assert np.abs(out["sigma_db"] - ref["sigma_db"]).max() < 0.01
    # the warm-started angles (the 2nd and 3rd of every run) take fewer
    # iterations than the same angles solved cold in mode 2
    warm = [a for a in range(12) if a % 3]
    assert b3["iters"][warm].sum() < b2["iters"][warm].sum()


def test_five_level_octree_against_binary(gpu_lib):
    g = load_golden("bin_ico4_mlfma.npz")
    m = MLFMA(RWG(g["tris"]), lam=0.5, ladomax=0.3)
    assert m.nlev == 5
    d = direction(90.0, 180.0)
    pol = ajustar_polariz(d, "VV")
    b = m.excitation(d, pol)
    assert np.linalg.norm(m.matvec(g["I"]) - b) / np.linalg.norm(b) < 5e-5
    out = m.cgs(b, errmax=1e-7, maxit=3000)
    assert out["status"] == "converged"
    # CGS to 1e-7 over ~560 erratic iterations: the stopping iteration moves
    # with the summation order (oracle 564, binary 560); the solution does not
    assert abs(out["iters"] - int(g["iterations"])) <= 0.15 * int(g["iterations"])
    assert _rel(out["x"], g["I"]) < 1e-5
    m.close()


def test_ilut_bitexact_and_cgs(ico3):
    """ILUT (the reference default, fill-in 5 %, drop 1e-3) against the oracle's ilutC."""
    _, m, o = ico3
    _, _, a = m.near_csr()
    o.set_near(a)
    assert m.ilut(5.0, 1e-3) == 0
    assert o.ilut(5.0, 1e-3) == 0
    alu, jlu, ju = m.ilu0_factors()
    oalu, ojlu, oju = o.ilu_factors()
    n1 = alu.size
    assert np.array_equal(jlu, ojlu[1:n1 + 1]) and np.array_equal(ju, oju[1:m.N + 1])
    assert np.array_equal(alu.view(np.uint32), oalu[1:n1 + 1].view(np.uint32))
    d = direction(90.0, 180.0)
    b = m.excitation(d, ajustar_polariz(d, "VV"))
    out = m.cgs(b, errmax=1e-6, maxit=500, precond=1)
    ref = o.cgs(b, tol=1e-6, maxit=500, prec=True)
    assert out["status"] == "converged" and ref["status"] == 0
    assert abs(out["iters"] - ref["iters"]) <= 2
    assert _rel(out["x"], ref["x"]) < 1e-5


def test_ilut_against_binary_run(gpu_lib):
    g = load_golden("bin_ico3_ilut.npz")
    m = MLFMA(RWG(g["tris"]), lam=1.0, ladomax=0.3)
    assert m.ilut(5.0, 1e-3) == 0
    d = direction(90.0, 180.0)
    b = m.excitation(d, ajustar_polariz(d, "VV"))
    out = m.cgs(b, errmax=1e-6, maxit=500, precond=1)
    assert out["status"] == "converged"
    assert abs(out["iters"] - int(g["iterations"])) <= 2
    assert _rel(out["x"], g["I"]) < 1e-5
    m.close()


def test_contexts_with_different_grids_coexist(gpu_lib):
    """A context with larger sampling grids stays usable after a context with
    smaller ones is created (the kernels' dynamic shared-memory limit is
    process-wide and must not shrink to the newer context's need)."""
    big = MLFMA(RWG(meshes.icosphere(4, 1.0, quantum=2.0 ** -12)), lam=0.5, ladomax=0.3)
    x = _vectors(big.N, [3])[0]
    y0 = big.matvec(x)
    small = MLFMA(RWG(meshes.icosphere(3, 1.0, quantum=2.0 ** -12)), lam=1.0, ladomax=0.3)
    small.matvec(_vectors(small.N, [4])[0])
    y1 = big.matvec(x)
    assert np.array_equal(y0, y1)
    y32 = big.matvec32(x)
    assert _rel(y32, y0) < 2e-5
    small.close()
    big.close()
