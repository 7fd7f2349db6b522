"""Parity of the CUDA path with the oracle at the benchmark's own sizes.

Workloads:
  * the 122 880-RWG sphere (icosphere-6, r = 6 lambda, leaf 0.25 lambda):
    7 levels, K = 5202/1922/800/338/162 -- the octree the matvec/s figure is
    measured on, with the largest sampling grid (K = 5202 at level 3), whose
    anterpolation takes the large-shared-memory path;
  * the 30 720-RWG sphere (icosphere-5, r = 3 lambda): 6 levels.

Checks (MatxVec_MLFMA, modMLFMA.f90:1901-1946; llenar_campoCyB / llenar_campoA
:1783-1897; calc_E / sigmaRCS, modRCS.f90:339-432):
  * the FP64 matvec on the 8 seeded complex-Gaussian vectors
    (numpy.random.default_rng(0..7)) against the oracle, 1e-12 relative, with
    the same complex(4) near values on both sides;
  * the C, B and A fields of every level for one vector, 1e-12;
  * the FP32 operator (mixed-precision inner loop) against the FP64 one,
    2e-5 relative, one column and a block of 8 columns;
  * on the 30 720-RWG sphere, the RCS of a converged solve (x-polarised wave
    from -z, CGS + neighbourhood inverse to 1e-4): the GPU RCS against the
    oracle's sigmaRCS on the same currents (1e-9 dB), the currents against the
    oracle's operator (true residual), and the RCS against the Mie series
    (the method's own accuracy, stated in the assertion).
"""
import numpy as np
import pytest

from lywell_gb300 import MLFMA, RWG, meshes
from oracle import core, mie
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
def sphere6(gpu_lib):
    tris = meshes.icosphere(6, 6.0)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=0.25)
    o = core.OracleMLFMA(ORWG(tris), lam=1.0, ladomax=0.25)
    _, _, a = m.near_csr()
    o.set_near(a)
    yield m, o
    m.close()


@pytest.fixture(scope="module")
def sphere5(gpu_lib):
    tris = meshes.icosphere(5, 3.0)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=0.25)
    o = core.OracleMLFMA(ORWG(tris), lam=1.0, ladomax=0.25)
    _, _, a = m.near_csr()
    o.set_near(a)
    yield tris, m, o
    m.close()


def test_bench_octree_matches_oracle(sphere6):
    m, o = sphere6
    assert m.N == 122880 and m.nlev == 7 and m.nnz == o.nnz
    assert [m.levels[l]["K"] for l in range(3, 8)] == [5202, 1922, 800, 338, 162]
    for l in range(3, 8):
        for k in ("nb", "L", "K", "ntrans"):
            assert m.levels[l][k] == o.levels[l][k], (l, k)


def test_bench_matvec_8_seeded_vectors(sphere6):
    m, o = sphere6
    errs = []
    for x in _vectors(m.N):
        errs.append(_rel(m.matvec(x), o.matvec(x)))
    print("122880-RWG matvec rel. errors vs oracle:", ["%.2e" % e for e in errs])
    assert max(errs) < 1e-12


def test_bench_stage_fields_all_levels(sphere6):
    m, o = sphere6
    x = _vectors(m.N, [11])[0]
    m.matvec(x)
    o.matvec(x)
    for l in range(3, m.nlev + 1):
        Co, Bo, Ao = o.fields(l)
        assert _rel(m.debug_field(l, 0), Co) < 1e-12, ("C", l)
        assert _rel(m.debug_field(l, 1), Bo) < 1e-12, ("B", l)
        if l >= 4:
            assert _rel(m.debug_field(l, 2), Ao) < 1e-12, ("A", l)


def test_bench_fp32_operator_vs_fp64(sphere6):
    m, _ = sphere6
    X = np.stack(_vectors(m.N, range(20, 28)), axis=1)
    Y = m.matvec(X)
    e1 = _rel(m.matvec32(X[:, 0]), Y[:, 0])
    Y32 = m.matvec32(X)
    eb = max(_rel(Y32[:, k], Y[:, k]) for k in range(X.shape[1]))
    print(f"FP32 operator vs FP64: one column {e1:.2e}, block of 8 worst column {eb:.2e}")
    assert e1 < 2e-5 and eb < 2e-5


def test_cfg2_matvec_8_seeded_vectors(sphere5):
    _, m, o = sphere5
    assert m.nlev == 6
    for x in _vectors(m.N):
        assert _rel(m.matvec(x), o.matvec(x)) < 1e-12


def test_cfg2_rcs_vs_oracle_and_mie(sphere5):
    """x-polarised plane wave from -z on the r = 3 lambda sphere, solved to 1e-4."""
    tris, m, o = sphere5
    d = np.array([0.0, 0.0, 1.0])
    p = np.array([1.0, 0.0, 0.0], dtype=complex)
    b = m.excitation(d, p)
    assert _rel(b, core.generar_onda(ORWG(tris), 1.0, d, p)) < 1e-13
    assert m.nearinv() == 0
    out = m.cgs(b, errmax=1e-4, maxit=3000, precond="nearinv")
    assert out["status"] == "converged"
    # the currents satisfy the oracle's operator (the reference method) to the solve tolerance
    res = np.linalg.norm(o.matvec(out["x"]) - b) / np.linalg.norm(b)
    assert res < 1.01e-4, res
    th = np.deg2rad(np.arange(0.0, 181.0))
    r = ORWG(tris)
    worst_oracle, mie_err = 0.0, []
    for ph in (0.0, np.pi / 2):
        phs = np.full_like(th, ph)
        s = 10 * np.log10(m.rcs(out["x"], p, th, phs))
        so = 10 * np.log10(core.sigma_rcs(r, 1.0, out["x"], p, th, phs))
        worst_oracle = max(worst_oracle, float(np.abs(s - so).max()))
        mie_err.append(np.abs(s - 10 * np.log10(mie.sphere_rcs(3.0, 1.0, th, ph))))
    mie_err = np.concatenate(mie_err)
    print(f"cfg2 RCS: {out['iters']} CGS iterations; vs oracle sigmaRCS max {worst_oracle:.2e} dB; "
          f"vs Mie mean {mie_err.mean():.3f} dB, median {np.median(mie_err):.3f} dB, max {mie_err.max():.3f} dB")
    assert worst_oracle < 1e-9
    # the reference method's own accuracy at leaf 0.19 lambda (one centroid per
    # triangle in the patterns, multipoles clipped to kD): measured mean 0.71 dB,
    # max 2.34 dB against Mie (the r = 0.5 lambda case of test_gpu_fmm /
    # test_gpu_mom separates it from the mesh's own error with the dense MoM)
    assert mie_err.mean() < 1.0 and mie_err.max() < 3.0
