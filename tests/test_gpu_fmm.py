"""Single-level FMM on the GPU (MLF_FLAG_FMM) against the oracle's
restatement of modFMM.f90 (ora_create_fmm) and the Mie series.

Workload: the r = 0.5 lambda sphere, icosphere-3 (1920 RWG), x-polarised
wave from -z, boxes of 0.25 lambda (56 boxes) and of the reference's
lambda/2 (8 boxes, all near: the FMM is then the dense MoM).

Tolerances: grid, lists and sizes exact; matvec 1e-12 relative with the same
complex(4) near values on both sides; CGS + ILU0 iteration counts within 2;
RCS within 0.6 dB of Mie for 0.25 lambda boxes (the FMM's own truncation
error, 4e-3 relative in the matvec, shows there; the oracle gives the same)
and within 0.2 dB with lambda/2 boxes."""
import numpy as np
import pytest

from lywell_gb300 import FMM, RWG, meshes
from oracle import core, mie
from oracle.rwg import RWG as ORWG

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module", params=[0.25, 0.5])
def fmm(request):
    tris = meshes.icosphere(3, 0.5)
    m = FMM(RWG(tris), lam=1.0, side=request.param)
    o = core.OracleMLFMA(ORWG(tris), lam=1.0, ladomax=request.param, fmm=True)
    yield request.param, m, o
    m.close()


def test_grid_matches_oracle(fmm):
    _, m, o = fmm
    assert m.nlev == o.nlev == 3
    for key in ("nb", "L", "K", "ntrans", "nfar"):
        assert m.levels[3][key] == o.levels[3][key], key
    assert m.nnz == o.nnz
    ia, ja, _ = m.near_csr()
    oia, oja, _ = o.near()
    assert np.array_equal(ia - 1, oia) and np.array_equal(ja - 1, oja)


def test_matvec_matches_oracle(fmm):
    _, m, o = fmm
    _, _, a = m.near_csr()
    o.set_near(a)
    rng = np.random.default_rng(0)
    for _ in range(3):
        x = rng.standard_normal(m.N) + 1j * rng.standard_normal(m.N)
        assert _rel(m.matvec(x), o.matvec(x)) < 1e-12


def test_cgs_ilu0_and_rcs(fmm):
    side, m, o = fmm
    _, _, a = m.near_csr()
    o.set_near(a)
    d = np.array([0.0, 0.0, 1.0])
    p = np.array([1.0, 0.0, 0.0], dtype=complex)
    b = m.excitation(d, p)
    assert m.ilu0() == 0 and o.ilu0() == 0
    out = m.cgs(b, errmax=1e-4, maxit=3000, precond="ilu0")
    ref = o.cgs(b, tol=1e-4, maxit=3000, prec=True)
    assert out["status"] == "converged"
    assert abs(out["iters"] - ref["iters"]) <= 2
    th = np.deg2rad(np.arange(0.0, 181.0))
    for ph in (0.0, np.pi / 2):
        s = m.rcs(out["x"], p, th, np.full_like(th, ph))
        err = np.abs(10 * np.log10(s) - 10 * np.log10(mie.sphere_rcs(0.5, 1.0, th, ph)))
        assert err.max() < (0.6 if side < 0.5 else 0.2), err.max()
