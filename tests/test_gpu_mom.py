"""Dense MoM operator on the GPU (MLF_FLAG_DENSE_MOM): against the oracle's
Zmn_MoM restatement, its CGS solve against the Mie series, and the MLFMA
matvec's error against it.

Tolerances: the dense matvec agrees with the oracle's matrix to 1e-12
relative (both FP64; different summation order); the RCS of the r = 0.5
lambda sphere to 0.2 dB of Mie (the oracle's own dense solve agrees to
0.09 dB).  The MLFMA operator differs from the dense one by about 2e-2
relative at r = 1.5 lambda: its far interactions use one centroid per
triangle in the radiation patterns (calcRad) where Zmn_MoM uses nine
sub-centroids, on top of the multipole truncation."""
import numpy as np
import pytest

from lywell_gb300 import MLFMA, MoM, RWG, meshes
from oracle import core, mie
from oracle.rwg import RWG as ORWG

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small():
    tris = meshes.icosphere(3, 0.5)
    m = MoM(RWG(tris), lam=1.0)
    o = core.OracleMLFMA(ORWG(tris), lam=1.0, ladomax=0.1)
    yield tris, m, o
    m.close()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_dense_matvec_matches_oracle(small):
    _, m, o = small
    Z = o.zmn_rows(0, m.N)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((m.N, 5)) + 1j * rng.standard_normal((m.N, 5))
    Y = m.matvec(X)
    assert _rel(Y, Z @ X) < 1e-12


def test_dense_cgs_rcs_against_mie(small):
    _, m, _ = small
    d = np.array([0.0, 0.0, 1.0])
    p = np.array([1.0, 0.0, 0.0], dtype=complex)
    b = m.excitation(d, p)
    out = m.cgs(b, errmax=1e-4, maxit=5000)
    assert out["status"] == "converged"
    th = np.deg2rad(np.arange(0.0, 181.0))
    for ph in (0.0, np.pi / 2):
        s = m.rcs(out["x"], p, th, np.full_like(th, ph))
        err = np.abs(10 * np.log10(s) - 10 * np.log10(mie.sphere_rcs(0.5, 1.0, th, ph)))
        assert err.max() < 0.2, err.max()


def test_octree_calls_refused(small):
    _, m, _ = small
    with pytest.raises(Exception):
        m.ilu0()
    with pytest.raises(Exception):
        m.nearinv()


def test_mlfma_matvec_error_against_dense():
    """r = 1.5 lambda icosphere-4 (7680 RWG): relative error of the MLFMA
    operator against the exact dense MoM operator on 4 seeded vectors."""
    tris = meshes.icosphere(4, 1.5)
    rwg = RWG(tris)
    dense = MoM(rwg, lam=1.0)
    ml = MLFMA(rwg, lam=1.0, ladomax=0.25)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((rwg.N, 4)) + 1j * rng.standard_normal((rwg.N, 4))
    err = _rel(ml.matvec(X), dense.matvec(X))
    print("MLFMA vs dense MoM relative matvec error", err)
    assert err < 3e-2
    dense.close()
    ml.close()
