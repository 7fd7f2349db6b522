"""The tcgen05 engine (block engine 4: near field, leaf aggregation and leaf
receive on tcgen05.mma) against the mma.sync box-block engine (engine 1) and
the FP64 operator.

Workloads: a 30 720-RWG prolate spheroid at the 722-RHS workload's mesh
density (icosphere-5, semi-axes 1.5 x 0.375 x 0.375 lambda, about 145 bases
per 0.25 lambda leaf box), and the same body with 0.5 lambda leaf boxes
(several hundred bases per box: boxes split over tiles of at most 160 rows).
The aggregation splits the 2K directions of a leaf box (324 with 0.25 lambda
leaves) over tiles of at most 160 as well.

Tolerances: engine 4 splits each FP32 operand of the near field and the
aggregation into scaled FP16 hi and lo parts (22 significant bits, as the
3xTF32 split of the receive and of engine 1) and drops the lo x lo term.
Against the FP64 operator both engines stay within the FP32 operator's own
accuracy: 2e-5 with 0.25 lambda leaves, 1e-4 with 0.5 lambda leaves (larger
sampling grids and longer FP32 translation sums).  Measured on the 30 720-RWG
spheroid: engine 4 1.0e-5 and 4.5e-5, engine 1 1.8e-5 and 7.7e-5, so the two
engines differ by up to 7.7e-6 and 3.3e-5; the same bounds apply between them.
"""
import numpy as np
import pytest

from lywell_gb300 import MLFMA, RWG, meshes

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


@pytest.fixture(scope="module", params=[0.25, 0.5])
def spheroid(request, gpu_lib):
    tris = meshes.spheroid(5, (1.5, 0.375, 0.375), noise=0.005, seed=1234)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=request.param)
    yield request.param, m
    m.close()


@pytest.mark.parametrize("nrhs", [2, 64, 70, 128])
def test_tc_engine_matches_mma_engine(spheroid, nrhs):
    side, m = spheroid
    rng = np.random.default_rng(100 + nrhs)
    X = rng.standard_normal((m.N, nrhs)) + 1j * rng.standard_normal((m.N, nrhs))
    m.set_block_engine(1)
    Y1 = m.matvec32(X)
    m.set_block_engine(4)
    Y4 = m.matvec32(X)
    Y4b = m.matvec32(X)
    m.set_block_engine(-1)
    assert np.array_equal(Y4, Y4b)            # deterministic: each output written by one CTA
    tol = 2e-5 if side == 0.25 else 1e-4
    worst = max(_rel(Y4[:, k], Y1[:, k]) for k in range(nrhs))
    e64 = {k: (_rel(Y4[:, k], m.matvec(X[:, k])), _rel(Y1[:, k], m.matvec(X[:, k]))) for k in sorted({0, nrhs - 1})}
    print(f"nrhs {nrhs}: tcgen05 vs mma.sync worst column {worst:.2e}; vs FP64 (tcgen05, mma.sync) "
          + " ".join(f"{a:.2e}/{b:.2e}" for a, b in e64.values()))
    assert worst < tol
    for a, b in e64.values():
        assert a < tol and b < tol


def test_tc_engine_mixed_solve(spheroid):
    """A batched mixed-precision solve on engine 4 meets the FP64 residual test."""
    side, m = spheroid
    if side != 0.25:
        pytest.skip("one body is enough for the solve")
    m.set_block_engine(4)
    assert m.nearinv(own_only=True) == 0
    d = np.stack([np.array([-np.cos(a), -np.sin(a), 0.0]) for a in np.deg2rad([0.0, 30.0, 60.0, 90.0])])
    p = np.tile(np.array([0, 0, 1.0], dtype=complex), (4, 1))
    B = m.excitation(d, p)
    out = m.solve(B, errmax=1e-4, maxit=4000, precond="nearinv", mixed=True)
    m.set_block_engine(-1)
    for k in range(4):
        assert out["status"][k] == "converged"
        assert np.linalg.norm(m.matvec(out["x"][:, k]) - B[:, k]) / np.linalg.norm(B[:, k]) < 1e-4
