"""Learned-preconditioner network on the GPU: the library's hand-written
forward / backward kernels against the NumPy oracle (oracle/mlp.py) on the
same BF16-rounded parameters, and training by the library's Adam kernels.

Tolerances: the kernels accumulate in FP32 in a different order from the
oracle's float64 sums, and a BF16 rounding of a hidden activation can land on
the other side of a tie; outputs agree to 1e-3 and gradients to 3e-3 in
relative norm."""
import numpy as np
import pytest

from oracle import mlp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def net():
    from lywell_gb300.learned import MLP
    n = MLP(seed=3)
    yield n
    n.close()


def _problem(seed, n=3000):
    rng = np.random.default_rng(seed)
    P = (mlp.init(seed) + rng.normal(0, 0.02, mlp.NPARAM)).astype(np.float32)
    norm = np.concatenate([rng.normal(0, 0.5, 16), rng.uniform(0.5, 2, 16)]).astype(np.float32)
    X = rng.normal(0, 1, (n, 16)).astype(np.float32)
    T = rng.normal(0, 1, (n, 2)).astype(np.float32)
    return P, norm, X, T


def test_forward_matches_oracle(net):
    import torch
    P, norm, X, _ = _problem(1, n=3001)          # a partial last tile
    net.set_params(P, norm)
    Y = net.forward(torch.from_numpy(X).cuda()).cpu().numpy()
    ref, _ = mlp.forward(P, norm, X)
    assert np.linalg.norm(Y - ref) / np.linalg.norm(ref) < 1e-3


def test_gradient_matches_oracle(net):
    import torch
    P, norm, X, T = _problem(2)
    net.set_params(P, norm)
    loss, G = net.grad(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())
    lref, gref = mlp.grad(P, norm, X, T)
    assert abs(loss - lref) < 1e-4 * lref
    assert np.linalg.norm(G - gref) / np.linalg.norm(gref) < 3e-3
    # per parameter block as well
    o = 0
    for name, shp in mlp.SHAPES:
        k = int(np.prod(shp))
        g, r = G[o:o + k], gref[o:o + k]
        assert np.linalg.norm(g - r) <= 3e-3 * np.linalg.norm(r) + 1e-9, name
        o += k


def test_training_reduces_loss(net):
    import torch
    rng = np.random.default_rng(5)
    X = rng.normal(0, 1, (20000, 16)).astype(np.float32)
    W = rng.normal(0, 0.5, (16, 2))
    T = np.tanh(X @ W).astype(np.float32)          # a smooth target the network can fit
    net.set_params(mlp.init(7).astype(np.float32),
                   np.concatenate([np.zeros(16), np.ones(16)]).astype(np.float32))
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    l0, _ = net.grad(Xd, Td)
    hist = net.train(Xd, Td, steps=400, batch=4096, lr=2e-3)
    l1, _ = net.grad(Xd, Td)
    assert np.all(np.isfinite(hist))
    assert l1 < 0.1 * l0


# ---------------------------------------------------------------------------
# tokens, 2-ring targets and the trained preconditioner

def _leaf_cells(o):
    cen = o.centres(o.nlev)
    side = o.levels[o.nlev]["side"]
    return np.rint((cen - cen.min(0)) / side).astype(int)


def test_ring_targets_match_numpy(gpu_lib):
    """2-ring targets (FP32 elimination on the device) against numpy inverses of
    the same complex(4) blocks: r = 1 lambda icosphere-3 (1920 RWG)."""
    from lywell_gb300 import MLFMA, RWG, meshes
    from lywell_gb300.learned import tokens
    from oracle import core
    from oracle.rwg import RWG as ORWG
    tris = meshes.icosphere(3, 1.0)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=0.25)
    o = core.OracleMLFMA(ORWG(tris), lam=1.0, ladomax=0.25)
    assert m.nearinv() == 0
    X, T, bad = tokens(m, True)
    assert bad == 0
    T = T.cpu().numpy()
    ia, ja, z = m.near_csr()
    ia, ja = ia - 1, ja - 1
    M1 = m.nearinv_values()
    Zd = o.zmn_rows(0, m.N).astype(np.complex64).astype(np.complex128)
    ptr, bases = o.leaf_boxes()
    cells = _leaf_cells(o)
    diag = np.array([z[ia[i] + np.searchsorted(ja[ia[i]:ia[i + 1]], i)] for i in range(m.N)], dtype=np.complex128)
    s = 1 / np.sqrt(diag)
    ref = np.zeros(len(ja), dtype=np.complex128)
    for b in range(len(ptr) - 1):
        ring = np.where(np.abs(cells - cells[b]).max(1) <= 2)[0]
        S = np.sort(np.concatenate([bases[ptr[j]:ptr[j + 1]] for j in ring]))
        Mi = np.linalg.inv(Zd[np.ix_(S, S)])
        for g in bases[ptr[b]:ptr[b + 1]]:
            cols = ja[ia[g]:ia[g + 1]]
            ref[ia[g]:ia[g + 1]] = Mi[np.searchsorted(S, g)][np.searchsorted(S, cols)]
    rows = np.repeat(np.arange(m.N), np.diff(ia))
    Dh = (ref - M1) / (s[rows] * s[ja])
    got = T[:, 0] + 1j * T[:, 1]
    assert np.linalg.norm(got - Dh) / np.linalg.norm(Dh) < 2e-3
    # features: the scaled near value and the scaled exact M1 entry
    Xh = X.cpu().numpy()
    zh = Xh[:, 0] + 1j * Xh[:, 1]
    assert np.linalg.norm(zh - z * s[rows] * s[ja]) / np.linalg.norm(zh) < 1e-5
    m.close()


def test_learned_preconditioner_gain(gpu_lib):
    """Train on three seeded superellipsoids (exponent U[2, 6], semi-axes
    (2, 1, 1) lambda x U[0.85, 1.15], icosphere-4: 7680 RWG, the mesh density
    of the held-out body), pick the damping from CGS traces, and solve the
    held-out superellipsoid (exponent 4, 2 x 1 x 1 lambda) from -z,
    x-polarised.  The learned preconditioner must converge, beat ILU0 and the
    unpreconditioned solve, and take strictly fewer iterations than the exact
    neighbourhood inverse M1 it corrects: the gain of the network over the
    method without it."""
    from lywell_gb300 import MLFMA, RWG, meshes
    from lywell_gb300.learned import solve_with_fallback, train
    rng = np.random.default_rng(7)
    d = np.array([0.0, 0.0, 1.0])
    p = np.array([1.0, 0.0, 0.0], dtype=complex)
    ctxs, bs = [], []
    for _ in range(3):
        e = rng.uniform(2, 6)
        ax = np.array([2.0, 1.0, 1.0]) * rng.uniform(0.85, 1.15, 3)
        mt = MLFMA(RWG(meshes.superellipsoid(4, tuple(ax), e)), lam=1.0, ladomax=0.25)
        assert mt.nearinv() == 0
        ctxs.append(mt)
        bs.append(mt.excitation(d, p))
    lp = train(ctxs, bs, steps=3000, batch=8192, lr=1e-3, seed=0)
    assert np.all(np.isfinite(lp.loss_history))
    assert lp.loss_history[-200:].mean() < 0.5 * lp.loss_history[:50].mean()
    for mt in ctxs:
        mt.close()
    m = MLFMA(RWG(meshes.superellipsoid(4, (2.0, 1.0, 1.0), 4.0)), lam=1.0, ladomax=0.25)
    b = m.excitation(d, p)
    none = m.cgs(b, errmax=1e-4, maxit=3000)
    plain = int(none["iters"]) if none["status"] == "converged" else 3000
    assert m.ilu0() == 0
    ilu = m.cgs(b, errmax=1e-4, maxit=3000, precond="ilu0")
    assert m.nearinv() == 0
    exact = m.cgs(b, errmax=1e-4, maxit=3000, precond="nearinv")
    out = solve_with_fallback(m, b, lp, plain_iters=plain)
    print("gamma", lp.gamma, "trace", lp.trace, "none", none["iters"], none["status"], "ilu0", ilu["iters"],
          ilu["status"], "exact nbhd", exact["iters"], "learned", out["iters"], out["used"])
    assert out["used"] == "learned"
    assert out["true_relres"] < 1.01e-4
    assert out["iters"] < plain
    assert ilu["status"] != "converged" or out["iters"] < ilu["iters"]
    assert exact["status"] == "converged"
    assert out["iters"] < exact["iters"]
    m.close()
