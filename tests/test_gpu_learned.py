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
