"""The NumPy restatement of the learned-preconditioner MLP (oracle/mlp.py):
its backward pass against central finite differences of its own forward
pass (float64, no BF16 rounding), and the BF16 rounding helper."""
import numpy as np

from oracle import mlp


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    P = mlp.init(1) + rng.normal(0, 0.05, mlp.NPARAM)
    norm = np.concatenate([rng.normal(0, 1, 16), rng.uniform(0.5, 2, 16)])
    X = rng.normal(0, 1, (50, 16))
    T = rng.normal(0, 1, (50, 2))
    _, g = mlp.grad(P, norm, X, T, bf=False)
    eps = 1e-6
    for i in rng.choice(mlp.NPARAM, 60, replace=False):
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += eps
        Pm[i] -= eps
        fd = (mlp.grad(Pp, norm, X, T, bf=False)[0] - mlp.grad(Pm, norm, X, T, bf=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) < 1e-7 + 1e-6 * abs(g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, 3.14159, -2.5e-3], np.float32)
    r = mlp.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == np.float32(1.0078125)
    assert r[3] == np.float32(3.140625)
    assert abs(r[4] / v[4] - 1) < 2 ** -8
