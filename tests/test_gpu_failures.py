"""Failure detection through the C ABI, with every failure made on the host.

The reference has almost none: CGSold iterates until it converges, with no
cap and no check for NaN or stagnation (modIterativo.f90:384-490); ilu0C only
reports a zero pivot through its ierr row (modIterativo.f90:1962-1965), which
crear_precond prints and ignores (main.f90:896-902); the learned
preconditioner has no counterpart.  Here each case is injected from the host
(a NaN in the right-hand side, a zeroed near-field row written over the
context's values, an unreachable tolerance, a fallback threshold of one
iteration); no kernel is made to fault or hang, and the context stays usable
after each case.
"""
import numpy as np
import pytest

from lywell_gb300 import MLFMA, RWG, MLFError, meshes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    m = MLFMA(RWG(meshes.icosphere(3, 1.0, quantum=2.0 ** -12)), lam=1.0, ladomax=0.3)
    yield m
    m.close()


def _rhs(m):
    d = np.array([0.0, 0.0, 1.0])
    p = np.array([1.0, 0.0, 0.0], dtype=complex)
    return m.excitation(d, p)


def test_nan_rhs_reports_not_finite(ctx):
    b = _rhs(ctx)
    b[123] = np.nan
    out = ctx.cgs(b, errmax=1e-4, maxit=200)
    assert out["status"] == "not_finite" and out["iters"] <= 2
    mixed = ctx.solve(b, errmax=1e-4, maxit=200, mixed=True)
    assert mixed["status"] == "not_finite"
    # a clean solve on the same context afterwards
    ok = ctx.cgs(_rhs(ctx), errmax=1e-4, maxit=2000)
    assert ok["status"] == "converged"


def test_zeroed_near_row_is_the_ilu0_zero_pivot(ctx):
    ia, ja, a = ctx.near_csr()
    assert ctx.nearinv() == 0
    row = 37                                            # 1-based, as ilu0C's ierr
    bad = a.copy()
    bad[ia[row - 1] - 1:ia[row] - 1] = 0
    ctx.set_near_values(bad)
    # overwriting the near values drops the preconditioners built on them
    with pytest.raises(MLFError):
        ctx.cgs(_rhs(ctx), errmax=1e-4, maxit=10, precond="nearinv")
    assert ctx.ilu0() == row
    with pytest.raises(MLFError):
        ctx.cgs(_rhs(ctx), errmax=1e-4, maxit=10, precond="ilu0")
    ctx.set_near_values(a)
    assert ctx.ilu0() == 0
    out = ctx.cgs(_rhs(ctx), errmax=1e-3, maxit=3000, precond="ilu0")
    assert out["status"] == "converged"


def test_forced_stagnation_cgs(gpu_lib):
    """ILU0-preconditioned CGS, the reference's method, on a body where it does
    not converge: the superellipsoid of exponent 4, 2 x 1 x 1 lambda
    (icosphere-4, 7680 RWG), x-polarised wave from -z.  The reference would
    iterate there without end; with a window of 100 iterations the solve stops
    as stagnated, and without one it runs to its cap."""
    m = MLFMA(RWG(meshes.superellipsoid(4, (2.0, 1.0, 1.0), 4.0)), lam=1.0, ladomax=0.25)
    b = _rhs(m)
    assert m.ilu0() == 0
    window = 100
    m.set_stagnation(window)
    out = m.cgs(b, errmax=1e-4, maxit=3000, precond="ilu0")
    m.set_stagnation(0)
    assert out["status"] == "stagnated" and out["iters"] < 3000
    h = m.cgs_history()
    assert len(h) == out["iters"]
    # no new minimum within the last `window` iterations
    assert int(np.argmin(h)) + 1 <= out["iters"] - window
    capped = m.cgs(b, errmax=1e-4, maxit=out["iters"] + 20, precond="ilu0")
    assert capped["status"] == "maxit"
    m.close()


def test_forced_stagnation_mixed(ctx):
    b = _rhs(ctx)
    ctx.set_gmres_restart(100)
    ctx.set_stagnation(300)
    try:
        out = ctx.solve(b, errmax=1e-30, maxit=40000, mixed=True)
    finally:
        ctx.set_stagnation(0)
        ctx.set_gmres_restart(0)
    assert out["status"] == "stagnated" and out["iters"] < 40000
    assert out["relres"] < 1e-12


def test_learned_fallback_takes_ilu0(ctx):
    """A learned solve that cannot converge within the threshold (one
    iteration) falls back to ILU0, judged by the true FP64 residual."""
    from lywell_gb300.learned import MLP, LearnedPreconditioner, solve_with_fallback
    assert ctx.nearinv() == 0
    lp = LearnedPreconditioner(MLP(seed=3), tscale=1.0, gamma=0.5)
    b = _rhs(ctx)
    out = solve_with_fallback(ctx, b, lp, plain_iters=1, errmax=1e-3, maxit=3000)
    assert out["used"] == "ilu0"
    assert out["status"] == "converged"
    true = np.linalg.norm(ctx.matvec(out["x"]) - b) / np.linalg.norm(b)
    assert abs(out["true_relres"] - true) <= 1e-12 * max(true, 1e-300) + 1e-15
    assert true < 2e-3
