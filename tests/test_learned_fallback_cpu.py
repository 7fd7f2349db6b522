"""Host logic of the learned preconditioner (no GPU): the fallback, with a
stand-in operator recording the calls that solve_with_fallback makes, and
the damping choice from training traces (choose_gamma, fed the iteration
counts measured on the GB300).

The rule: keep the learned solve when it converged within the
unpreconditioned iteration count AND its true residual ||b - Z x|| / ||b||
meets the tolerance; otherwise solve again with the exact neighbourhood
inverse M1 under the correction (same test), then with ILU0 (the reference's
preconditioner, crear_precond main.f90:851-902), or without a preconditioner
when ILU0 meets a zero pivot."""
import numpy as np
import pytest

from lywell_gb300.learned import choose_gamma, solve_with_fallback


class FakeOperator:
    """Z = 2 I.  cgs() returns the scripted result for each preconditioner."""

    def __init__(self, n, learned_status="converged", learned_x_scale=1.0, ilu0_ierr=0, m1_status=None,
                 m1_x_scale=None):
        self.n = n
        self.calls = []
        self.learned_status = learned_status
        self.learned_x_scale = learned_x_scale
        self.ilu0_ierr = ilu0_ierr
        # the base M1 fails the same way unless told
        self.m1_status = m1_status or learned_status
        self.m1_x_scale = learned_x_scale if m1_x_scale is None else m1_x_scale
        self.m1 = False                                # the correction removed

    def matvec(self, x):
        return 2.0 * x

    def ilu0(self):
        self.calls.append("ilu0")
        return self.ilu0_ierr

    def cgs(self, b, errmax=1e-4, maxit=1000, precond=0):
        self.calls.append(("cgs", precond, maxit))
        if precond == "nearinv" and self.m1:
            self.calls[-1] = ("cgs", "m1", maxit)
            return dict(x=self.m1_x_scale * b / 2.0, iters=min(maxit, 9), relres=0.0, status=self.m1_status)
        if precond == "nearinv":
            return dict(x=self.learned_x_scale * b / 2.0, iters=min(maxit, 7), relres=0.0,
                        status=self.learned_status)
        return dict(x=b / 2.0, iters=11, relres=0.0, status="converged")


class FakeLearned:
    def __init__(self, gamma=0.5):
        self.installed = 0
        self.gamma = gamma

    def apply_to(self, m):
        self.installed += 1
        m.m1 = False
        return 0

    def remove_from(self, m):
        m.calls.append("remove")
        m.m1 = True
        return 0


@pytest.fixture
def b():
    rng = np.random.default_rng(0)
    return rng.standard_normal(50) + 1j * rng.standard_normal(50)


def test_learned_kept_when_converged(b):
    m, lp = FakeOperator(50), FakeLearned()
    out = solve_with_fallback(m, b, lp, plain_iters=30)
    assert out["used"] == "learned" and lp.installed == 1
    assert m.calls == [("cgs", "nearinv", 30)]
    assert out["true_relres"] < 1e-15


def test_falls_back_to_ilu0_past_the_plain_count(b):
    m, lp = FakeOperator(50, learned_status="maxit"), FakeLearned()
    out = solve_with_fallback(m, b, lp, plain_iters=1, maxit=900)
    assert out["used"] == "ilu0"
    assert m.calls == [("cgs", "nearinv", 1), "remove", ("cgs", "m1", 1), "ilu0", ("cgs", "ilu0", 900)]
    assert out["true_relres"] < 1e-15


def test_falls_back_to_m1_first(b):
    m, lp = FakeOperator(50, learned_status="maxit", m1_status="converged", m1_x_scale=1.0), FakeLearned()
    out = solve_with_fallback(m, b, lp, plain_iters=30)
    assert out["used"] == "neighbourhood inverse"
    assert m.calls == [("cgs", "nearinv", 30), "remove", ("cgs", "m1", 30)]
    assert out["true_relres"] < 1e-15


def test_no_m1_retry_without_a_correction(b):
    # gamma = 0: the learned solve already was the M1 solve
    m, lp = FakeOperator(50, learned_status="maxit"), FakeLearned(gamma=0.0)
    out = solve_with_fallback(m, b, lp, plain_iters=1, maxit=900)
    assert out["used"] == "ilu0"
    assert "remove" not in m.calls


def test_falls_back_when_true_residual_misses(b):
    # the recursion claims convergence but the currents are 10 % off
    m, lp = FakeOperator(50, learned_x_scale=1.1), FakeLearned()
    out = solve_with_fallback(m, b, lp, plain_iters=30, errmax=1e-4)
    assert out["used"] == "ilu0"
    assert "ilu0" in m.calls


def test_no_preconditioner_when_ilu0_has_a_zero_pivot(b):
    m, lp = FakeOperator(50, learned_status="stagnated", ilu0_ierr=17), FakeLearned()
    out = solve_with_fallback(m, b, lp, plain_iters=5)
    assert out["used"] == "none"
    assert m.calls[-1] == ("cgs", "none", 5000)


# ---- the damping choice from training traces (CGS iterations per body)

def test_gamma_with_a_clear_gain_is_chosen():
    # 7680-RWG superellipsoids: M1 1012, 1754, 231; gamma 0.5 a third of that
    base = [1012, 1754, 231]
    traces = {0.25: [560, 1122, 230], 0.5: [336, 645, 221], 0.75: [473, 604, 222], 1.0: [3001, 2874, 240]}
    g, r = choose_gamma(base, traces)
    assert g == 0.5 and r < 0.6


def test_gamma_within_the_margin_falls_back_to_m1():
    # 30 720-RWG superellipsoids at 60 bases per box: M1 231, 128, 90; the best gamma 4 % ahead
    base = [231, 128, 90]
    traces = {0.25: [222, 133, 99], 0.5: [222, 125, 87], 0.75: [222, 125, 85], 1.0: [230, 143, 104]}
    assert choose_gamma(base, traces)[0] == 0.0
    assert choose_gamma(base, traces, margin=1.0)[0] == 0.75


def test_no_gamma_helps():
    assert choose_gamma([100, 100], {0.5: [120, 110], 1.0: [150, 101]})[0] == 0.0
