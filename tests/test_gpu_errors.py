"""Error behaviour of the C ABI on a live context: invalid arguments and
calls out of order return status codes (never abort the process), and the
context stays usable afterwards.  The reference stops or loops on these
(CGSold has no iteration cap, inicializar_MLFMA stops on small bodies); the
library reports them."""
import ctypes as C

import numpy as np
import pytest

from lywell_gb300 import MLFMA, MoM, RWG, meshes
from lywell_gb300._capi import MLFError, load

pytestmark = pytest.mark.gpu

E_ARG, E_TOO_SMALL, E_STATE = -1, -2, -6


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    m = MLFMA(RWG(meshes.icosphere(3, 1.0)), lam=1.0, ladomax=0.3)
    yield m
    m.close()


def _p(a):
    return C.c_void_p(a.ctypes.data)


def test_matvec_argument_checks(ctx):
    L = load()
    x = np.zeros(ctx.N, dtype=np.complex128)
    y = np.zeros(ctx.N, dtype=np.complex128)
    assert L.mlf_matvec(ctx.handle, _p(x), _p(y), 0, ctx.N) == E_ARG        # no columns
    assert L.mlf_matvec(ctx.handle, _p(x), _p(y), 1, ctx.N - 1) == E_ARG    # ld < N
    assert L.mlf_matvec(ctx.handle, None, _p(y), 1, ctx.N) == E_ARG
    assert L.mlf_cgs(ctx.handle, _p(x), None, 1e-4, 0, 1, _p(y), None, None, 0, None) == E_ARG


def test_preconditioner_out_of_order(ctx):
    L = load()
    y = np.ones(ctx.N, dtype=np.complex128)
    x = np.zeros(ctx.N, dtype=np.complex128)
    if L.mlf_ilu0_solve(ctx.handle, _p(y), _p(x), 1) != E_STATE:
        pytest.skip("an ILU factorisation is already present on this context")
    with pytest.raises(MLFError):
        ctx.solve(y, errmax=1e-4, maxit=10, precond="nearinv", mixed=True)


def test_context_usable_after_errors(ctx):
    rng = np.random.default_rng(0)
    x = rng.standard_normal(ctx.N) + 1j * rng.standard_normal(ctx.N)
    y1 = ctx.matvec(x)
    assert np.all(np.isfinite(y1))
    assert np.array_equal(ctx.matvec(x), y1)


def test_small_body_reports_too_small(gpu_lib):
    # r = 0.5 lambda: nivel_max = 3, where inicializar_MLFMA stops
    with pytest.raises(MLFError) as e:
        MLFMA(RWG(meshes.icosphere(3, 0.5)), lam=1.0, ladomax=0.25)
    assert e.value.code == E_TOO_SMALL


def test_cgs_iteration_cap_and_status(ctx):
    d = np.array([0.0, 0.0, 1.0])
    p = np.array([1.0, 0.0, 0.0], dtype=complex)
    b = ctx.excitation(d, p)
    out = ctx.cgs(b, errmax=1e-14, maxit=5)
    assert out["status"] == "maxit" and out["iters"] == 5


def test_dense_context_refuses_octree_calls(gpu_lib):
    m = MoM(RWG(meshes.icosphere(2, 0.5)), lam=1.0)
    for call in (lambda: m.ilu0(), lambda: m.nearinv(), lambda: m.matvec32(np.ones(m.N, complex)),
                 lambda: m.near_csr()):
        with pytest.raises(MLFError) as e:
            call()
        assert e.value.code == E_STATE
    m.close()
