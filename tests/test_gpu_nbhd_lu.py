"""The blocked FP32 LU of the neighbourhood-inverse preconditioner
(mlf_set_nearinv_precision 32, automatic above 768 unknowns per
neighbourhood) against the FP64 elimination and against numpy.

Workloads: the r = 1.5 lambda sphere (icosphere-4, 7680 RWG, a few hundred
unknowns per neighbourhood), where both eliminations run; the 30 720-RWG
prolate spheroid at the 722-RHS workload's density (about 145 bases per
0.25 lambda leaf box, neighbourhoods of ~2000 unknowns), where only the
blocked LU is practical.

Tolerances: FP32 elimination with partial pivoting, 1e-4 relative to the
FP64 rows (measured a few 1e-6); numpy inverses in FP64 of the same
complex(4) blocks, 1e-4.  The many-CTA path for the largest neighbourhoods
(mlf_set_lu_split) runs the same tiles in the same order as the one-CTA
kernel, so its rows are compared bit for bit.
"""
import time

import numpy as np
import pytest

from lywell_gb300 import MLFMA, RWG, meshes

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def test_blocked_fp32_matches_fp64_elimination(gpu_lib):
    m = MLFMA(RWG(meshes.icosphere(4, 1.5)), lam=1.0, ladomax=0.25)
    m.set_nearinv_precision(64)
    assert m.nearinv() == 0
    v64 = m.nearinv_values()
    m.set_nearinv_precision(32)
    assert m.nearinv() == 0
    v32 = m.nearinv_values()
    m.set_nearinv_precision(0)
    err = _rel(v32, v64)
    print(f"blocked FP32 LU vs FP64 elimination: {err:.2e}")
    assert err < 1e-4
    # the preconditioned solve behaves the same
    d = np.array([0.0, 0.0, 1.0])
    p = np.array([1.0, 0.0, 0.0], dtype=complex)
    b = m.excitation(d, p)
    it32 = m.cgs(b, errmax=1e-4, maxit=3000, precond="nearinv")
    m.set_nearinv_precision(64)
    assert m.nearinv() == 0
    it64 = m.cgs(b, errmax=1e-4, maxit=3000, precond="nearinv")
    m.set_nearinv_precision(0)
    assert it32["status"] == it64["status"] == "converged"
    assert abs(it32["iters"] - it64["iters"]) <= max(3, 0.05 * it64["iters"])
    m.close()


@pytest.fixture(scope="module")
def spheroid30k(gpu_lib):
    tris = meshes.spheroid(5, (1.5, 0.375, 0.375), noise=0.005, seed=1234)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=0.25)
    yield m
    m.close()


def test_many_cta_boxes_match_one_cta_kernel(spheroid30k):
    """The largest neighbourhoods factorised on many CTAs each give the same
    rows, bit for bit, as the one-CTA-per-box kernel."""
    m = spheroid30k
    m.set_lu_split(0)
    t0 = time.time()
    assert m.nearinv() == 0
    t_one = time.time() - t0
    v_one = m.nearinv_values()
    m.set_lu_split(1024)
    t0 = time.time()
    assert m.nearinv() == 0
    t_split = time.time() - t0
    nbig = m.lu_split()[1]
    v_split = m.nearinv_values()
    print(f"spheroid 30720 RWG: one CTA per box {t_one:.2f} s; {nbig} boxes on many CTAs {t_split:.2f} s")
    assert nbig > 0
    assert np.array_equal(v_split.view(np.float64), v_one.view(np.float64))


def test_large_neighbourhoods_against_numpy(spheroid30k):
    m = spheroid30k
    t0 = time.time()
    assert m.nearinv() == 0
    t_lu = time.time() - t0
    ia, ja, a = m.near_csr()
    ia, ja = ia - 1, ja - 1
    M = m.nearinv_values()
    lens = np.diff(ia)
    print(f"spheroid 30720 RWG: neighbourhoods of {lens.min()}..{lens.max()} unknowns "
          f"(mean {lens.mean():.0f}); blocked FP32 LU set-up {t_lu:.2f} s")
    assert lens.max() > 768
    # rows of three bases with the largest neighbourhood, against numpy's FP64 inverse of Z[S, S]
    g = int(np.argmax(lens))
    S = ja[ia[g]:ia[g + 1]]
    pos = {int(s): k for k, s in enumerate(S)}
    Zs = np.zeros((S.size, S.size), dtype=np.complex128)
    for r, s in enumerate(S):
        cols = ja[ia[s]:ia[s + 1]]
        keep = np.array([c in pos for c in cols])
        Zs[r, [pos[int(c)] for c in cols[keep]]] = a[ia[s]:ia[s + 1]][keep]
    inv = np.linalg.inv(Zs)
    rows = [g] + [int(s) for s in S if ia[s + 1] - ia[s] == S.size and np.array_equal(ja[ia[s]:ia[s + 1]], S)][1:3]
    for r in rows:
        got = M[ia[r]:ia[r + 1]]
        assert _rel(got, inv[pos[r]]) < 1e-4, r
