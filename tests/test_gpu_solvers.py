"""Preconditioner and mixed-precision paths on the GPU (no counterpart in the
reference; checked against the oracle's restatement of the same algorithm
and against the FP64 path).  Needs a GB300.

Tolerances: neighbourhood-inverse rows 1e-11 relative (FP64 elimination
with partial pivoting on both sides, different rounding order); the FP32
operator agrees with the FP64 one to 2e-5 relative; a mixed-precision solve
meets the FP64 residual test and its RCS lies within 0.1 dB of the FP64
solve's.
"""
import numpy as np
import pytest

from lywell_gb300 import MLFMA, RWG, _capi, ajustar_polariz, direction, meshes
from oracle import core
from oracle.rwg import RWG as ORWG

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


@pytest.fixture(scope="module")
def ico4(gpu_lib):
    tris = meshes.icosphere(4, 1.5)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=0.25)
    o = core.OracleMLFMA(ORWG(tris), lam=1.0, ladomax=0.25)
    _, _, a = m.near_csr()
    o.set_near(a)
    yield tris, m, o
    m.close()


def test_nearinv_rows_match_oracle(ico4):
    _, m, o = ico4
    assert m.nearinv() == 0
    assert o.nearinv() == 0
    assert _rel(m.nearinv_values(), o.nearinv_values()) < 1e-11


def test_nearinv_is_local_inverse(ico4):
    """Row block of box b times Znear[S, S] gives the identity rows of b."""
    _, m, o = ico4
    ia, ja, z = m.near_csr()
    ia0, ja0 = ia - 1, ja - 1
    Mv = m.nearinv_values()
    ptr, bases = o.leaf_boxes()
    import scipy.sparse as sps
    Z = sps.csr_matrix((z.astype(np.complex128), ja0, ia0), shape=(m.N, m.N))
    for b in (0, len(ptr) // 2, len(ptr) - 2):
        own = bases[ptr[b]:ptr[b + 1]]
        S = ja0[ia0[own[0]]:ia0[own[0] + 1]]
        A = Z[S][:, S].toarray()
        rows = np.stack([Mv[ia0[g]:ia0[g + 1]] for g in own])
        E = rows @ A
        target = (S[None, :] == own[:, None]).astype(float)
        assert np.abs(E - target).max() < 1e-8


def test_cgs_nearinv_matches_oracle(ico4):
    _, m, o = ico4
    assert m.nearinv() == 0 and o.nearinv() == 0
    b = m.excitation(np.array([0, 0, 1.0]), np.array([1, 0, 0], complex))
    out = m.cgs(b, errmax=1e-4, maxit=2000, precond="nearinv")
    ref = o.cgs(b, tol=1e-4, maxit=2000, prec=2)
    assert out["status"] == "converged" and ref["status"] == 0
    assert abs(out["iters"] - ref["iters"]) <= max(3, 0.05 * ref["iters"])
    none = m.cgs(b, errmax=1e-4, maxit=3000)
    assert out["iters"] < 0.5 * none["iters"]
    res = np.linalg.norm(m.matvec(out["x"]) - b) / np.linalg.norm(b)
    assert res < 1.01e-4


def test_fp32_operator_close_to_fp64(ico4):
    _, m, _ = ico4
    rng = np.random.default_rng(3)
    for _ in range(3):
        x = rng.standard_normal(m.N) + 1j * rng.standard_normal(m.N)
        assert _rel(m.matvec32(x), m.matvec(x)) < 2e-5


def test_mixed_solve_meets_fp64_test_and_rcs(ico4):
    _, m, _ = ico4
    assert m.nearinv() == 0
    d = np.array([0, 0, 1.0])
    pol = np.array([1, 0, 0], complex)
    b = m.excitation(d, pol)
    ref = m.solve(b, errmax=1e-4, maxit=3000, precond="nearinv", mixed=False)
    mix = m.solve(b, errmax=1e-4, maxit=3000, precond="nearinv", mixed=True)
    assert ref["status"] == "converged" and mix["status"] == "converged"
    res = np.linalg.norm(m.matvec(mix["x"]) - b) / np.linalg.norm(b)
    assert res < 1e-4
    assert abs(res - mix["relres"]) < 1e-9
    th = np.deg2rad(np.arange(0, 181, 2.0))
    for phi in (0.0, np.pi / 2):
        s_ref = 10 * np.log10(m.rcs(ref["x"], pol, th, np.full_like(th, phi)))
        s_mix = 10 * np.log10(m.rcs(mix["x"], pol, th, np.full_like(th, phi)))
        assert np.abs(s_ref - s_mix).max() < 0.1


@pytest.mark.parametrize("engine", [2, 1])
def test_mixed_multi_rhs(ico4, engine):
    _, m, _ = ico4
    m.set_block_engine(engine)
    assert m.nearinv() == 0
    dirs = np.stack([direction(90.0, a) for a in (0.0, 45.0, 90.0)])
    pols = np.stack([ajustar_polariz(d, "VV") for d in dirs])
    B = m.excitation(dirs, pols)
    out = m.solve(B, errmax=1e-4, maxit=3000, precond="nearinv", mixed=True)
    for k in range(3):
        assert out["status"][k] == "converged"
        r = np.linalg.norm(m.matvec(out["x"][:, k]) - B[:, k]) / np.linalg.norm(B[:, k])
        assert r < 1e-4


@pytest.mark.parametrize("engine", [1, 0, 2, 3, 4])
@pytest.mark.parametrize("nrhs", [2, 3, 5, 20, 40, 70])
def test_fp32_multi_rhs_columns(ico4, nrhs, engine):
    """The batched FP32 operator (near field, aggregation and receive as dense
    per-box GEMMs on the tensor cores (3xTF32) or FP32 FMAs, 8- and 32-column
    tiles, ragged last tile; or one warp per basis over 2, 4 or 8 columns,
    ragged last chunk; translation over 1, 2, 4 or 8 columns per thread)
    against one column at a time."""
    _, m, _ = ico4
    m.set_block_engine(engine)
    rng = np.random.default_rng(11 + nrhs)
    X = rng.standard_normal((m.N, nrhs)) + 1j * rng.standard_normal((m.N, nrhs))
    Y = m.matvec32(X)
    for k in sorted({0, nrhs // 2, nrhs - 1}):
        # FP32 FMAs in another order: 1e-6; 3xTF32 drops the lo x lo term: 5e-6
        assert _rel(Y[:, k], m.matvec32(X[:, k])) < (5e-6 if engine in (1, 4) else 1e-6)
        assert _rel(Y[:, k], m.matvec(X[:, k])) < 2e-5


def test_own_box_inverse_apply(ico4):
    """Own-box mode: x = blockdiag(Z_bb^-1) y against numpy on the same near field."""
    _, m, o = ico4
    assert m.nearinv(own_only=True) == 0
    ia, ja, z = m.near_csr()
    import scipy.sparse as sps
    Z = sps.csr_matrix((z.astype(np.complex128), ja - 1, ia - 1), shape=(m.N, m.N))
    ptr, bases = o.leaf_boxes()
    y = np.random.default_rng(4).standard_normal(m.N) + 1j * np.random.default_rng(5).standard_normal(m.N)
    x = m.precond_apply(y, "nearinv")
    ref = np.zeros_like(y)
    for b in range(len(ptr) - 1):
        own = bases[ptr[b]:ptr[b + 1]]
        ref[own] = np.linalg.solve(Z[own][:, own].toarray(), y[own])
    assert _rel(x, ref) < 1e-10
    assert m.nearinv() == 0   # back to the full neighbourhood for the other tests


@pytest.mark.parametrize("engine", [1, 0, 2])
@pytest.mark.parametrize("ncols", [1, 6, 12, 40])
def test_own_box_fp32_block_apply(ico4, ncols, engine):
    """The FP32 own-box preconditioner of the mixed inner loop (per-box GEMMs
    for blocks of columns, 8- and 32-column tiles) against numpy block
    solves on the same near field; FP32 values and sums, so 1e-4 relative."""
    _, m, o = ico4
    m.set_block_engine(engine)
    assert m.nearinv(own_only=True) == 0
    try:
        ia, ja, z = m.near_csr()
        import scipy.sparse as sps
        Z = sps.csr_matrix((z.astype(np.complex128), ja - 1, ia - 1), shape=(m.N, m.N))
        ptr, bases = o.leaf_boxes()
        rng = np.random.default_rng(ncols)
        Y = rng.standard_normal((m.N, ncols)) + 1j * rng.standard_normal((m.N, ncols))
        X = m.precond_apply32(Y).reshape(m.N, ncols)
        ref = np.zeros_like(Y)
        for b in range(len(ptr) - 1):
            own = bases[ptr[b]:ptr[b + 1]]
            ref[own] = np.linalg.solve(Z[own][:, own].toarray(), Y[own])
        for k in range(ncols):
            assert _rel(X[:, k], ref[:, k]) < 1e-4
    finally:
        assert m.nearinv() == 0


@pytest.mark.parametrize("engine", [1, 0, 2, 4])
@pytest.mark.parametrize("ncols", [1, 3, 12, 40])
def test_neighbourhood_fp32_block_apply(ico4, ncols, engine):
    """The FP32 neighbourhood inverse of the mixed inner loop: one column by the
    CSR kernel, blocks of columns as near-pattern box-pair blocks through the
    GEMM engines or one warp per basis on the CSR values; against the FP64
    apply of the same preconditioner."""
    _, m, _ = ico4
    m.set_block_engine(engine)
    assert m.nearinv() == 0
    rng = np.random.default_rng(30 + ncols)
    Y = rng.standard_normal((m.N, ncols)) + 1j * rng.standard_normal((m.N, ncols))
    X32 = m.precond_apply32(Y).reshape(m.N, ncols)
    X64 = m.precond_apply(Y, "nearinv").reshape(m.N, ncols)
    for k in range(ncols):
        assert _rel(X32[:, k], X64[:, k]) < 1e-4


def test_autotune_block_covers_all_engines(ico4):
    """mlf_autotune_block picks a candidate block, an engine among the three and
    keeps them: a later batched operator call agrees with one column at a time."""
    _, m, _ = ico4
    res = m.autotune_block((4, 8, 16))
    assert res["block"] in (4, 8, 16)
    assert res["engine"] in _capi.ENGINES.values()
    assert all(t > 0 for t in res["per_rhs_ms"].values())
    rng = np.random.default_rng(77)
    X = rng.standard_normal((m.N, res["block"])) + 1j * rng.standard_normal((m.N, res["block"]))
    Y = m.matvec32(X)
    assert _rel(Y[:, -1], m.matvec32(X[:, -1])) < 5e-6
    m.set_block_engine(-1)



@pytest.mark.parametrize("nrhs", [1, 3])
def test_fp16_basis_meets_fp64_test_and_rcs(ico4, nrhs):
    """Mode 1 with the Krylov basis stored in FP16 (scaled by sqrt(N)): every
    column still meets the FP64 residual test, and the RCS stays within
    0.1 dB of the FP64 CGS solve's."""
    _, m, _ = ico4
    m.set_block_engine(-1)
    assert m.nearinv() == 0
    dirs = np.stack([direction(90.0, a) for a in (0.0, 60.0, 120.0)[:nrhs]])
    pols = np.stack([ajustar_polariz(d, "VV") for d in dirs])
    B = m.excitation(dirs, pols).reshape(m.N, nrhs)
    try:
        m.set_basis_precision(16)
        mix = m.solve(B, errmax=1e-4, maxit=3000, precond="nearinv", mixed=True)
    finally:
        m.set_basis_precision(32)
    X = np.asarray(mix["x"]).reshape(m.N, nrhs)
    th = np.deg2rad(np.arange(0, 181, 2.0))
    for k in range(nrhs):
        assert mix["status"][k] == "converged"   # 2-D right-hand sides give per-column lists
        assert np.linalg.norm(m.matvec(X[:, k]) - B[:, k]) / np.linalg.norm(B[:, k]) < 1e-4
        ref = m.solve(B[:, k], errmax=1e-4, maxit=3000, precond="nearinv", mixed=False)
        s_ref = 10 * np.log10(m.rcs(ref["x"], pols[k], th, np.zeros_like(th)))
        s_mix = 10 * np.log10(m.rcs(X[:, k], pols[k], th, np.zeros_like(th)))
        assert np.abs(s_ref - s_mix).max() < 0.1


@pytest.mark.parametrize("boxes,cols", [(2, 0), (4, 0), (4, 4)])
@pytest.mark.parametrize("nrhs", [1, 2, 3, 8, 11])
def test_translation_groups_match_per_box(ico4, nrhs, boxes, cols):
    """FP32 translation by groups of consecutive boxes over their merged far
    lists against one box at a time: the same sums in another order, 1e-6."""
    _, m, _ = ico4
    rng = np.random.default_rng(90 + nrhs)
    X = rng.standard_normal((m.N, nrhs)) + 1j * rng.standard_normal((m.N, nrhs))
    try:
        m.set_translation_group(boxes, cols)
        Yg = m.matvec32(X).reshape(m.N, nrhs)
        m.set_translation_group(1)
        Yb = m.matvec32(X).reshape(m.N, nrhs)
    finally:
        m.set_translation_group(0)
    for k in range(nrhs):
        assert _rel(Yg[:, k], Yb[:, k]) < 1e-6
        assert _rel(Yg[:, k], m.matvec(X[:, k])) < 2e-5
