"""C ABI checks that need no GPU: the library builds and loads, exports every
symbol include/lywell_mlfma.h declares, validates arguments on the host, and
its RWG builder reproduces the oracle's restatement of the reference bit for
bit."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from lywell_gb300 import build as libbuild
from lywell_gb300 import meshes


@pytest.fixture(scope="module")
def lib():
    libbuild.build()
    from lywell_gb300 import _capi
    return _capi.load()


def _declared():
    src = open(os.path.join(ROOT, "include", "lywell_mlfma.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mlf_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 17
    from lywell_gb300 import _capi
    for n in names:
        assert hasattr(lib, n), n
        assert n in _capi.SIGNATURES, n


def test_init_rejects_bad_arguments(lib):
    h = C.c_void_p()
    rc = lib.mlf_init(C.byref(h), None, 0, None, None, None, None, None, None, None, None, None, 0, 0, None,
                      1.0, 0.5, 0)
    assert rc == -1
    assert b"invalid" in lib.mlf_last_error(None)


def test_null_context_calls_fail_cleanly(lib):
    assert lib.mlf_matvec(None, None, None, 1, 1) == -1
    assert lib.mlf_cgs(None, None, None, 1e-3, 10, 1, None, None, None, 0, None) == -1
    # tuning and diagnostics entry points: argument checks before any device work
    out = (C.c_double * 7)()
    assert lib.mlf_solve_phases(None, out, 7) == -1
    assert lib.mlf_set_lu_split(None, 1024) == -1
    a, b = C.c_int(), C.c_int()
    assert lib.mlf_get_lu_split(None, C.byref(a), C.byref(b)) == -1
    assert lib.mlf_set_block_engine(None, 4, 0) == -1


@pytest.mark.parametrize("body", ["ico3", "spheroid", "superellipsoid"])
def test_rwg_builder_matches_oracle(lib, body):
    from lywell_gb300 import RWG
    from oracle.rwg import RWG as ORWG
    if body == "ico3":
        t = meshes.icosphere(3, 1.0, quantum=2.0 ** -12)
    elif body == "spheroid":
        t = meshes.spheroid(3, (3.0, 0.75, 0.75), noise=0.01, seed=1234)
    else:
        t = meshes.superellipsoid(3, (4.0, 2.0, 2.0), 4.0)
    a, b = RWG(t), ORWG(t)
    assert a.N == b.N == 3 * t.shape[0] // 2
    for k in ("e_t", "e_po", "e_long", "e_centro", "t_baric", "t_baric_sub", "t_area"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert np.array_equal(a.p_coord[a.e_p], b.p_coord[b.e_p])


def test_rwg_builder_shared_node_topology(lib):
    """Each interior edge joins two triangles; T+ is the first listing."""
    from lywell_gb300 import RWG
    t = meshes.icosphere(2, 1.0)
    a = RWG(t)
    assert np.all(a.e_t[:, 0] < a.e_t[:, 1])
    # the opposite vertices are not on the edge
    for s in range(2):
        assert not np.any(a.e_po[:, s] == a.e_p[:, 0]) and not np.any(a.e_po[:, s] == a.e_p[:, 1])


def test_rwg_builder_open_and_degenerate_meshes(lib):
    """The one-call builder sizes its outputs by the bounds (P <= 3T, N <= 3T/2)
    and trims them: a lone triangle has no edge, an open strip's boundary
    sides make none, and a side shared by three triangles pairs the first two
    listings (the reference's first-occurrence rule) -- as the oracle does."""
    from lywell_gb300 import RWG
    from oracle.rwg import RWG as ORWG
    one = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], float)
    a = RWG(one)
    assert (a.N, a.P) == (0, 3) and a.e_p.shape == (0, 2) and a.p_coord.shape == (3, 3)
    fan = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 0, 0], [1, 0, 0], [0, -1, 0]],
                    [[0, 0, 0], [1, 0, 0], [0, 0, 1]]], float)
    strip = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[1, 0, 0], [1, 1, 0], [0, 1, 0]],
                      [[1, 0, 0], [2, 0, 0], [1, 1, 0]]], float)
    for t in (fan, strip):
        a, b = RWG(t), ORWG(t)
        assert a.N == b.N
        for k in ("e_t", "e_po", "e_long", "e_centro"):
            assert np.array_equal(getattr(a, k), getattr(b, k)), k
        assert np.array_equal(a.p_coord[a.e_p], b.p_coord[b.e_p])
    assert RWG(fan).e_t.tolist() == [[0, 1]]


def test_init_without_gpu_reports_no_device(lib):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("GPU present")
    from lywell_gb300 import MLFMA, RWG, MLFError
    with pytest.raises(MLFError) as e:
        MLFMA(RWG(meshes.icosphere(3, 1.0)), lam=1.0, ladomax=0.3)
    assert e.value.code == -8
