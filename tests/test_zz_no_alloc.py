"""The allocation-free matvec (mlf_matvec_device_noalloc), called through the
C ABI, against the regular device matvec.

Callers that cannot allocate device memory mid-solve (graph-captured
iterations, hosts whose device memory belongs to another runtime) use this
entry point; it keeps the multipole fields in the library's fixed device
scratch.  The file is named to be collected last.  Tolerance: the 1e-12
relative bound used for the FP64 matvec everywhere in these tests; the two
paths issue the same launches on different field buffers, so the results
are also checked to be bit-identical.
"""
import numpy as np
import pytest

from lywell_gb300 import MLFError, MLFMA, RWG, meshes

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_matches_device_matvec_twice(gpu_lib):
    import torch
    tris = meshes.icosphere(3, 1.0, quantum=2.0 ** -12)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=0.3)
    rng = np.random.default_rng(7)
    x = torch.from_numpy(rng.standard_normal(m.N) + 1j * rng.standard_normal(m.N)).to("cuda")
    y_ref = torch.zeros_like(x)
    y1 = torch.zeros_like(x)
    y2 = torch.zeros_like(x)
    s = torch.cuda.current_stream().cuda_stream
    m.matvec_device(x.data_ptr(), y_ref.data_ptr(), 1, s)
    m.matvec_device_noalloc(x.data_ptr(), y1.data_ptr(), s)
    m.matvec_device_noalloc(x.data_ptr(), y2.data_ptr(), s)
    torch.cuda.synchronize()
    ref = y_ref.cpu().numpy()
    assert _rel(y1.cpu().numpy(), ref) < 1e-12
    assert _rel(y2.cpu().numpy(), ref) < 1e-12
    assert np.array_equal(y1.cpu().numpy(), ref) and np.array_equal(y2.cpu().numpy(), ref)
    # a second, different input through the shared scratch
    x2 = torch.from_numpy(rng.standard_normal(m.N) + 1j * rng.standard_normal(m.N)).to("cuda")
    m.matvec_device(x2.data_ptr(), y_ref.data_ptr(), 1, s)
    m.matvec_device_noalloc(x2.data_ptr(), y1.data_ptr(), s)
    torch.cuda.synchronize()
    assert _rel(y1.cpu().numpy(), y_ref.cpu().numpy()) < 1e-12
    m.close()


def test_noalloc_rejects_octree_larger_than_scratch(gpu_lib):
    import torch
    tris = meshes.icosphere(5, 3.0)
    m = MLFMA(RWG(tris), lam=1.0, ladomax=0.25)
    x = torch.zeros(m.N, dtype=torch.complex128, device="cuda")
    y = torch.zeros_like(x)
    with pytest.raises(MLFError) as e:
        m.matvec_device_noalloc(x.data_ptr(), y.data_ptr())
    assert e.value.code == -1 and "scratch" in str(e.value)
    m.close()
