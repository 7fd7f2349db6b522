"""Profiling runs of single operators, for ncu captures and engine comparisons.

  python -m lywell_gb300.profiling fp32 --mesh spheroid5 --nrhs 64 --engine 4 --steps 5
  python -m lywell_gb300.profiling fp64 --mesh sphere5 --steps 5
  python -m lywell_gb300.profiling nearinv --mesh spheroid4 --steps 1

fp32: the batched FP32 operator (mlf_matvec32_device) on `nrhs` random
columns with a chosen multi-column engine (-1 automatic, 0 FMA box blocks,
1 mma.sync box blocks, 2/3 warp engine, 4 tcgen05 box blocks) and tile
width; fp64: the FP64 matvec (mlf_matvec_device) on one column.  Each prints
one JSON line: time per call (CUDA events over `steps` calls after two
warm-up calls) and the per-stage times of one more call.  nearinv: the
27-box neighbourhood-inverse set-up (mlf_nearinv, the blocked FP32 LU for
large neighbourhoods), one untimed call and `steps` timed ones, with the
neighbourhood sizes.

Meshes: spheroid4 / spheroid5 = 7 680 / 30 720-RWG prolate spheroids with
the 722-RHS workload's mesh density (icosphere-4 / -5, semi-axes 0.75 x
0.1875 x 0.1875 / 1.5 x 0.375 x 0.375 lambda, ~145 bases per leaf box); spheroid6 = the 122 880-RWG spheroid of that workload
(3 x 0.75 x 0.75 lambda); sphere5 / sphere6 = the r = 3 / 6 lambda
icospheres (30 720 / 122 880 RWG, ~7-11 bases per leaf box).  Leaf boxes of
0.25 lambda, lambda = 1 m.
"""
from __future__ import annotations

import argparse
import ctypes
import json

import numpy as np

MESHES = ("spheroid4", "spheroid5", "spheroid6", "sphere5", "sphere6")


def make_mesh(name):
    from . import meshes
    if name == "sphere6":
        return meshes.icosphere(6, 6.0)
    if name == "sphere5":
        return meshes.icosphere(5, 3.0)
    if name == "spheroid6":
        return meshes.spheroid(6, (3.0, 0.75, 0.75), noise=0.01, seed=1234)
    if name == "spheroid4":
        return meshes.spheroid(4, (0.75, 0.1875, 0.1875), noise=0.0025, seed=1234)
    return meshes.spheroid(5, (1.5, 0.375, 0.375), noise=0.005, seed=1234)


def run(kind, mesh, nrhs=64, steps=5, engine=-1, cols=0):
    import torch
    from . import MLFMA, RWG, _capi

    m = MLFMA(RWG(make_mesh(mesh)), lam=1.0, ladomax=0.25)
    if kind == "fp32" and (engine >= 0 or cols):
        m.set_block_engine(engine, cols)
    lib = _capi.load()
    n = nrhs if kind == "fp32" else 1
    X = torch.randn(n, m.N, dtype=torch.complex128, device="cuda")
    Y = torch.empty_like(X)
    stream = torch.cuda.Stream()            # a real stream handle (the default stream's is 0)
    torch.cuda.set_stream(stream)
    s = ctypes.c_void_p(stream.cuda_stream)
    xp, yp = ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(Y.data_ptr())
    if kind == "fp32":
        call = lambda: lib.mlf_matvec32_device(m.handle, xp, yp, n, m.N, s)
    else:
        call = lambda: lib.mlf_matvec_device(m.handle, xp, yp, n, m.N, s)
    for _ in range(2):
        assert call() == 0
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        call()
    e1.record()
    torch.cuda.synchronize()
    m.set_profiling(True)
    assert call() == 0
    torch.cuda.synchronize()
    stages = [float(v) for v in m.stage_times()]
    m.set_profiling(False)
    out = {"profile": f"{kind} operator", "mesh": mesh, "N": m.N, "nrhs": n, "near_nnz": m.nnz,
           "engine": engine, "cols": cols, "ms_per_call": e0.elapsed_time(e1) / steps,
           "stage_ms": dict(zip(["aggregation", "interpolation", "translation", "anterpolation", "receive_near"],
                                stages))}
    m.close()
    return out


def run_nearinv(mesh, steps=1):
    import time
    import torch
    from . import MLFMA, RWG

    m = MLFMA(RWG(make_mesh(mesh)), lam=1.0, ladomax=0.25)
    assert m.nearinv() == 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        assert m.nearinv() == 0
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    ia, _, _ = m.near_csr()
    rows = np.diff(np.asarray(ia))
    out = {"profile": "neighbourhood inverse", "mesh": mesh, "N": m.N, "near_nnz": m.nnz,
           "neighbourhood_mean": float(rows.mean()), "neighbourhood_max": int(rows.max()),
           "seconds_per_call": dt}
    m.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("kind", choices=["fp32", "fp64", "nearinv"])
    ap.add_argument("--mesh", default="spheroid5", choices=MESHES)
    ap.add_argument("--nrhs", type=int, default=64)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--engine", type=int, default=-1)
    ap.add_argument("--cols", type=int, default=0)
    a = ap.parse_args(argv)
    if a.kind == "nearinv":
        print(json.dumps(run_nearinv(a.mesh, a.steps)), flush=True)
    else:
        print(json.dumps(run(a.kind, a.mesh, a.nrhs, a.steps, a.engine, a.cols)), flush=True)


if __name__ == "__main__":
    main()
