"""Build the CUDA extension in-tree: lywell_gb300/lib/liblywell_mlfma.so.

nvcc compiles the device translation units for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host C++ is compiled with
``-ffp-contract=off`` so that set-up tables round the same way on x86-64 and
aarch64.  Translation units are compiled in parallel, then linked with the
static CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
OUT = os.path.join(OUT_DIR, "liblywell_mlfma.so")
OBJ_DIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["mlf_setup.cpp", "mlf_device.cu", "mlf_solver.cu", "mlf_capi.cu", "mlf_noalloc.cu", "mlf_precond.cu", "mlf_mixed.cu", "mlf_sweep.cu", "mlf_nearblk.cu", "mlf_nearwarp.cu", "mlf_autotune.cu", "mlf_mlp.cu", "mlf_learned.cu", "mlf_mom.cu", "mlf_tc.cu", "mlf_nbhd_lu.cu"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src: str) -> str:
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path, os.path.join(CSRC, "mlf_internal.h"), os.path.join(CSRC, "mlf_tcgen05.h"),
            os.path.join(os.path.dirname(HERE), "include", "lywell_mlfma.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [_nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd.insert(1, "-x=cu")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(o) for o in objs):
        return OUT
    cmd = [_nvcc(), "-shared", *ARCH, "-o", OUT, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", OUT)
    return OUT


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
