"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run once, in a container that holds the reference tree (read-only) at
``/root/reference``:

    python tests/golden/make_golden.py

What it does:
  1. Runs the reference's shipped Release binary ``MLFMAxwell`` as a black box
     (stdin ``key=value`` script, the interface of ``waitcommands``,
     main.f90:221-368) on synthetic icosphere meshes written as ASCII STL with
     coordinates quantised to 2^-12 m, so that the program's decimal parser
     reads back exactly the doubles this library uses.  It collects the
     current vectors (``*_IMLFMA.dat`` / ``*_IMoM.dat``, f16.8 "Re Im" lines,
     modGlobalMetod.f90:285-306), the bistatic RCS grids (``*_RCSBI_*.dat``)
     and the monostatic sweep (``*_RCSMONOVV.dat``), and the interpolation dump
     that ``test_interp`` (modMLFMA.f90:1637-1779) writes at the 10th matvec.
  2. Converts the known-answer files the reference ships for its own checks
     (the ILU0 10x10 case ``i.dat j.dat s.dat si.dat -> ilu0_*``, main.f90:719-826,
     and the L=16 -> L=11 interpolation dump ``_Winterp.dat`` etc.) into
     compact ``.npz`` fixtures.

Nothing at test time reads the reference tree; the tests only read the
``.npz`` files written here.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from lywell_gb300 import meshes  # noqa: E402

REF = "/root/reference"
BIN = os.path.join(REF, "Release_Intel64", "MLFMAxwell")
QUANTUM = 2.0 ** -12

# name -> (mesh builder, script lines, timeout s)
CASES = {
    # 4-level octree (L = 15 / 11), 1920 RWG, unpreconditioned CGS to 1e-8.
    "ico3_mlfma": (lambda: meshes.icosphere(3, 1.0, quantum=QUANTUM),
                   ["lambda=1", "ladomax=0.3", "precond=no", "errsolver=1e-8",
                    "rcsmono.active=false", "rcsbi.ntheta=5", "rcsbi.nphi=8",
                    "run=mlfma"], 600),
    # same body, dense MoM (the near-field entries are Zmn_MoM).
    "ico3_mom": (lambda: meshes.icosphere(3, 1.0, quantum=QUANTUM),
                 ["lambda=1", "precond=no", "errsolver=1e-8",
                  "rcsmono.active=false", "rcsbi.ntheta=5", "rcsbi.nphi=8",
                  "run=mom"], 900),
    # same body, CGS + ILU0 preconditioner.
    "ico3_ilu0": (lambda: meshes.icosphere(3, 1.0, quantum=QUANTUM),
                  ["lambda=1", "ladomax=0.3", "precond=ilu0", "errsolver=1e-3",
                   "rcsmono.active=false", "rcsbi.ntheta=5", "rcsbi.nphi=8",
                   "run=mlfma"], 900),
    # same body, CGS + ILUT (the reference default: fill-in 5 %, drop 1e-3).
    "ico3_ilut": (lambda: meshes.icosphere(3, 1.0, quantum=QUANTUM),
                  ["lambda=1", "ladomax=0.3", "precond=ilut", "ilut.fillin=5", "ilut.droptol=0.001",
                   "errsolver=1e-6", "rcsmono.active=false", "rcsbi.ntheta=5", "rcsbi.nphi=8",
                   "run=mlfma"], 900),
    # monostatic sweep, 4 angles of phi, VV, warm-started CGS.
    "ico3_mono": (lambda: meshes.icosphere(3, 1.0, quantum=QUANTUM),
                  ["lambda=1", "ladomax=0.3", "precond=no", "errsolver=1e-8",
                   "rcsmono.active=true", "rcsmono.samples=4", "polariz=VV",
                   "run=mlfma"], 900),
    # 5-level octree (L = 23 / 15 / 10), 7680 RWG.
    "ico4_mlfma": (lambda: meshes.icosphere(4, 1.0, quantum=QUANTUM),
                   ["lambda=0.5", "ladomax=0.3", "precond=no", "errsolver=1e-7",
                    "rcsmono.active=false", "rcsbi.ntheta=5", "rcsbi.nphi=8",
                    "run=mlfma"], 1800),
}


def _read_matrix(path):
    rows = []
    with open(path) as fh:
        for line in fh:
            w = line.split()
            if w:
                rows.append([float(x) for x in w])
    return np.asarray(rows, dtype=np.float64)


def _read_cvec(path):
    m = _read_matrix(path)
    return m[:, 0] + 1j * m[:, 1]


def _run_case(name, build, script, timeout):
    tris = build()
    work = tempfile.mkdtemp(prefix="golden_" + name + "_")
    shutil.copy(BIN, work)
    meshes.write_stl(os.path.join(work, "body.stl"), tris, digits=12)
    lines = ["filename=body.stl", "testname=T"] + script
    t0 = time.time()
    # The program exits with a Fortran end-of-file error once stdin is
    # exhausted; that is its normal end in script mode.
    try:
        proc = subprocess.run(["./MLFMAxwell"], input="\n".join(lines) + "\n", cwd=work,
                              capture_output=True, text=True, timeout=timeout)
        log = proc.stdout
        timed_out = False
    except subprocess.TimeoutExpired as exc:
        log = exc.stdout.decode() if isinstance(exc.stdout, bytes) else (exc.stdout or "")
        timed_out = True
    dt = time.time() - t0
    out = {"tris": tris, "script": np.array("\n".join(lines)), "wall_s": np.array(dt),
           "timed_out": np.array(timed_out)}
    iters = [l.split() for l in log.splitlines() if l.strip().startswith("Iterac:")]
    out["iterations"] = np.array(int(iters[-1][1]) if iters else -1)
    # per-iteration residual history "Iterac: i residuo r de b - time"
    out["res_hist"] = np.array([float(w[3]) for w in iters]) if iters else np.zeros(0)
    out["bnorm"] = np.array(float(iters[-1][5]) if iters else 0.0)
    for fn, key in (("T_IMLFMA.dat", "I"), ("T_IMoM.dat", "I"),
                    ("T_RCSBI_FMM-MLFMA.dat", "rcsbi"), ("T_RCSBI_MoM.dat", "rcsbi"),
                    ("T_RCSMONOVV.dat", "rcsmono")):
        p = os.path.join(work, fn)
        if os.path.exists(p):
            out[key] = _read_cvec(p) if key == "I" else _read_matrix(p)
    if os.path.exists(os.path.join(work, "_orig_t_R.dat")):
        for part in ("orig", "inter", "anter"):
            for pol in ("t", "p"):
                re = _read_matrix(os.path.join(work, f"_{part}_{pol}_R.dat"))
                im = _read_matrix(os.path.join(work, f"_{part}_{pol}_I.dat"))
                out[f"{part}_{pol}"] = re + 1j * im
        w = _read_matrix(os.path.join(work, "_Winterp.dat"))
        out["W_rows"], out["W_cols"] = np.nonzero(w)
        out["W_vals"] = w[out["W_rows"], out["W_cols"]]
        out["W_shape"] = np.array(w.shape)
    shutil.rmtree(work)
    print(f"{name}: {dt:.1f}s, timed_out={timed_out}, iterations={int(out['iterations'])}, "
          f"keys={sorted(out)}", flush=True)
    return out


def _reference_kats():
    rd = os.path.join(REF, "Release_Intel64")

    def vec(fn):
        with open(os.path.join(rd, fn)) as fh:
            vals = fh.read().split()
        return vals

    i = np.array([int(x) for x in vec("i.dat")[1:]])
    j = np.array([int(x) for x in vec("j.dat")[1:]])
    sr = np.array([float(x) for x in vec("s.dat")[1:]])
    si = np.array([float(x) for x in vec("si.dat")[1:]])
    ao_r = np.array([float(x) for x in vec("ilu0_ao_real")])
    ao_i = np.array([float(x) for x in vec("ilu0_ao_imag")])
    ir = np.array([int(x) for x in vec("ilu0_ir")])
    jc = np.array([int(x) for x in vec("ilu0_jc")])
    np.savez_compressed(os.path.join(HERE, "ilu0_kat.npz"), i=i, j=j, s=sr + 1j * si,
                        ao=ao_r + 1j * ao_i, ir=ir, jc=jc)
    w = _read_matrix(os.path.join(rd, "_Winterp.dat"))
    r, c = np.nonzero(w)
    interp = {"W_rows": r, "W_cols": c, "W_vals": w[r, c], "W_shape": np.array(w.shape)}
    for part in ("orig", "inter", "anter"):
        for pol in ("t", "p"):
            re = _read_matrix(os.path.join(rd, f"_{part}_{pol}_R.dat"))
            im = _read_matrix(os.path.join(rd, f"_{part}_{pol}_I.dat"))
            interp[f"{part}_{pol}"] = re + 1j * im
    for fn in ("_thetas_n", "_thetas_n1", "_phis_n", "_phis_n1"):
        interp[fn.strip("_")] = _read_matrix(os.path.join(rd, fn + ".dat")).ravel()
    np.savez_compressed(os.path.join(HERE, "interp_kat_L16_L11.npz"), **interp)
    print("reference KATs written")


def main(argv):
    names = argv[1:] or list(CASES)
    if "kat" in names or not argv[1:]:  # reference known-answer files
        _reference_kats()
    for name in names:
        if name in CASES:
            b, s, to = CASES[name]
            out = _run_case(name, b, s, to)
            np.savez_compressed(os.path.join(HERE, f"bin_{name}.npz"), **out)


if __name__ == "__main__":
    main(sys.argv)
