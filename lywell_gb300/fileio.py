"""The reference's text file formats, so results drop into its tool chain.

* ``write_vector_c`` / ``read_vector_c`` — currents, one ``Re Im`` line per
  unknown, Fortran ``2f16.8`` (guardarVectorC, modGlobalMetod.f90:285-306).
* ``write_matrix_r`` / ``read_matrix_r`` — RCS grids, one row per line,
  ``<ncols>f16.8`` (guardarMatrizR, modGlobalMetod.f90:254-276); the bistatic
  file holds (ntheta x nphi) dB values, the monostatic one (angle, dB) rows.
* ``write_vector_r`` / ``write_vector_i`` — ``f16.8`` / ``I10`` per line
  (guardarVectorR / guardarVectorI, modGlobalMetod.f90:190-247).
* ASCII STL: :func:`lywell_gb300.meshes.write_stl` / ``read_stl``.

A value that does not fit ``f16.8`` prints as 16 asterisks, as Fortran does.
"""
from __future__ import annotations

import numpy as np

__all__ = ["write_vector_c", "read_vector_c", "write_matrix_r", "read_matrix_r", "write_vector_r",
           "write_vector_i", "f16_8"]


def f16_8(v: float) -> str:
    s = "%16.8f" % v
    return "*" * 16 if len(s) > 16 else s


def write_vector_c(path: str, v) -> None:
    v = np.asarray(v, dtype=np.complex128).ravel()
    with open(path, "w") as fh:
        for z in v:
            fh.write(f16_8(z.real) + f16_8(z.imag) + "\n")


def write_matrix_r(path: str, m) -> None:
    m = np.atleast_2d(np.asarray(m, dtype=np.float64))
    with open(path, "w") as fh:
        for row in m:
            fh.write("".join(f16_8(x) for x in row) + "\n")


def write_vector_r(path: str, v) -> None:
    with open(path, "w") as fh:
        for x in np.asarray(v, dtype=np.float64).ravel():
            fh.write(f16_8(x) + "\n")


def write_vector_i(path: str, v) -> None:
    with open(path, "w") as fh:
        for x in np.asarray(v).ravel():
            fh.write("%10d\n" % int(x))


def _fixed_fields(line: str, width: int = 16):
    line = line.rstrip("\n")
    return [line[i:i + width] for i in range(0, len(line), width) if line[i:i + width].strip()]


def read_matrix_r(path: str) -> np.ndarray:
    rows = []
    with open(path) as fh:
        for line in fh:
            f = _fixed_fields(line)
            if f:
                rows.append([np.nan if "*" in x else float(x) for x in f])
    return np.asarray(rows, dtype=np.float64)


def read_vector_c(path: str) -> np.ndarray:
    m = read_matrix_r(path)
    return m[:, 0] + 1j * m[:, 1]
