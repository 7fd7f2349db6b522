"""The reference's file formats (f16.8 currents and RCS grids)."""
import numpy as np

from conftest import load_golden
from lywell_gb300 import fileio


def test_vector_c_round_trip_matches_reference_precision(tmp_path):
    g = load_golden("bin_ico3_mlfma.npz")
    p = tmp_path / "T_IMLFMA.dat"
    fileio.write_vector_c(p, g["I"])
    lines = open(p).read().splitlines()
    assert len(lines) == g["I"].size and all(len(l) == 32 for l in lines)
    back = fileio.read_vector_c(p)
    # the fixture itself came from the reference's f16.8 file: the round trip is exact
    np.testing.assert_array_equal(back, g["I"])


def test_matrix_r_layout(tmp_path):
    g = load_golden("bin_ico3_mlfma.npz")
    p = tmp_path / "T_RCSBI.dat"
    fileio.write_matrix_r(p, g["rcsbi"])
    lines = open(p).read().splitlines()
    assert len(lines) == g["rcsbi"].shape[0]
    assert all(len(l) == 16 * g["rcsbi"].shape[1] for l in lines)
    np.testing.assert_array_equal(fileio.read_matrix_r(p), g["rcsbi"])


def test_f16_8_edge_cases():
    assert fileio.f16_8(-1e-10) == "     -0.00000000"
    assert fileio.f16_8(0.5) == "      0.50000000"
    assert fileio.f16_8(1e9) == "*" * 16
