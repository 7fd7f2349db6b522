"""ilu0C on host arrays through the C ABI (mlf_ilu0_csr): no GPU needed.

The reference's ILU(0) (ilu0C, modIterativo.f90:1805-1976) reports a zero
pivot only through its ierr row and checks nothing about its CSR input.  The
library's entry point keeps the routine's arguments and results, and adds
host-side failure detection; these tests inject the failures on the host:
  * the 10 x 10 known-answer case of the reference's testSAAD
    (main.f90:719-826) and a random sparse matrix, bit-exact against the
    oracle's restatement;
  * a zeroed row, and a row without a diagonal entry, reported as that
    zero-pivot row (ierr = k, as ilu0C);
  * corrupted CSR arrays (ia(1) != 1, ia decreasing, a column out of range,
    columns out of order, duplicates) rejected with MLF_E_ARG naming the row.
"""
import numpy as np
import pytest

from lywell_gb300 import MLFError, build as libbuild, ilu0C
from oracle import core
from test_oracle_golden import _ilu_kat_inputs


@pytest.fixture(scope="module", autouse=True)
def lib():
    libbuild.build()


def _random_csr(n, seed, density=0.2):
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n):
        cols = np.flatnonzero(rng.random(n) < density)
        cols = np.union1d(cols, [i])
        rows.append(cols)
    ia = np.zeros(n + 1, dtype=np.int32)
    ia[0] = 1
    for i, c in enumerate(rows):
        ia[i + 1] = ia[i] + len(c)
    ja = np.concatenate(rows).astype(np.int32) + 1
    a = (rng.standard_normal(ja.size) + 1j * rng.standard_normal(ja.size)).astype(np.complex64)
    diag = np.array([ia[i] - 1 + np.searchsorted(rows[i], i) for i in range(n)])
    a[diag] += np.complex64(4.0 + 1.0j)
    return a, ja, ia


def _oracle(n, a, ja, ia):
    pa = np.concatenate([[0], a]).astype(np.complex64)
    pja = np.concatenate([[0], ja]).astype(np.int32)
    pia = np.concatenate([[0], ia]).astype(np.int32)
    ierr, alu, jlu, ju = core.ilu0_raw(n, pa, pja, pia)
    nnz = a.size
    return ierr, alu[1:nnz + 2], jlu[1:nnz + 2], ju[1:n + 1]


def test_kat_bitexact_against_oracle():
    _, n, a, ja, ia = _ilu_kat_inputs()
    alu, jlu, ju, ierr = ilu0C(n, a[1:], ja[1:], ia[1:])
    oerr, oalu, ojlu, oju = _oracle(n, a[1:], ja[1:], ia[1:])
    assert ierr == oerr == 0
    assert np.array_equal(jlu, ojlu) and np.array_equal(ju, oju)
    assert np.array_equal(alu.view(np.uint32), oalu.view(np.uint32))


@pytest.mark.parametrize("seed", [0, 1])
def test_random_csr_bitexact_against_oracle(seed):
    n = 60
    a, ja, ia = _random_csr(n, seed)
    alu, jlu, ju, ierr = ilu0C(n, a, ja, ia)
    oerr, oalu, ojlu, oju = _oracle(n, a, ja, ia)
    assert ierr == oerr == 0
    assert np.array_equal(jlu, ojlu) and np.array_equal(ju, oju)
    assert np.array_equal(alu.view(np.uint32), oalu.view(np.uint32))


@pytest.mark.parametrize("row", [1, 17, 60])
def test_zeroed_row_is_reported_as_zero_pivot(row):
    n = 60
    a, ja, ia = _random_csr(n, 2)
    a = a.copy()
    a[ia[row - 1] - 1:ia[row] - 1] = 0
    _, _, _, ierr = ilu0C(n, a, ja, ia)
    assert ierr == row
    assert _oracle(n, a, ja, ia)[0] == row


def test_missing_diagonal_is_a_zero_pivot():
    n = 30
    a, ja, ia = _random_csr(n, 3)
    row = 12
    lo, hi = ia[row - 1] - 1, ia[row] - 1
    keep = np.ones(a.size, dtype=bool)
    keep[lo + np.flatnonzero(ja[lo:hi] == row)] = False
    # zero the row's L part too, so nothing is eliminated into the missing pivot
    a = a.copy()
    a[lo:hi][ja[lo:hi] < row] = 0
    ia2 = ia.copy()
    ia2[row:] -= 1
    _, _, _, ierr = ilu0C(n, a[keep], ja[keep], ia2)
    assert ierr == row


@pytest.mark.parametrize("kind", ["ia1", "decreasing", "col_range", "col_zero", "order", "duplicate"])
def test_corrupted_csr_is_rejected(kind):
    n = 20
    a, ja, ia = _random_csr(n, 4)
    ja, ia = ja.copy(), ia.copy()
    row = 7
    lo = ia[row - 1] - 1
    if kind == "ia1":
        ia[0] = 0
        ia[1:] -= 1
        a, ja = a[1:], ja[1:]
        expect = "ia(1)"
    elif kind == "decreasing":
        ia[row] = ia[row - 1] - 1
        expect = f"row {row}"
    elif kind == "col_range":
        ja[lo] = n + 1
        expect = f"row {row}"
    elif kind == "col_zero":
        ja[lo] = 0
        expect = f"row {row}"
    elif kind == "order":
        assert ia[row] - ia[row - 1] >= 2
        ja[lo], ja[lo + 1] = ja[lo + 1], ja[lo]
        expect = f"row {row}"
    else:
        ja[lo + 1] = ja[lo]
        expect = f"row {row}"
    with pytest.raises(MLFError) as e:
        ilu0C(n, a, ja, ia)
    assert e.value.code == -1
    assert expect in str(e.value)
