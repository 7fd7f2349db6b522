"""ORACLE — test infrastructure, not part of the product.

A CPU restatement of MLFMAxwell's iterative solve (gabsantamaria/lywell, serial
Fortran 90): RWG construction (``oracle.rwg``), the MLFMA setup and matvec,
ILU0 + its triangular solves, CGS, the plane-wave excitation and the RCS
far-field sum (``oracle/mlfma_oracle.c`` through ``oracle.core``), plus the
Mie series for a PEC sphere (``oracle.mie``).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline /
reference arm use this package, and only as the checker or as the timed CPU
baseline.  The lywell_gb300 library never imports it.

Parity pinning: tests/golden/ holds fixtures produced by running the
reference's own binary on synthetic meshes, and the reference's committed
known-answer files; tests/test_oracle_golden.py checks this oracle against
them.
"""
