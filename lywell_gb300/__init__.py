"""lywell_gb300 — MLFMAxwell's iterative solve on one GB300 (sm_103a).

The MLFMA octree matvec, CGS with its ILU0 preconditioner and the RCS
far-field sum run as hand-written CUDA behind the C ABI in
include/lywell_mlfma.h; :mod:`lywell_gb300.mlfma` is the host-side mirror of
the reference's Fortran interface, :mod:`lywell_gb300.meshes` makes the
synthetic PEC bodies.
"""
from .mlfma import FMM, MLFMA, RWG, MLFError, MoM, ajustar_polariz, direction, ilu0C  # noqa: F401

__all__ = ["MLFMA", "FMM", "MoM", "RWG", "MLFError", "ajustar_polariz", "direction", "ilu0C"]
