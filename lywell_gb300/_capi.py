"""ctypes binding of include/lywell_mlfma.h (lib/liblywell_mlfma.so).

The library is built in-tree by lywell_gb300.build.  Loading fails loudly
when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liblywell_mlfma.so")

# Every symbol the header declares, with (restype, argtypes).
vp = C.c_void_p
ip = C.POINTER(C.c_int)
SIGNATURES = {
    "mlf_rwg_build": (C.c_int, [vp, C.c_int, ip, ip, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "mlf_init": (C.c_int, [C.POINTER(vp), vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int,
                           vp, C.c_double, C.c_double, C.c_int]),
    "mlf_free": (None, [vp]),
    "mlf_last_error": (C.c_char_p, [vp]),
    "mlf_matvec": (C.c_int, [vp, vp, vp, C.c_int, C.c_int]),
    "mlf_matvec_device": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, vp]),
    "mlf_matvec_device_noalloc": (C.c_int, [vp, vp, vp, vp]),
    "mlf_near_csr": (C.c_int, [vp, C.POINTER(C.c_longlong), vp, vp, vp]),
    "mlf_ilu0": (C.c_int, [vp, ip]),
    "mlf_ilu0_factors": (C.c_int, [vp, vp, vp, vp]),
    "mlf_ilut": (C.c_int, [vp, C.c_double, C.c_double, ip]),
    "mlf_ilu_size": (C.c_int, [vp, C.POINTER(C.c_longlong)]),
    "mlf_ilu0_solve": (C.c_int, [vp, vp, vp, C.c_int]),
    "mlf_ilu0_csr": (C.c_int, [C.c_int, vp, vp, vp, vp, vp, vp, ip]),
    "mlf_set_near_values": (C.c_int, [vp, vp]),
    "mlf_set_stagnation": (C.c_int, [vp, C.c_int]),
    "mlf_set_nearinv_precision": (C.c_int, [vp, C.c_int]),
    "mlf_cgs": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, C.c_int, vp, vp, vp, C.c_int, vp]),
    "mlf_nearinv": (C.c_int, [vp, ip]),
    "mlf_nearinv_own": (C.c_int, [vp, ip]),
    "mlf_precond_apply": (C.c_int, [vp, C.c_int, vp, vp, C.c_int]),
    "mlf_solve": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, vp, vp, vp,
                            vp, ip]),
    "mlf_matvec32": (C.c_int, [vp, vp, vp, C.c_int, C.c_int]),
    "mlf_set_gmres_restart": (C.c_int, [vp, C.c_int]),
    "mlf_set_gs_passes": (C.c_int, [vp, C.c_int]),
    "mlf_set_basis_precision": (C.c_int, [vp, C.c_int]),
    "mlf_set_translation_group": (C.c_int, [vp, C.c_int, C.c_int]),
    "mlf_solve_times": (C.c_int, [vp, vp]),
    "mlf_solve_phases": (C.c_int, [vp, vp, C.c_int]),
    "mlf_set_lu_split": (C.c_int, [vp, C.c_int]),
    "mlf_get_lu_split": (C.c_int, [vp, vp, vp]),
    "mlf_precond_apply32": (C.c_int, [vp, vp, vp, C.c_int]),
    "mlf_autotune_block": (C.c_int, [vp, vp, C.c_int, vp, vp, vp, vp]),
    "mlf_set_block_engine": (C.c_int, [vp, C.c_int, C.c_int]),
    "mlf_mlp_create": (C.c_int, [vp, C.c_int, C.c_ulonglong]),
    "mlf_mlp_free": (None, [vp]),
    "mlf_mlp_last_error": (C.c_char_p, [vp]),
    "mlf_mlp_nparam": (C.c_int, []),
    "mlf_mlp_set_params": (C.c_int, [vp, vp, vp]),
    "mlf_mlp_get_params": (C.c_int, [vp, vp, vp]),
    "mlf_mlp_forward": (C.c_int, [vp, vp, C.c_longlong, vp, vp]),
    "mlf_mlp_grad": (C.c_int, [vp, vp, vp, C.c_longlong, vp, vp]),
    "mlf_lp_tokens": (C.c_int, [vp, C.c_int, vp, vp, C.c_longlong, vp, vp]),
    "mlf_lp_install": (C.c_int, [vp, vp, C.c_float, vp]),
    "mlf_mlp_train": (C.c_int, [vp, vp, vp, C.c_longlong, C.c_int, C.c_int, C.c_float, C.c_ulonglong, vp]),
    "mlf_matvec32_device": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, vp]),
    "mlf_nearinv_values": (C.c_int, [vp, vp]),
    "mlf_cgs_history": (C.c_int, [vp, C.c_int, vp, C.c_int, ip]),
    "mlf_excitation": (C.c_int, [vp, vp, vp, C.c_double, C.c_double, C.c_int, vp]),
    "mlf_rcs": (C.c_int, [vp, vp, vp, C.c_double, C.c_double, vp, vp, C.c_int, vp]),
    "mlf_info": (C.c_int, [vp, vp, C.POINTER(C.c_longlong)]),
    "mlf_monostatic": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                 C.c_int, C.c_int, vp, vp, vp]),
    "mlf_set_profiling": (C.c_int, [vp, C.c_int]),
    "mlf_stage_times": (C.c_int, [vp, vp]),
    "mlf_debug_field": (C.c_int, [vp, C.c_int, C.c_int, vp]),
}

STATUS = {0: "MLF_OK", -1: "MLF_E_ARG", -2: "MLF_E_TOO_SMALL", -3: "MLF_E_CUDA", -4: "MLF_E_NOMEM",
          -5: "MLF_E_TABLE", -6: "MLF_E_STATE", -7: "MLF_E_NOT_FINITE", -8: "MLF_E_NO_DEVICE"}
CGS_STATUS = {0: "converged", 1: "maxit", 2: "breakdown", 3: "not_finite", 4: "stagnated"}
FLAG_LEGENDRE_RECURRENCE = 1
FLAG_DENSE_MOM = 2
FLAG_FMM = 4
PRECOND = {"none": 0, "ilu0": 1, "nearinv": 2}
ENGINES = {0: "FP32 FMA", 1: "tensor cores (3xTF32 mma.sync)", 2: "warp per basis", 3: "warp per basis, per-basis receive",
           4: "tensor cores (tcgen05: FP16-split near field and aggregation, 3xTF32 receive; TMEM accumulators)"}

_lib = None


class MLFError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def load(build_if_missing: bool = False):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build as _b
            _b.build()
        else:
            raise ImportError(f"lywell_gb300 CUDA library not built: {LIB_PATH} is missing "
                              "(run `python -m lywell_gb300.build`)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
