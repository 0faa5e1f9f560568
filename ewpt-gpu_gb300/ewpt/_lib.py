"""ctypes binding of libewpt.so (include/ewpt.h).

The library is built in-tree by ewpt-gpu_gb300/build_lib.py (nvcc, sm_103a).
Loading fails loudly when it has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(ROOT, "build", "libewpt.so")
HEADER = os.path.join(os.path.dirname(ROOT), "include", "ewpt.h")

NARR = 36
NDIAG = 20

OK, ERR_ARG, ERR_CUDA, ERR_CUFFT, ERR_OOM, ERR_NONFINITE, ERR_TIMEOUT, ERR_STATE = range(8)
FP64, FP32, DF64 = 0, 1, 2
FIELD_B, FIELD_B2, FIELD_HIGGS, FIELD_DENSITY = 0, 1, 2, 3
BUBBLE_REFERENCE, BUBBLE_TANH = 0, 1
SPEC_LOG, SPEC_UNIQUE = 0, 1
THERMAL_ONE_BASED_MODES = 1


class EwptParams(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("precision", C.c_int32),
                ("dx", C.c_double), ("dt", C.c_double),
                ("gw", C.c_double), ("gy", C.c_double), ("gp2", C.c_double),
                ("lam", C.c_double), ("vev", C.c_double), ("theta_w", C.c_double),
                ("beta_w", C.c_double), ("beta_y", C.c_double), ("gamma_inp", C.c_double),
                ("mH", C.c_double), ("t_sat", C.c_double),
                ("thermal_init", C.c_int32), ("device", C.c_int32), ("stencil_order", C.c_int32)]


class EwptError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None
DP = C.POINTER(C.c_double)
DPA = DP * NARR


def _sig(L):
    P = C.POINTER(EwptParams)
    V = C.c_void_p
    L.ewpt_params_default.argtypes = [P, C.c_int32]
    L.ewpt_create.argtypes = [P, C.POINTER(V)]
    L.ewpt_destroy.argtypes = [V]
    L.ewpt_last_error.argtypes = [V]
    L.ewpt_last_error.restype = C.c_char_p
    L.ewpt_set_state.argtypes = [V, DPA, C.c_int32]
    L.ewpt_get_state.argtypes = [V, DPA, C.c_int32]
    L.ewpt_set_state_packed.argtypes = [V, C.c_void_p, C.c_int32]
    L.ewpt_get_state_packed.argtypes = [V, C.c_void_p, C.c_int32]
    L.ewpt_step.argtypes = [V, C.c_int32]
    L.ewpt_step_explicit.argtypes = [V, C.c_int32, C.c_double, C.c_double]
    L.ewpt_step_host.argtypes = [V, C.c_void_p, C.c_void_p, C.c_int32]
    L.ewpt_iteration.argtypes = [V]
    L.ewpt_iteration.restype = C.c_int64
    L.ewpt_sync.argtypes = [V]
    L.ewpt_stream.argtypes = [V]
    L.ewpt_stream.restype = C.c_void_p
    L.ewpt_rk4_rates.argtypes = [P, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p]
    L.ewpt_diagnostics.argtypes = [V, DP]
    L.ewpt_spectrum.argtypes = [V, C.c_int32, C.c_int32, C.c_int32, DP, DP, DP, DP, C.POINTER(C.c_int32)]
    L.ewpt_init_thermal.argtypes = [V, C.c_double, C.c_double, C.c_double, C.c_uint64]
    L.ewpt_init_thermal_gauss.argtypes = [V, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_int32]
    L.ewpt_gauss_project.argtypes = [V, C.c_int32]
    L.ewpt_ensemble_init_thermal_gauss.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double,
                                                   C.c_uint64, C.c_int32]
    L.ewpt_init_thermal_deviates.argtypes = [V, C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_int32,
                                             C.c_int32]
    L.ewpt_field_components.argtypes = [C.c_int32]
    L.ewpt_field_components.restype = C.c_int32
    L.ewpt_fields.argtypes = [V, C.c_int32, DP, C.c_int32]
    L.ewpt_kc_bin_nums.argtypes = [C.c_int32, C.c_int32, C.c_int32]
    L.ewpt_kc_bin_nums.restype = C.c_int64
    L.ewpt_diagnostics_noalloc.argtypes = [P, C.c_void_p, DP, C.c_void_p]
    L.ewpt_fp64_peak.argtypes = [C.c_int32, DP, DP]
    E = C.c_void_p
    L.ewpt_ensemble_create.argtypes = [C.c_int32, C.POINTER(EwptParams), C.POINTER(E)]
    L.ewpt_ensemble_destroy.argtypes = [E]
    L.ewpt_ensemble_last_error.argtypes = [E]
    L.ewpt_ensemble_last_error.restype = C.c_char_p
    L.ewpt_ensemble_size.argtypes = [E]
    L.ewpt_ensemble_size.restype = C.c_int32
    L.ewpt_ensemble_sites.argtypes = [E]
    L.ewpt_ensemble_sites.restype = C.c_int64
    L.ewpt_ensemble_set_state.argtypes = [E, C.c_int32, C.c_void_p, C.c_int32]
    L.ewpt_ensemble_get_state.argtypes = [E, C.c_int32, C.c_void_p, C.c_int32]
    L.ewpt_ensemble_set_drive.argtypes = [E, C.c_int32, C.c_double, C.c_double]
    L.ewpt_ensemble_init_thermal.argtypes = [E, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_uint64]
    L.ewpt_ensemble_set_tiling.argtypes = [E, C.c_int32, C.c_int32, C.c_int32]
    L.ewpt_ensemble_set_member_tiling.argtypes = [E, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.ewpt_ensemble_step.argtypes = [E, C.c_int32]
    L.ewpt_ensemble_sync.argtypes = [E]
    L.ewpt_ensemble_stream.argtypes = [E]
    L.ewpt_ensemble_stream.restype = C.c_void_p
    L.ewpt_ensemble_diagnostics.argtypes = [E, C.c_int32, DP]
    L.ewpt_ensemble_spectrum.argtypes = [E, C.c_int32, C.c_int32, C.c_int32, C.c_int32, DP, DP, DP, DP,
                                         C.POINTER(C.c_int32)]
    L.ewpt_init_bubbles.argtypes = [V, C.c_int32, DP, C.c_int32, C.c_double, C.c_double]
    L.ewpt_ensemble_init_bubbles.argtypes = [E, C.c_int32, C.c_int32, DP, C.c_int32, C.c_double, C.c_double]
    FP = C.POINTER(C.c_float)
    L.ewpt_mlp_create.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.POINTER(V)]
    L.ewpt_mlp_destroy.argtypes = [V]
    L.ewpt_mlp_last_error.argtypes = [V]
    L.ewpt_mlp_last_error.restype = C.c_char_p
    L.ewpt_mlp_num_params.argtypes = [V]
    L.ewpt_mlp_num_params.restype = C.c_int64
    L.ewpt_mlp_set_params.argtypes = [V, FP]
    L.ewpt_mlp_get_params.argtypes = [V, FP]
    L.ewpt_mlp_forward.argtypes = [V, FP, C.c_int32, FP]
    L.ewpt_mlp_gradients.argtypes = [V, FP, FP, C.c_int32, FP, FP]
    L.ewpt_mlp_train_step.argtypes = [V, FP, FP, C.c_int32, C.c_float, C.c_float, FP]
    L.ewpt_set_tiling.argtypes = [V, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    I32P = C.POINTER(C.c_int32)
    L.ewpt_get_tiling.argtypes = [V, I32P, I32P, I32P, I32P]
    L.ewpt_set_fp32_compensated.argtypes = [V, C.c_int32]
    L.ewpt_get_fp32_compensated.argtypes = [V]
    L.ewpt_get_fp32_compensated.restype = C.c_int32
    L.ewpt_set_wait_limit.argtypes = [V, C.c_int64]
    I32A = C.POINTER(C.c_int32)
    L.ewpt_slabs_create.argtypes = [P, C.c_int32, I32A, I32A, C.POINTER(V)]
    L.ewpt_slabs_destroy.argtypes = [V]
    L.ewpt_slabs_last_error.argtypes = [V]
    L.ewpt_slabs_last_error.restype = C.c_char_p
    L.ewpt_slabs_count.argtypes = [V]
    L.ewpt_slabs_count.restype = C.c_int32
    L.ewpt_slabs_set_state.argtypes = [V, C.c_void_p, C.c_int32]
    L.ewpt_slabs_get_state.argtypes = [V, C.c_void_p, C.c_int32]
    L.ewpt_slabs_set_tiling.argtypes = [V, C.c_int32, C.c_int32, C.c_int32]
    L.ewpt_slabs_step.argtypes = [V, C.c_int32]
    L.ewpt_slabs_step_explicit.argtypes = [V, C.c_int32, C.c_double, C.c_double]
    L.ewpt_slabs_sync.argtypes = [V]
    L.ewpt_slabs_stream.argtypes = [V, C.c_int32]
    L.ewpt_slabs_stream.restype = C.c_void_p
    L.ewpt_create_slab.argtypes = [P, C.c_int32, C.c_int32, C.POINTER(V)]
    L.ewpt_slab_pack.argtypes = [V, C.c_int32, C.c_void_p, C.c_void_p]
    L.ewpt_slab_unpack.argtypes = [V, C.c_int32, C.c_void_p, C.c_void_p]
    L.ewpt_slab_stage.argtypes = [V, C.c_int32, C.c_double, C.c_double]
    L.ewpt_mlp_set_wait_limit.argtypes = [V, C.c_int64]


def load():
    """The loaded libewpt (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libewpt.so not built ({LIB_PATH}); run ewpt-gpu_gb300/build_lib.py "
                               "(or __graft_entry__.build()) first")
        L = C.CDLL(LIB_PATH)
        _sig(L)
        _lib = L
    return _lib


def fp64_peak(device: int = 0) -> float:
    """Measured FP64 FLOP/s of the device (ewpt_fp64_peak)."""
    f, t = C.c_double(), C.c_double()
    check(load().ewpt_fp64_peak(int(device), C.byref(f), C.byref(t)))
    return f.value


def declared_symbols() -> list[str]:
    """Names of the functions declared in include/ewpt.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ewpt_\w+)\s*\(", txt)))


def check(rc: int, ctx=None):
    if rc != OK:
        msg = load().ewpt_last_error(ctx).decode()
        raise EwptError(rc, msg)
    return rc
