"""ewpt -- host-side driver of libewpt, the GB300 implementation of the
EWPT-GPU real-time RK4 lattice evolution (Teerthal/EWPT-GPU).

Mirrors the reference's parameters/driver surface (gpu-kernels-rk4/
parameters.jl, main_rk4.jl run()); the compute runs in libewpt.so through
its C ABI (include/ewpt.h).
"""
from . import _lib, ic
from ._lib import DF64, FP32, FP64, EwptError, load
from .ensemble import Ensemble
from .lattice import DIAG_NAMES, Lattice, kc_bin_nums, rk4_rates_device
from .params import Params, baseline_couplings
from .slabs import DistributedSlab, SlabGroup

__all__ = ["Ensemble", "Lattice", "Params", "SlabGroup", "DistributedSlab", "baseline_couplings", "ic", "FP32", "FP64", "DF64", "EwptError", "load",
           "DIAG_NAMES", "kc_bin_nums", "rk4_rates_device", "_lib"]
