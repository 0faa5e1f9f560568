"""ctypes binding of oracle/devphys.cu: the stage kernels' per-site
arithmetic (csrc/physics.cuh, csrc/accessors.cuh) compiled for the host.

TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the tests use it to compare the
kernels' own equations with the oracle on the CPU and to count the FP64
operations of one site-update exactly; the product library never links it.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "ewpt-gpu_gb300", "csrc")
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "libdevphys.so")
SRC = os.path.join(HERE, "devphys.cu")
DEPS = [SRC, os.path.join(CSRC, "physics.cuh"), os.path.join(CSRC, "accessors.cuh"),
        os.path.join(CSRC, "ewpt_internal.cuh"), os.path.join(ROOT, "include", "ewpt.h")]

# epilogue of the FP64 stage kernels per site-update: 2 FMAs per array in
# stages 1-3 (yn and the next stage input), 1 in stage 4
EPILOGUE_FMA = 36 * (2 + 2 + 2 + 1)


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.check_call([_nvcc(), "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17", "--expt-relaxed-constexpr",
                           "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.join(ROOT, "include"),
                           "-I", CSRC, SRC, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.dp_count.argtypes = [C.c_int, C.POINTER(C.c_longlong)]
        dp = C.POINTER(C.c_double)
        L.dp_rates.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, dp, C.c_double, C.c_double]
        _lib = L
    return _lib


def count(beta: bool = False) -> dict:
    """Operation count of one site of one stage and of one site-update."""
    c = (C.c_longlong * 8)()
    if lib().dp_count(int(bool(beta)), c):
        raise RuntimeError("dp_count: not all 36 rates delivered")
    add, mul, div, neg, inst, sflops, sinst, _ = list(c)
    stage_flops = add + mul
    return {"add_sub": add, "mul": mul, "div": div, "neg": neg, "flops_per_stage": stage_flops,
            "stencil_flops_per_stage": sflops, "physics_flops_per_stage": stage_flops - sflops,
            "fp64_inst_est_per_stage": inst, "stencil_inst_est_per_stage": sinst,
            "flops_per_site_update": 4 * stage_flops + 2 * EPILOGUE_FMA,
            "fp64_inst_est_per_site_update": 4 * inst + EPILOGUE_FMA,
            "div_per_site_update": 4 * div}


def rates(shape, coef, y: np.ndarray, Jex: float = 0.0, gamma: float = 0.0) -> np.ndarray:
    """Rates of every site from the kernels' physics evaluated on the host.
    coef: (gw, gy, gp2, lambda, vev, beta_w, beta_y, dx)."""
    nx, ny, nz = shape
    y = np.ascontiguousarray(y, dtype=np.float64)
    r = np.zeros_like(y)
    cp = np.ascontiguousarray(coef, dtype=np.float64)
    dp = C.POINTER(C.c_double)
    if lib().dp_rates(nx, ny, nz, cp.ctypes.data_as(dp), y.ctypes.data_as(dp), r.ctypes.data_as(dp), Jex, gamma):
        raise ValueError("dp_rates: lattice too small")
    return r
