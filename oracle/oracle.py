"""ctypes binding of the CPU FP64 oracle (oracle/ewpt_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The product library never links
or calls it.

Parity status: pinned.  tests/test_oracle_golden.py checks this oracle
against fixtures that tests/golden/make_golden.py produced by executing the
reference's own Julia kernel source (rk4_step!, compute_*!, convolve_1d,
initializer!, J_ext, damp) on seeded lattices.

State layout: float64 array of shape (36, S), S = nx*ny*nz, site index
i + nx*(j + ny*k) (x fastest), array order as in ewpt_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "libewpt_oracle.so")
SRC = os.path.join(HERE, "ewpt_oracle.c")

NARR = 36
NDIAG = 20
DENSITY_NAMES = ["PE", "KE", "GE", "EEW", "MEW", "EEY", "MEY", "Bx", "By", "Bz",
                 "B2x", "B2y", "B2z", "Ax", "Ay", "Az", "modphi",
                 "GW1", "GW2", "GW3", "GY", "CW1", "CW2", "CW3", "CY"]


class OrParams(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("order", C.c_int32),
                ("dx", C.c_double), ("gw", C.c_double), ("gy", C.c_double), ("gp2", C.c_double),
                ("lam", C.c_double), ("vev", C.c_double), ("beta_w", C.c_double),
                ("beta_y", C.c_double), ("theta_w", C.c_double)]


def build(force: bool = False) -> str:
    """Compile the oracle with the recipe in oracle/Makefile (gcc, no FMA contraction)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        L.or_rates.argtypes = [C.POINTER(OrParams), dp, dp, C.c_double, C.c_double]
        L.or_rk4_step.argtypes = [C.POINTER(OrParams), dp, dp, C.c_double, C.c_double, C.c_double]
        L.or_densities.argtypes = [C.POINTER(OrParams), dp, dp]
        L.or_diagnostics.argtypes = [C.POINTER(OrParams), dp, dp]
        L.or_jext.argtypes = [C.c_int64, C.c_double, C.c_double, C.c_double, C.c_int]
        L.or_jext.restype = C.c_double
        L.or_damp.argtypes = [C.c_int64, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double]
        L.or_damp.restype = C.c_double
        L.or_kc_bin_nums.argtypes = [C.c_int, C.c_int, C.c_int]
        L.or_kc_bin_nums.restype = C.c_int64
        L.or_convolve_1d.argtypes = [C.POINTER(OrParams), dp, C.c_int, C.c_int, C.c_int, dp, dp, C.c_int64]
        L.or_convolve_1d.restype = C.c_int64
        L.or_shell_spectrum.argtypes = [C.POINTER(OrParams), dp, C.c_int, dp, dp, dp, dp]
        L.or_bubble_rmag.argtypes = [C.POINTER(OrParams), dp] + [C.c_double] * 8
        L.or_num_threads.restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def params(shape, dx, gw, gy, gp2, lam, vev, beta_w=0.0, beta_y=0.0, theta_w=0.0, order=6) -> OrParams:
    """order: stencil order 2, 6, 8, 10 or 12; -2 = the reference's 2nd-order
    module as written (derivatives 0 on the planes i = 2 and N-1, 1-based)."""
    nx, ny, nz = shape
    return OrParams(nx, ny, nz, int(order), dx, gw, gy, gp2, lam, vev, beta_w, beta_y, theta_w)


def rates(p: OrParams, y: np.ndarray, Jex: float = 0.0, gamma: float = 0.0) -> np.ndarray:
    y = np.ascontiguousarray(y, dtype=np.float64)
    r = np.zeros_like(y)
    rc = lib().or_rates(C.byref(p), _dp(y), _dp(r), Jex, gamma)
    if rc:
        raise ValueError(f"or_rates failed ({rc})")
    return r


def rk4_step(p: OrParams, y: np.ndarray, dt: float, Jex: float = 0.0, gamma: float = 0.0,
             nsteps: int = 1, work: np.ndarray | None = None) -> np.ndarray:
    y = np.array(y, dtype=np.float64, order="C", copy=True)
    if work is None:
        work = np.empty(3 * y.size)
    for _ in range(nsteps):
        rc = lib().or_rk4_step(C.byref(p), _dp(y), _dp(work), dt, Jex, gamma)
        if rc:
            raise ValueError(f"or_rk4_step failed ({rc})")
    return y


def densities(p: OrParams, y: np.ndarray) -> np.ndarray:
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.zeros((len(DENSITY_NAMES), y.shape[1]))
    rc = lib().or_densities(C.byref(p), _dp(y), _dp(out))
    if rc:
        raise ValueError("or_densities failed")
    return out


def diagnostics(p: OrParams, y: np.ndarray) -> np.ndarray:
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.zeros(NDIAG)
    rc = lib().or_diagnostics(C.byref(p), _dp(y), _dp(out))
    if rc:
        raise ValueError("or_diagnostics failed")
    return out


def jext(it, dt, mH, t_sat, thermal):
    return lib().or_jext(int(it), dt, mH, t_sat, int(bool(thermal)))


def damp(it, dt, mH, t_sat, thermal, gamma_inp):
    return lib().or_damp(int(it), dt, mH, t_sat, int(bool(thermal)), gamma_inp)


def convolve_1d(p: OrParams, P: np.ndarray, cut) -> np.ndarray:
    P = np.ascontiguousarray(P, dtype=np.float64)
    nb = lib().or_kc_bin_nums(*cut)
    k = np.zeros(nb)
    v = np.zeros(nb)
    got = lib().or_convolve_1d(C.byref(p), _dp(P), cut[0], cut[1], cut[2], _dp(k), _dp(v), nb)
    return np.stack([k[:got], v[:got]], axis=1)


def shell_spectrum(p: OrParams, P: np.ndarray, nshell: int = 40):
    P = np.ascontiguousarray(P, dtype=np.float64)
    s, c, m, kc = (np.zeros(nshell) for _ in range(4))
    lib().or_shell_spectrum(C.byref(p), _dp(P), nshell, _dp(s), _dp(c), _dp(m), _dp(kc))
    return dict(sum=s, count=c, mean=m, k=kc)


def bubble_rmag(p: OrParams, y: np.ndarray, centre, direction, mH):
    """Adds one reference-profile bubble to phi in place (centre is 1-based)."""
    assert y.dtype == np.float64 and y.flags.c_contiguous
    lib().or_bubble_rmag(C.byref(p), _dp(y), float(centre[0]), float(centre[1]), float(centre[2]),
                         *[float(v) for v in direction], mH)
    return y


def set_threads(n: int):
    lib().or_set_threads(int(n))


def num_threads() -> int:
    return lib().or_num_threads()
