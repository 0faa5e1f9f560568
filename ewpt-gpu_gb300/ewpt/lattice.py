"""Host-side handle of one lattice context of libewpt.

This is the Python mirror of the reference driver's data path: the 36 CuArrays
of run() (gpu-kernels-rk4/main_rk4.jl:5178-5304) become one device context,
`@cuda rk4_step!` + broadcasts (:6146-6437) become `step()`, the compute_*!
kernels + host sums (:6451-6805) become `diagnostics()`, and fft + convolve_1d
(:6580-6685, spec_routines.jl:47-77) become `spectrum()`.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .params import Params

DIAG_NAMES = ["PE", "KE", "GE", "EEW", "MEW", "EEY", "MEY", "EB", "EB2", "min_phi", "zero", "mean_phi",
              "helicity", "total", "gauss_W", "gauss_W_max", "gauss_Y", "gauss_Y_max", "aux_W", "aux_Y"]

FIELDS = {"B": _lib.FIELD_B, "B2": _lib.FIELD_B2, "higgs": _lib.FIELD_HIGGS, "density": _lib.FIELD_DENSITY}
# components of fields("density"): the E_t of compute_PE! .. compute_MEY!
DENSITY_NAMES = ["PE", "KE", "GE", "EEW", "MEW", "EEY", "MEY"]
MODES = {"log": _lib.SPEC_LOG, "unique": _lib.SPEC_UNIQUE}


class Lattice:
    def __init__(self, params: Params):
        self.params = params
        self.L = _lib.load()
        self._cp = params.to_c()
        h = C.c_void_p()
        _lib.check(self.L.ewpt_create(C.byref(self._cp), C.byref(h)))
        self.h = h
        self.S = params.sites

    # ------------------------------------------------------------ lifetime
    def close(self):
        if self.h:
            self.L.ewpt_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        return _lib.check(rc, self.h)

    # ------------------------------------------------------------ state I/O
    def set_state(self, y: np.ndarray):
        """y: float64 array (36, S) on the host."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        if y.shape != (36, self.S):
            raise ValueError(f"state must have shape (36, {self.S})")
        self._chk(self.L.ewpt_set_state_packed(self.h, y.ctypes.data, 0))

    def get_state(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((36, self.S))
        self._chk(self.L.ewpt_get_state_packed(self.h, out.ctypes.data, 0))
        return out

    def set_state_device(self, ptr: int):
        """ptr: device address of 36*S contiguous doubles."""
        self._chk(self.L.ewpt_set_state_packed(self.h, C.c_void_p(ptr), 1))

    def get_state_device(self, ptr: int):
        self._chk(self.L.ewpt_get_state_packed(self.h, C.c_void_p(ptr), 1))

    # ------------------------------------------------------------ stepping
    def step(self, n: int = 1, Jex: float | None = None, gamma: float | None = None):
        if Jex is None and gamma is None:
            self._chk(self.L.ewpt_step(self.h, int(n)))
        else:
            self._chk(self.L.ewpt_step_explicit(self.h, int(n), float(Jex or 0.0), float(gamma or 0.0)))

    def step_host(self, state_in, state_out, n: int = 1):
        """Host state in, n RK4 steps, host state out (ewpt_step_host).

        state_in / state_out: C-contiguous float64 buffers of shape (36, S),
        numpy arrays or CPU torch tensors (may be the same object).  With
        page-locked buffers (``torch.empty(..., pin_memory=True)``) the copies
        of an FP64 lattice overlap the first and last steps' stencil work;
        the result is that of set_state + step(n) + get_state in any case.
        """
        ptrs = [self._host_state_ptr(state_in, "state_in"), self._host_state_ptr(state_out, "state_out")]
        if isinstance(state_out, np.ndarray) and not state_out.flags.writeable:
            raise ValueError("state_out must be writeable")
        self._chk(self.L.ewpt_step_host(self.h, C.c_void_p(ptrs[0]), C.c_void_p(ptrs[1]), int(n)))
        return state_out

    def _host_state_ptr(self, buf, name: str) -> int:
        """Address of a (36, S) C-contiguous float64 host buffer: a numpy
        array or a CPU torch tensor."""
        if isinstance(buf, np.ndarray):
            ok = buf.dtype == np.float64 and buf.flags.c_contiguous
            ptr = buf.ctypes.data
        elif hasattr(buf, "data_ptr") and hasattr(buf, "is_cuda"):
            ok = str(buf.dtype) == "torch.float64" and buf.is_contiguous() and not buf.is_cuda
            ptr = buf.data_ptr()
        else:
            ok, ptr = False, 0
        if not ok or tuple(buf.shape) != (36, self.S):
            raise ValueError(f"{name} must be a C-contiguous float64 host buffer of shape (36, {self.S})")
        return ptr

    def sync(self):
        self._chk(self.L.ewpt_sync(self.h))

    @property
    def iteration(self) -> int:
        return int(self.L.ewpt_iteration(self.h))

    @property
    def stream(self) -> int:
        return int(self.L.ewpt_stream(self.h) or 0)

    # ------------------------------------------------------------ tiling
    def set_tiling(self, bx: int, by: int, reg: int = 0, pair: int = 0):
        self._chk(self.L.ewpt_set_tiling(self.h, int(bx), int(by), int(reg), int(pair)))

    def set_wait_limit(self, polls: int):
        """Limit of the TMA-staged kernels' device waits in polls (< 0: default)."""
        self._chk(self.L.ewpt_set_wait_limit(self.h, int(polls)))

    def set_fp32_compensated(self, on: bool = True):
        """FP32 form: compensated gauge Laplacians and auxiliary gradients
        (ewpt_set_fp32_compensated); needs a tiling with two sites per thread."""
        self._chk(self.L.ewpt_set_fp32_compensated(self.h, int(bool(on))))

    def fp32_compensated(self) -> bool:
        return bool(self.L.ewpt_get_fp32_compensated(self.h))

    def tiling(self) -> tuple:
        a, b, c, d = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        self._chk(self.L.ewpt_get_tiling(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return (a.value, b.value, c.value, d.value)

    # ------------------------------------------------------------ initial conditions
    def init_bubbles(self, bubbles: np.ndarray, profile: str = "tanh", radius: float = 0.0, width: float = 0.0):
        """Device bubble IC (ewpt_init_bubbles): bubbles is (nb, 7)."""
        b = np.ascontiguousarray(bubbles, dtype=np.float64).reshape(-1, 7)
        prof = _lib.BUBBLE_TANH if profile == "tanh" else _lib.BUBBLE_REFERENCE
        self._chk(self.L.ewpt_init_bubbles(self.h, len(b), b.ctypes.data_as(_lib.DP), prof, float(radius),
                                           float(width)))

    def init_thermal(self, T: float, seed: int = 0, mH: float | None = None, mW: float | None = None):
        """Device thermal IC (ewpt_init_thermal): Bose-Einstein modes at T,
        Higgs mass mH (default sqrt(2 lambda) vev), W mass mW (default
        g vev / 2), Gamma/Sigma = divergence of W/Y, momenta zero."""
        p = self.params
        mH = math.sqrt(2.0 * p.lam) * p.vev if mH is None else mH
        mW = p.gw * p.vev / 2.0 if mW is None else mW
        self._chk(self.L.ewpt_init_thermal(self.h, float(T), float(mH), float(mW), int(seed) & (2 ** 64 - 1)))

    def init_thermal_gauss(self, T: float, seed: int = 0, gauss_iters: int = 20, mH: float | None = None,
                           mW: float | None = None):
        """ewpt_init_thermal_gauss: the thermal IC with thermal momenta
        projected onto the Gauss law (gauss_iters iterations)."""
        p = self.params
        mH = math.sqrt(2.0 * p.lam) * p.vev if mH is None else mH
        mW = p.gw * p.vev / 2.0 if mW is None else mW
        self._chk(self.L.ewpt_init_thermal_gauss(self.h, float(T), float(mH), float(mW), int(seed) & (2 ** 64 - 1),
                                                 int(gauss_iters)))

    def gauss_project(self, iters: int = 20):
        """ewpt_gauss_project: project the state's electric fields onto the Gauss law."""
        self._chk(self.L.ewpt_gauss_project(self.h, int(iters)))

    def init_thermal_deviates(self, T: float, deviates: np.ndarray, mH: float, mW: float = 0.0,
                              one_based: bool = True):
        """The reference's thermal IC from the caller's random draws
        (ewpt_init_thermal_deviates): deviates (44, S) in run()'s draw order;
        the reference itself uses mH = sqrt(meff_sq), mW = 0 and one-based
        mode indices."""
        d = np.ascontiguousarray(deviates, dtype=np.float64)
        if d.shape != (44, self.S):
            raise ValueError(f"deviates must be (44, {self.S})")
        flags = _lib.THERMAL_ONE_BASED_MODES if one_based else 0
        self._chk(self.L.ewpt_init_thermal_deviates(self.h, float(T), float(mH), float(mW),
                                                    C.c_void_p(d.ctypes.data), 0, flags))

    # ------------------------------------------------------------ observables
    def diagnostics(self, allow_nonfinite: bool = False) -> np.ndarray:
        out = np.zeros(_lib.NDIAG)
        rc = self.L.ewpt_diagnostics(self.h, out.ctypes.data_as(_lib.DP))
        if rc == _lib.ERR_NONFINITE and allow_nonfinite:
            return out
        self._chk(rc)
        return out

    def fields(self, field: str = "B") -> np.ndarray:
        """Per-site fields (ewpt_fields): (ncomp, S) float64, each row in the
        state's order; julia_array(row, dims) gives the [x, y, z] view."""
        f = FIELDS[field]
        n = int(self.L.ewpt_field_components(f))
        out = np.empty((n, self.params.sites))
        self._chk(self.L.ewpt_fields(self.h, f, out.ctypes.data_as(_lib.DP), 0))
        return out

    def spectrum(self, field: str = "B", mode: str = "log", nbins: int = 40) -> dict:
        k, s, c, m = (np.zeros(nbins) for _ in range(4))
        nout = C.c_int32(0)
        self._chk(self.L.ewpt_spectrum(self.h, FIELDS[field], MODES[mode], int(nbins),
                                       k.ctypes.data_as(_lib.DP), s.ctypes.data_as(_lib.DP),
                                       c.ctypes.data_as(_lib.DP), m.ctypes.data_as(_lib.DP), C.byref(nout)))
        n = nout.value
        return dict(k=k[:n], sum=s[:n], count=c[:n], mean=m[:n])


def rk4_rates_device(params: Params, in_ptrs, out_ptrs, Jex: float = 0.0, gamma: float = 0.0, stream: int = 0):
    """One rk4_step! launch on device arrays (36 input and 36 output addresses)."""
    L = _lib.load()
    cp = params.to_c()
    ia = (C.c_void_p * 36)(*[C.c_void_p(int(p)) for p in in_ptrs])
    oa = (C.c_void_p * 36)(*[C.c_void_p(int(p)) for p in out_ptrs])
    _lib.check(L.ewpt_rk4_rates(C.byref(cp), ia, oa, float(Jex), float(gamma), C.c_void_p(stream)))


def kc_bin_nums(cx: int, cy: int, cz: int) -> int:
    return int(_lib.load().ewpt_kc_bin_nums(cx, cy, cz))


def julia_array(row: np.ndarray, dims) -> np.ndarray:
    """View of one [S] state-order array as the reference's Array{T,3}:
    a[i, j, k] with i (x) fastest in memory (Fortran order)."""
    return np.asarray(row).reshape(tuple(dims), order="F")
