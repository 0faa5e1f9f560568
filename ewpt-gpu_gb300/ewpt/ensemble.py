"""Batched ensemble of independent lattices (FP32 form): every member a
single-lattice FP32 context, one step of all members one CUDA graph with a
concurrent branch per member (ewpt_ensemble_* in include/ewpt.h)."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .lattice import FIELDS, MODES
from .params import Params


class Ensemble:
    def __init__(self, members: list[Params]):
        self.L = _lib.load()
        self.members = list(members)
        arr = (_lib.EwptParams * len(members))(*[m.to_c() for m in members])
        h = C.c_void_p()
        _lib.check(self.L.ewpt_ensemble_create(len(members), arr, C.byref(h)))
        self.h = h

    def _chk(self, rc):
        if rc != _lib.OK:
            raise _lib.EwptError(rc, self.L.ewpt_ensemble_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.ewpt_ensemble_destroy(self.h)
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

    def __len__(self):
        return int(self.L.ewpt_ensemble_size(self.h))

    @property
    def sites(self) -> int:
        return int(self.L.ewpt_ensemble_sites(self.h))

    @property
    def stream(self) -> int:
        return int(self.L.ewpt_ensemble_stream(self.h) or 0)

    def set_state(self, m: int, y: np.ndarray):
        y = np.ascontiguousarray(y, dtype=np.float64)
        if y.shape != (36, self.members[m].sites):
            raise ValueError("state shape")
        self._chk(self.L.ewpt_ensemble_set_state(self.h, m, y.ctypes.data, 0))

    def get_state(self, m: int) -> np.ndarray:
        out = np.empty((36, self.members[m].sites))
        self._chk(self.L.ewpt_ensemble_get_state(self.h, m, out.ctypes.data, 0))
        return out

    def init_bubbles(self, m: int, bubbles: np.ndarray, profile: str = "tanh", radius: float = 0.0,
                     width: float = 0.0):
        b = np.ascontiguousarray(bubbles, dtype=np.float64).reshape(-1, 7)
        prof = _lib.BUBBLE_TANH if profile == "tanh" else _lib.BUBBLE_REFERENCE
        self._chk(self.L.ewpt_ensemble_init_bubbles(self.h, m, len(b), b.ctypes.data_as(_lib.DP), prof,
                                                    float(radius), float(width)))

    def init_thermal(self, m: int, T: float, seed: int = 0, mH: float | None = None, mW: float | None = None):
        """Device thermal IC of member m (ewpt_ensemble_init_thermal); the
        defaults of Lattice.init_thermal."""
        p = self.members[m]
        mH = math.sqrt(2.0 * p.lam) * p.vev if mH is None else mH
        mW = p.gw * p.vev / 2.0 if mW is None else mW
        self._chk(self.L.ewpt_ensemble_init_thermal(self.h, m, float(T), float(mH), float(mW),
                                                    int(seed) & (2 ** 64 - 1)))

    def init_thermal_gauss(self, m: int, T: float, seed: int = 0, gauss_iters: int = 20, mH: float | None = None,
                           mW: float | None = None):
        """Member m from the thermal IC with Gauss-projected thermal momenta
        (ewpt_ensemble_init_thermal_gauss)."""
        p = self.members[m]
        mH = math.sqrt(2.0 * p.lam) * p.vev if mH is None else mH
        mW = p.gw * p.vev / 2.0 if mW is None else mW
        self._chk(self.L.ewpt_ensemble_init_thermal_gauss(self.h, m, float(T), float(mH), float(mW),
                                                          int(seed) & (2 ** 64 - 1), int(gauss_iters)))

    def set_drive(self, m: int, Jex: float, gamma: float):
        self._chk(self.L.ewpt_ensemble_set_drive(self.h, m, float(Jex), float(gamma)))

    def set_tiling(self, bx: int, by: int, pair: int):
        self._chk(self.L.ewpt_ensemble_set_tiling(self.h, bx, by, pair))

    def set_member_tiling(self, m: int, bx: int, by: int, reg: int = 2, pair: int = 1):
        """Launch shape of member m alone (as Lattice.set_tiling, pair 0 or 1)."""
        self._chk(self.L.ewpt_ensemble_set_member_tiling(self.h, int(m), int(bx), int(by), int(reg), int(pair)))

    def step(self, n: int = 1):
        self._chk(self.L.ewpt_ensemble_step(self.h, int(n)))

    def sync(self):
        self._chk(self.L.ewpt_ensemble_sync(self.h))

    def diagnostics(self, m: int) -> np.ndarray:
        out = np.zeros(_lib.NDIAG)
        self._chk(self.L.ewpt_ensemble_diagnostics(self.h, m, out.ctypes.data_as(_lib.DP)))
        return out

    def spectrum(self, m: int, field: str = "B", mode: str = "log", nbins: int = 40) -> dict:
        k, s, c, mn = (np.zeros(nbins) for _ in range(4))
        nout = C.c_int32(0)
        self._chk(self.L.ewpt_ensemble_spectrum(self.h, m, FIELDS[field], MODES[mode], int(nbins),
                                                k.ctypes.data_as(_lib.DP), s.ctypes.data_as(_lib.DP),
                                                c.ctypes.data_as(_lib.DP), mn.ctypes.data_as(_lib.DP),
                                                C.byref(nout)))
        n = nout.value
        return dict(k=k[:n], sum=s[:n], count=c[:n], mean=mn[:n])
