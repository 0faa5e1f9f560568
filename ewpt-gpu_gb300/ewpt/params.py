"""Parameter surface of the reference driver (gpu-kernels-rk4/parameters.jl).

`Params.from_args` parses the reference's 12 positional command-line
arguments in the same order and with the same derived quantities:

    ARG1 gamma_inp  ARG2 no_bubbles  ARG3 nte  ARG4 dx  ARG5 dt divisor
    ARG6 N          ARG7 gp2         ARG8 nsnaps  ARG9 T  ARG10 beta_Y
    ARG11 beta_W    ARG12 seed multiplier (base_seed = 123456*ARG12)

(parameters.jl:14-55); derived: dt = dx/ARG5 (:23), mH = 2 sqrt(lambda) vev
(:24), gy = gw tan(asin(sqrt(0.22))) (:16-18), dsnaps = floor(nte/nsnaps)
(:43), bub_diam = floor(30*0.1 ÷ dx) (:65), spec_cut = N÷4 (:79),
t_sat = 2 (:40), meff_sq = 8119.43/174^2 (:37).
"""
from __future__ import annotations

import dataclasses
import math

from . import _lib


@dataclasses.dataclass
class Params:
    N: int = 64
    dx: float = 0.25
    dt: float = 0.025
    gw: float = 0.65
    gy: float = 0.65 * math.tan(math.asin(math.sqrt(0.22)))
    gp2: float = 0.99
    lam: float = 0.129
    vev: float = 1.0
    theta_w: float = math.asin(math.sqrt(0.22))
    beta_w: float = 0.0
    beta_y: float = 0.0
    gamma_inp: float = 0.0
    T: float = 0.0
    nte: int = 1000
    nsnaps: int = 10
    nsnaps_fft: int = 50
    no_bubbles: int = 10
    base_seed: int = 123456
    mH: float = 2.0 * math.sqrt(0.129)
    t_sat: float = 2.0
    meff_sq: float = 8119.43 / 174.0 ** 2
    thermal_init: bool = False
    precision: int = _lib.FP64
    shape: tuple | None = None  # (nx, ny, nz); defaults to (N, N, N)
    device: int = 0
    stencil_order: int = 6  # 2, 6, 8, 10 or 12 (diff_scheme.jl modules); != 6 needs FP64

    @classmethod
    def from_args(cls, args: list[str], **over) -> "Params":
        """The 12 positional ARGS of `julia main_rk4.jl` (parameters.jl:14-55)."""
        if len(args) != 12:
            raise ValueError("expected the reference's 12 positional arguments")
        gamma, nb, nte, dx, dtdiv, N, gp2, nsnaps, T, bY, bW, seed = args
        dx = float(dx)
        lam, vev = 0.129, 1.0
        p = cls(N=int(N), dx=dx, dt=dx / float(dtdiv), gp2=float(gp2), lam=lam, vev=vev,
                beta_w=float(bW), beta_y=float(bY), gamma_inp=float(gamma), T=float(T),
                nte=int(nte), nsnaps=int(nsnaps), no_bubbles=int(nb),
                base_seed=123456 * int(seed), mH=2.0 * math.sqrt(lam) * vev)
        return dataclasses.replace(p, **over)

    @property
    def dims(self) -> tuple:
        return tuple(self.shape) if self.shape else (self.N, self.N, self.N)

    @property
    def sites(self) -> int:
        nx, ny, nz = self.dims
        return nx * ny * nz

    @property
    def dsnaps(self) -> int:
        return max(1, int(math.floor(self.nte / self.nsnaps)))

    @property
    def dsnaps_fft(self) -> int:
        """Steps between 3D B-FFT dumps: floor(nte / nsnaps_fft), nsnaps_fft = 50
        (parameters.jl:46-48); at least 1."""
        return max(1, int(math.floor(self.nte / self.nsnaps_fft)))

    @property
    def bub_diam(self) -> int:
        # floor(int_prec, 30*0.1 ÷ dx): ÷ is Julia's truncating division
        return int(math.floor(math.floor((30 * 0.1) / self.dx)))

    @property
    def spec_cut(self) -> tuple:
        return tuple(n // 4 for n in self.dims)

    def to_c(self) -> _lib.EwptParams:
        nx, ny, nz = self.dims
        return _lib.EwptParams(nx, ny, nz, int(self.precision), self.dx, self.dt, self.gw, self.gy, self.gp2,
                               self.lam, self.vev, self.theta_w, self.beta_w, self.beta_y, self.gamma_inp,
                               self.mH, self.t_sat, int(bool(self.thermal_init)), int(self.device),
                               int(self.stencil_order))


def baseline_couplings(**over) -> Params:
    """Couplings of the benchmark configurations: lambda = 0.129, g = 0.65,
    g' = 0.35, vev = 1, gamma = 0, gp2 = 0.99, beta = 0, theta_w = asin(sqrt 0.22)."""
    p = Params(gy=0.35, gp2=0.99, lam=0.129, gw=0.65, vev=1.0, gamma_inp=0.0)
    return dataclasses.replace(p, **over)
