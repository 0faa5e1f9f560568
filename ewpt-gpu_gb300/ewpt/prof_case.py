"""Small profiling case for the stage kernels (one RK4 step per form/tiling).

    python -m ewpt.prof_case [N] [--forms fp64,fp32,fp32x2]

Builds an N^3 lattice (default 80: 512,000 sites, larger than L2 in every
form) with 8 seeded tanh bubbles and runs one RK4 step in each requested
form: fp64 (k_stage_fp64), df64 (k_stage_dd, 64x2 tiles, <=168 registers), fp32 (k_stage_fp32,
64x2 tiles, <=168 registers), fp32x2 (k_stage_fp32x2, two sites per thread, 32x1 tiles),
fp32x2r2 (k_stage_fp32x2, 64x2 pair-threads, <=168 registers: the tuned 256^3 shape) and fp32tma
(k_stage_tma, TMA-staged 32x4x4-site tiles; N a multiple of 32) and fp32c
(k_stage_fp32x2 in the compensated mode, 64x2 pair-threads).  Meant to
be wrapped by ncu with -k regex:k_stage.  The form ens runs one step of a
batched ensemble of FP32-form members of 48^3, 96^3, 96^3 and 128^3 (4.0 M
sites; the members' k_stage_fp32x2 launches, 16x8 pair-threads), the member mix of the
96-member configuration at 1/29 of its size; N is ignored there.
"""
import argparse

from . import _lib, ic
from .lattice import Lattice
from .params import baseline_couplings

TILES = {"fp64": (_lib.FP64, (32, 2, 0, 0)), "df64": (_lib.DF64, (64, 2, 2, 0)), "fp32": (_lib.FP32, (64, 2, 2, 0)),
         "fp32x2": (_lib.FP32, (32, 1, 0, 1)), "fp32x2r2": (_lib.FP32, (64, 2, 2, 1)),
         "fp32tma": (_lib.FP32, (32, 4, 4, 2)), "fp32c": (_lib.FP32, (64, 2, 2, 1))}


ENSEMBLE_SIZES = [48, 96, 96, 128]


def ensemble_step():
    from .ensemble import Ensemble

    ps = [baseline_couplings(N=n, dx=0.25, dt=0.025, precision=_lib.FP32) for n in ENSEMBLE_SIZES]
    with Ensemble(ps) as ens:
        ens.set_tiling(16, 8, 1)
        for m, p in enumerate(ps):
            R, w = ic.tanh_profile_params(p.lam, p.vev)
            ens.init_bubbles(m, ic.tanh_bubble_list(p.dims, p.dx, 8, seed=m), "tanh", R, w)
        ens.step(1)
        ens.sync()


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("N", nargs="?", type=int, default=80)
    ap.add_argument("--forms", default="fp64,fp32,fp32x2")
    a = ap.parse_args(argv)
    for form in a.forms.split(","):
        if form == "ens":
            ensemble_step()
            continue
        prec, tile = TILES[form]
        p = baseline_couplings(N=a.N, dx=0.25, dt=0.025, precision=prec)
        with Lattice(p) as lat:
            R, w = ic.tanh_profile_params(p.lam, p.vev)
            lat.init_bubbles(ic.tanh_bubble_list(p.dims, p.dx, 8, seed=1), "tanh", R, w)
            lat.set_tiling(*tile)
            if form == "fp32c":
                lat.set_fp32_compensated(True)
            lat.step(1)
            lat.sync()
    print("ok")


if __name__ == "__main__":
    main()
