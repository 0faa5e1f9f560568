"""Driver with the reference's command-line and output cadence.

    python -m ewpt.run gamma no_bubbles nte dx dtdiv N gp2 nsnaps T beta_Y beta_W seed \\
        [--thermal] [--fp32] [--out DIR] [--nshell 40]

Mirrors run() of gpu-kernels-rk4/main_rk4.jl:5174-7081 on top of libewpt:
parameters from the 12 positional ARGS (parameters.jl:14-55), a bubble
nucleation IC (placement on the bub_diam sub-lattice, gen_phi directions,
rmag profile; main_rk4.jl:5638-5697) or a thermal IC, the J_ext/damp schedule
when thermal (main_rk4.jl:5154-5172), a snapshot every dsnaps steps with the
13-column energy table of main_rk4.jl:6790-6805 (plus total energy and the
Gauss-constraint columns), log-shell B and Higgs spectra per snapshot and the
convolve_1d B spectrum (cut N/4, spec_routines.jl:47-77) at the first and last
snapshot (main_rk4.jl:6065-6069, 7068-7072).  Outputs are .npy files (HDF5 is
not available): energies.npy, gauss.npy, spectra_B.npy, spectra_higgs.npy,
spec_unique_first.npy, spec_unique_last.npy, params.json.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import time

import numpy as np

from . import _lib, ic
from .lattice import Lattice, kc_bin_nums
from .params import Params

ENERGY_COLUMNS = ["PE", "KE", "GE", "EEW", "MEW", "EEY", "MEY", "EB", "EB2", "min_phi", "zero", "mean_phi",
                  "helicity"]


def reference_bubble_list(p: Params, seed: int | None = None) -> np.ndarray:
    """(nb, 7) rows (1-based centre, gen_phi direction) of the reference's bubble
    placement (main_rk4.jl:5638-5684) drawn with the project's seeded RNG."""
    rng = np.random.default_rng(p.base_seed if seed is None else seed)
    bd = p.bub_diam
    nx, ny, nz = p.dims
    coords = [(a, b, c) for a in range(bd, nx + 1, bd) for b in range(bd, ny + 1, bd) for c in range(bd, nz + 1, bd)]
    if p.no_bubbles > len(coords):
        raise ValueError(f"{p.no_bubbles} bubbles do not fit the {len(coords)}-point placement sub-lattice")
    pick = rng.choice(len(coords), size=p.no_bubbles, replace=False)
    hoft = rng.random((p.no_bubbles, 3))
    signs = rng.choice([-1.0, 1.0], size=p.no_bubbles)
    rows = [list(coords[pick[b]]) + ic.gen_phi(*hoft[b], signs[b]) for b in range(p.no_bubbles)]
    if p.no_bubbles == 2:  # two bubbles on the y = N/2 plane (main_rk4.jl:5664-5670)
        rows[0][:3] = [nx // 2 - 2 * bd, ny // 2, nz // 2]
        rows[1][:3] = [nx // 2 + 2 * bd, ny // 2, nz // 2]
    return np.array(rows, dtype=np.float64)


def run(p: Params, thermal_init: bool = False, out_dir: str | None = None, nshell: int = 40,
        verbose: bool = True) -> dict:
    p = dataclasses.replace(p, thermal_init=thermal_init)
    nsnap = p.nsnaps
    dsn = p.dsnaps
    cut = p.spec_cut
    nb_unique = kc_bin_nums(*cut)
    energies = np.zeros((nsnap + 1, 13))
    total = np.zeros(nsnap + 1)
    gauss = np.zeros((nsnap + 1, 6))
    specB, specH = [], []
    t0 = time.perf_counter()
    with Lattice(p) as lat:
        if thermal_init:
            lat.set_state(ic.thermal(p.dims, p.dx, T=p.T if p.T > 0 else 1.5, lam=p.lam, gw=p.gw, gy=p.gy,
                                     vev=p.vev, seed=p.base_seed))
        else:
            lat.init_bubbles(reference_bubble_list(p), "reference")
        for snap in range(nsnap + 1):
            if snap > 0:
                lat.step(dsn)
            d = lat.diagnostics(allow_nonfinite=True)
            energies[snap] = d[:13]
            total[snap] = d[13]
            gauss[snap] = d[14:20]
            specB.append(lat.spectrum("B", "log", nshell)["mean"])
            specH.append(lat.spectrum("higgs", "log", nshell)["mean"])
            if snap == 0:
                first = lat.spectrum("B", "unique", nb_unique)
            if verbose:
                print(f"--------Energies--t:{lat.iteration}--------")
                for name, v in zip(ENERGY_COLUMNS, d[:13]):
                    print(f"{name:10s} {v: .10e}")
                print(f"{'total':10s} {d[13]: .10e}   Gauss |G_W| {d[14]:.3e}  |G_Y| {d[16]:.3e}", flush=True)
        last = lat.spectrum("B", "unique", nb_unique)
        it = lat.iteration
    res = dict(energies=energies, total=total, gauss=gauss, spectra_B=np.array(specB), spectra_higgs=np.array(specH),
               spec_unique_first=np.stack([first["k"], first["mean"]], 1),
               spec_unique_last=np.stack([last["k"], last["mean"]], 1), iterations=it,
               seconds=time.perf_counter() - t0)
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
        for k, v in res.items():
            if isinstance(v, np.ndarray):
                np.save(os.path.join(out_dir, f"{k}.npy"), v)
        with open(os.path.join(out_dir, "params.json"), "w") as f:
            json.dump({k: (list(v) if isinstance(v, tuple) else v) for k, v in dataclasses.asdict(p).items()}, f,
                      indent=1)
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("args", nargs=12, help="gamma no_bubbles nte dx dtdiv N gp2 nsnaps T beta_Y beta_W seed")
    ap.add_argument("--thermal", action="store_true", help="thermal IC and the J_ext/damp schedule")
    ap.add_argument("--fp32", action="store_true", help="FP32 stencil/flux form")
    ap.add_argument("--out", default=None)
    ap.add_argument("--nshell", type=int, default=40)
    a = ap.parse_args(argv)
    p = Params.from_args(a.args, precision=_lib.FP32 if a.fp32 else _lib.FP64)
    res = run(p, thermal_init=a.thermal, out_dir=a.out, nshell=a.nshell)
    print(f"done: {res['iterations']} RK4 steps in {res['seconds']:.2f} s")


if __name__ == "__main__":
    main()
