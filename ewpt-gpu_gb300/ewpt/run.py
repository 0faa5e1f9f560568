"""Driver with the reference's command-line and output cadence.

    python -m ewpt.run gamma no_bubbles nte dx dtdiv N gp2 nsnaps T beta_Y beta_W seed \\
        [--thermal] [--fp32 | --df64] [--out DIR] [--nshell 40] [--fft-dumps]

Mirrors run() of gpu-kernels-rk4/main_rk4.jl:5174-7081 on top of libewpt:
parameters from the 12 positional ARGS (parameters.jl:14-55), a bubble
nucleation IC (placement on the bub_diam sub-lattice, gen_phi directions,
rmag profile; main_rk4.jl:5638-5697) or a thermal IC, the J_ext/damp schedule
when thermal (main_rk4.jl:5154-5172), a snapshot every dsnaps steps with the
13-column energy table of main_rk4.jl:6790-6805 (plus total energy and the
Gauss-constraint columns), log-shell B and Higgs spectra per snapshot and the
convolve_1d B spectrum (cut N/4, spec_routines.jl:47-77) at the first and last
snapshot (main_rk4.jl:6065-6069, 7068-7072).

Outputs (HDF5 is not available here, so NumPy containers with the
reference's dataset names; `python -m ewpt.h5convert DIR` writes the .h5
files where h5py exists):
- data.npz: the datasets of data.h5 (main_rk4.jl:6930-6958): Nx, gp2, dx, dt,
  nte, gamma, T, meff_sq, t_sat_jex, nsnaps, dsnaps, (bubble runs)
  no_bubbles, bubble_locations, Hoft_angles, energies (nsnaps+1, 13) and
  y_slices_snaps (nsnaps+1, 7, Nx, Nz): the y = Ny/2 plane of PE, KE, GE,
  MEW+EEW+MEY+EEY, B_x+B_y+B_z, B2_x+B2_y+B2_z and zeros, times dx^3
  (main_rk4.jl:5700-5960, 6451-6830).  Array axes are the reference's
  (Julia) axes, stored in Fortran order.
- 3d-fft-data-<it>.npz with --fft-dumps: 3D_fft_x/y/z and 3D_fft_x2/y2/z2,
  the unnormalised complex FFTs of B and B_2 over (x, y, z) at iteration 0
  and at every snapshot iteration that is a multiple of dsnaps_fft
  (main_rk4.jl:6085-6092, 6579-6868).
- energies.npy, total.npy, gauss.npy, spectra_B.npy, spectra_higgs.npy,
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
from .lattice import Lattice, julia_array, kc_bin_nums
from .params import Params

ENERGY_COLUMNS = ["PE", "KE", "GE", "EEW", "MEW", "EEY", "MEY", "EB", "EB2", "min_phi", "zero", "mean_phi",
                  "helicity"]


def reference_bubble_draw(p: Params, seed: int | None = None):
    """The reference's bubble placement (main_rk4.jl:5638-5684) drawn with the
    project's seeded RNG: 1-based centres (nb, 3), Hoft angles (nb, 3) and
    signs (nb,)."""
    rng = np.random.default_rng(p.base_seed if seed is None else seed)
    bd = p.bub_diam
    nx, ny, nz = p.dims
    coords = [(a, b, c) for a in range(bd, nx + 1, bd) for b in range(bd, ny + 1, bd) for c in range(bd, nz + 1, bd)]
    if p.no_bubbles > len(coords):
        raise ValueError(f"{p.no_bubbles} bubbles do not fit the {len(coords)}-point placement sub-lattice")
    pick = rng.choice(len(coords), size=p.no_bubbles, replace=False)
    hoft = rng.random((p.no_bubbles, 3))
    signs = rng.choice([-1.0, 1.0], size=p.no_bubbles)
    locs = np.array([coords[q] for q in pick], dtype=np.int64).reshape(-1, 3)
    if p.no_bubbles == 2:  # two bubbles on the y = N/2 plane (main_rk4.jl:5664-5670)
        locs[0] = [nx // 2 - 2 * bd, ny // 2, nz // 2]
        locs[1] = [nx // 2 + 2 * bd, ny // 2, nz // 2]
    return locs, hoft, signs


def reference_bubble_list(p: Params, seed: int | None = None) -> np.ndarray:
    """(nb, 7) rows (1-based centre, gen_phi direction) of reference_bubble_draw."""
    locs, hoft, signs = reference_bubble_draw(p, seed)
    rows = [list(locs[b]) + ic.gen_phi(*hoft[b], signs[b]) for b in range(len(locs))]
    return np.array(rows, dtype=np.float64).reshape(-1, 7)


def y_slices(lat: Lattice, p: Params) -> np.ndarray:
    """One row of the reference's slices_arr (7, Nx, Nz): the plane j = Ny/2
    (Julia's Ny÷2, 1-based) of the energy densities and the summed B / B_2
    components, each times dx^3, summed in the reference's order
    (main_rk4.jl:5700-5960)."""
    nx, ny, nz = p.dims
    vol = p.dx ** 3
    j = ny // 2 - 1

    def plane(row):
        return julia_array(row, (nx, ny, nz))[:, j, :] * vol

    d = lat.fields("density")  # PE KE GE EEW MEW EEY MEY
    b = lat.fields("B")
    b2 = lat.fields("B2")
    out = np.zeros((7, nx, nz))
    out[0] = plane(d[0])
    out[1] = plane(d[1])
    out[2] = plane(d[2])
    out[3] = ((plane(d[4]) + plane(d[3])) + plane(d[6])) + plane(d[5])  # MEW, EEW, MEY, EEY
    out[4] = (plane(b[0]) + plane(b[1])) + plane(b[2])
    out[5] = (plane(b2[0]) + plane(b2[1])) + plane(b2[2])
    return out


def b_fft_dump(lat: Lattice, p: Params) -> dict:
    """Datasets of one 3d-fft-data-<it>.h5 (main_rk4.jl:6861-6868): fft(E_t)
    of each B and B_2 component over the (x, y, z) axes."""
    dims = p.dims
    out = {}
    for field, suffix in (("B", ""), ("B2", "2")):
        f = lat.fields(field)
        for c, axis in enumerate("xyz"):
            out[f"3D_fft_{axis}{suffix}"] = np.asfortranarray(_fftn(julia_array(f[c], dims)))
    return out


def _fftn(a):
    try:
        import scipy.fft as sfft

        return sfft.fftn(a, workers=-1)
    except ImportError:
        return np.fft.fftn(a)


def run(p: Params, thermal_init: bool = False, out_dir: str | None = None, nshell: int = 40,
        verbose: bool = True, fft_dumps: bool = False) -> dict:
    p = dataclasses.replace(p, thermal_init=thermal_init)
    nsnap = p.nsnaps
    dsn = p.dsnaps
    cut = p.spec_cut
    nb_unique = kc_bin_nums(*cut)
    nx, ny, nz = p.dims
    energies = np.zeros((nsnap + 1, 13))
    total = np.zeros(nsnap + 1)
    gauss = np.zeros((nsnap + 1, 6))
    slices = np.zeros((nsnap + 1, 7, nx, nz), order="F")
    specB, specH = [], []
    dumps = []
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
    locs = hoft = None
    t0 = time.perf_counter()
    with Lattice(p) as lat:
        if thermal_init:
            lat.set_state(ic.thermal(p.dims, p.dx, T=p.T if p.T > 0 else 1.5, lam=p.lam, gw=p.gw, gy=p.gy,
                                     vev=p.vev, seed=p.base_seed))
        else:
            locs, hoft, signs = reference_bubble_draw(p)
            lat.init_bubbles(reference_bubble_list(p), "reference")
        for snap in range(nsnap + 1):
            if snap > 0:
                lat.step(dsn)
            it = lat.iteration
            d = lat.diagnostics(allow_nonfinite=True)
            energies[snap] = d[:13]
            total[snap] = d[13]
            gauss[snap] = d[14:20]
            slices[snap] = y_slices(lat, p)
            specB.append(lat.spectrum("B", "log", nshell)["mean"])
            specH.append(lat.spectrum("higgs", "log", nshell)["mean"])
            if fft_dumps and (snap == 0 or it % p.dsnaps_fft == 0):
                dumps.append(it)
                if out_dir:
                    np.savez(os.path.join(out_dir, f"3d-fft-data-{it}.npz"), **b_fft_dump(lat, p))
            if snap == 0:
                first = lat.spectrum("B", "unique", nb_unique)
            if verbose:
                print(f"--------Energies--t:{it}--------")
                for name, v in zip(ENERGY_COLUMNS, d[:13]):
                    print(f"{name:10s} {v: .10e}")
                print(f"{'total':10s} {d[13]: .10e}   Gauss |G_W| {d[14]:.3e}  |G_Y| {d[16]:.3e}", flush=True)
        last = lat.spectrum("B", "unique", nb_unique)
        it = lat.iteration
    res = dict(energies=energies, total=total, gauss=gauss, spectra_B=np.array(specB), spectra_higgs=np.array(specH),
               spec_unique_first=np.stack([first["k"], first["mean"]], 1),
               spec_unique_last=np.stack([last["k"], last["mean"]], 1), y_slices_snaps=slices,
               fft_dump_iterations=np.array(dumps, dtype=np.int64), iterations=it,
               seconds=time.perf_counter() - t0)
    if out_dir:
        for k, v in res.items():
            if isinstance(v, np.ndarray) and k not in ("y_slices_snaps", "fft_dump_iterations"):
                np.save(os.path.join(out_dir, f"{k}.npy"), v)
        data = dict(Nx=np.int64(nx), gp2=np.float64(p.gp2), dx=np.float64(p.dx), dt=np.float64(p.dt),
                    nte=np.int64(p.nte), gamma=np.float64(p.gamma_inp), T=np.float64(p.T),
                    meff_sq=np.float64(p.meff_sq), t_sat_jex=np.float64(p.t_sat), nsnaps=np.int64(nsnap),
                    dsnaps=np.int64(dsn), energies=energies, y_slices_snaps=slices)
        if not thermal_init:
            data.update(no_bubbles=np.int64(p.no_bubbles), bubble_locations=locs, Hoft_angles=hoft)
        np.savez(os.path.join(out_dir, "data.npz"), **data)
        with open(os.path.join(out_dir, "params.json"), "w") as f:
            json.dump({k: (list(v) if isinstance(v, tuple) else v) for k, v in dataclasses.asdict(p).items()}, f,
                      indent=1)
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("args", nargs=12, help="gamma no_bubbles nte dx dtdiv N gp2 nsnaps T beta_Y beta_W seed")
    ap.add_argument("--thermal", action="store_true", help="thermal IC and the J_ext/damp schedule")
    ap.add_argument("--fp32", action="store_true", help="FP32 stencil/flux form")
    ap.add_argument("--df64", action="store_true", help="double-float form (the FP64 scheme on the FP32 pipes)")
    ap.add_argument("--out", default=None)
    ap.add_argument("--nshell", type=int, default=40)
    ap.add_argument("--fft-dumps", action="store_true", help="3d-fft-data-<it>.npz B / B_2 FFT dumps")
    a = ap.parse_args(argv)
    if a.fp32 and a.df64:
        ap.error("--fp32 and --df64 exclude each other")
    p = Params.from_args(a.args, precision=_lib.FP32 if a.fp32 else _lib.DF64 if a.df64 else _lib.FP64)
    res = run(p, thermal_init=a.thermal, out_dir=a.out, nshell=a.nshell, fft_dumps=a.fft_dumps)
    print(f"done: {res['iterations']} RK4 steps in {res['seconds']:.2f} s")


if __name__ == "__main__":
    main()
