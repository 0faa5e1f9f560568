"""Precision report: the FP32 and DF64 forms against the FP64 form.

    python -m ewpt.precision_report [--N 256] [--steps 500] [--every 50] [--T 1.5]
        [--forms fp64,fp32,df64] [--gauss-iters 20] [--out FILE]

Evolves one seeded thermal initial condition (ewpt.ic.thermal: Bose-Einstein
modes at temperature T, momenta projected onto the Gauss constraint,
dx = 0.25, dt = dx/10, the benchmark couplings) in the FP64 form, the FP32
form (FP32 stencils and fluxes, compensated hi/lo state, autotuned launch
shape) and the DF64 form, from identical inputs.  The FP64 form is the
reference here: it matches the CPU oracle to 1e-11 per field over 100 steps
(tests), and the oracle itself cannot evolve these lattices in useful time.

`--device-ic` starts every form from the device thermal IC instead
(ewpt_init_thermal with the seed: the reference's construction, momenta
zero, generated in milliseconds at any size).  The form fp32c is the FP32
form in its compensated mode (ewpt_set_fp32_compensated).  `--device-gauss` starts
every form from the device IC of the precision configuration
(ewpt_init_thermal_gauss: thermal fields and momenta, the momenta projected
onto the Gauss law on the device with `--gauss-iters` iterations).
`--gauss-iters` sets the iterations of the Gauss projection (host IC:
fixed-point iterations, each removing about half of the remaining
constraint residual, 20 leave ~1e-7 of the charge density).  `--forms`
picks the forms; fp64 always runs, as the reference.

`--control EPS` adds the control run "fp64_perturbed": the FP64 form from
the same initial state with every value multiplied by (1 + EPS xi), xi
standard normal (seeded), reported against FP64 like the other forms.  It
measures how far the dynamics alone carries a perturbation of the size of
FP32 rounding (EPS ~ 1e-7): a bar on the FP32 form tighter than this
control's difference cannot be met by any arithmetic.

Reported per form: the total energy every `every` steps and its drift
|E(t) - E(0)| / |E(0)|, the Gauss-constraint violation ||G_W|| and ||G_Y||
(diagnostic columns 14 and 16) and, against FP64, the largest relative field
difference (per array, over its largest magnitude), the energy-history
difference, and the B-spectrum (40 log shells) relative difference at the
end, over the shells holding more than 1e-12 of the peak.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import _lib, autotune, ic
from .lattice import Lattice
from .params import baseline_couplings


def evolve(p, y0, steps, every, tune=True, perturb=0.0, perturb_seed=11, comp=False):
    """y0: the (36, S) initial state, or ("device", T, seed) for the device
    thermal IC (identical in every form up to the form's storage).
    perturb: relative size of the seeded perturbation of the initial state."""
    hist, t0 = [], time.perf_counter()
    # the sweep runs on its own scratch lattice: pick the shape before this one exists
    tile = autotune.best_tiling(p) if tune else None
    with Lattice(p) as lat:
        if isinstance(y0, tuple) and y0[0] == "device-gauss":
            lat.init_thermal_gauss(y0[1], seed=y0[2], gauss_iters=y0[3])
        elif isinstance(y0, tuple):
            lat.init_thermal(y0[1], seed=y0[2])
        else:
            lat.set_state(y0)
        if perturb:
            y = lat.get_state()
            rng = np.random.default_rng(perturb_seed)
            for q in range(y.shape[0]):
                y[q] *= 1.0 + perturb * rng.standard_normal(y.shape[1])
            lat.set_state(y)
            del y
        if tile:
            lat.set_tiling(*tile)
        if comp:  # the compensated mode runs the two-sites-per-thread kernel
            if not tile or tile[3] != 1:
                lat.set_tiling(64, 2, 2, 1)
            lat.set_fp32_compensated(True)
        d = lat.diagnostics(allow_nonfinite=True)
        hist.append([0, d[13], d[14], d[16]])
        done = 0
        while done < steps:
            n = min(every, steps - done)
            lat.step(n)
            done += n
            d = lat.diagnostics(allow_nonfinite=True)
            hist.append([done, d[13], d[14], d[16]])
        y = lat.get_state()
        spec = lat.spectrum("B", "log", 40)["mean"]
    return dict(hist=np.array(hist), y=y, spec=spec, seconds=time.perf_counter() - t0,
                tile=list(tile) if tile else None)


def rel_field_err(a, b):
    """max over arrays of max|a - b| / max|b| (one array at a time)."""
    return max(float(np.abs(a[q] - b[q]).max() / max(np.abs(b[q]).max(), 1e-300)) for q in range(a.shape[0]))


FORMS = {"fp64": _lib.FP64, "fp32": _lib.FP32, "fp32c": _lib.FP32, "df64": _lib.DF64}


def report(N=256, steps=500, every=50, T=1.5, seed=7, forms=("fp64", "fp32", "df64"), gauss_iters=20,
           device_ic=False, control=0.0, device_gauss=False):
    shape = (N, N, N)
    t0 = time.perf_counter()
    if device_gauss:
        y0 = ("device-gauss", T, seed, gauss_iters)
    elif device_ic:
        y0 = ("device", T, seed)
    else:
        y0 = ic.thermal(shape, 0.25, T=T, seed=seed, gauss_iters=gauss_iters)
    t_ic = time.perf_counter() - t0
    runs = {}
    names = ["fp64"] + [f for f in forms if f != "fp64"] + (["fp64_perturbed"] if control else [])
    for name in names:
        prec = FORMS["fp64" if name == "fp64_perturbed" else name]
        p = baseline_couplings(N=N, dx=0.25, dt=0.025, precision=prec)
        r = evolve(p, y0, steps, every, perturb=control if name == "fp64_perturbed" else 0.0, comp=name == "fp32c")
        if name != "fp64":  # keep one end state besides the reference's (16 GB each at 384^3)
            r["field_err"] = rel_field_err(r.pop("y"), runs["fp64"]["y"])
        runs[name] = r
    ref = runs["fp64"]
    E0 = ref["hist"][0, 1]
    smask = ref["spec"] > 1e-12 * ref["spec"].max()
    out = dict(lattice=list(shape), steps=steps, every=every, T=T, seed=seed, dt=0.025, dx=0.25,
               ic=(f"device (thermal momenta, Gauss projection on the device, {gauss_iters} iterations)"
                   if device_gauss else "device (momenta zero)" if device_ic
                   else f"host (Gauss projection, {gauss_iters} iterations)"),
               ic_seconds=t_ic, control_perturbation=control, forms={})
    for name, r in runs.items():
        h = r["hist"]
        f = dict(seconds=r["seconds"], tile=r["tile"],
                 energy_drift=float(np.abs(h[:, 1] - h[0, 1]).max() / abs(h[0, 1])),
                 gauss_w_final=float(h[-1, 2]), gauss_y_final=float(h[-1, 3]),
                 gauss_w_max=float(h[:, 2].max()), gauss_y_max=float(h[:, 3].max()),
                 energy_history=h[:, 1].tolist())
        if name != "fp64":
            f["field_rel_err_vs_fp64"] = r["field_err"]
            f["energy_hist_rel_diff_vs_fp64"] = float(np.abs(h[:, 1] - ref["hist"][:, 1]).max() / abs(E0))
            f["b_spectrum_rel_err_vs_fp64"] = float(
                (np.abs(r["spec"] - ref["spec"])[smask] / ref["spec"][smask]).max())
        out["forms"][name] = f
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--T", type=float, default=1.5)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--forms", default="fp64,fp32,df64")
    ap.add_argument("--gauss-iters", type=int, default=20)
    ap.add_argument("--device-ic", action="store_true",
                    help="the device thermal IC (ewpt_init_thermal: the reference's construction, momenta zero)")
    ap.add_argument("--device-gauss", action="store_true",
                    help="the device IC with thermal momenta projected onto the Gauss law (ewpt_init_thermal_gauss)")
    ap.add_argument("--control", type=float, default=0.0,
                    help="relative size of the perturbed-IC FP64 control run (0: none)")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    forms = [f for f in a.forms.split(",") if f]
    bad = [f for f in forms if f not in FORMS]
    if bad:
        ap.error(f"unknown forms {bad}; choose from {sorted(FORMS)}")
    r = report(a.N, a.steps, a.every, a.T, a.seed, forms, a.gauss_iters, a.device_ic, a.control, a.device_gauss)
    s = json.dumps(r, indent=1)
    print(s)
    if a.out:
        with open(a.out, "w") as f:
            f.write(s)


if __name__ == "__main__":
    main()
