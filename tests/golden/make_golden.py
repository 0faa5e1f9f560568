"""Generate golden fixtures from the reference's own Julia source text.

Run in a container where the reference checkout exists:

    python tests/golden/make_golden.py <reference_root>

The reference (Teerthal/EWPT-GPU) is Julia + CUDA.jl and Julia is not
available, so this script mechanically translates the device-kernel bodies it
needs (julia_subset.py) and evaluates them site by site in IEEE double
precision on seeded inputs:

  rk4_step!                      gpu-kernels-rk4/main_rk4.jl:52-661
  dfdx..d2fdz2 (6th order)       gpu-kernels-rk4/diff_scheme.jl:157-311
  the 2nd/8th/10th/12th-order modules   gpu-kernels-rk4/diff_scheme.jl:370-1438
  D_2phi_a..D_4phi_a             gpu-kernels-rk4/cov_derivs_temporal.jl:23-130
  W_a_xy.., Y_2_y..              gpu-kernels-rk4/field_strengths.jl:34-311
  compute_PE!..compute_Az!       gpu-kernels-rk4/main_rk4.jl:1334-4250
  initializer!                   gpu-kernels-rk4/main_rk4.jl:4930-4946
  J_ext, damp                    gpu-kernels-rk4/main_rk4.jl:5154-5172
  K_c_mag, Kc_bin_nums, convolve_1d   gpu-kernels-rk4/spec_routines.jl:6-77
  thermal_initializer_phi!, thermal_initializer_gauge!
                                 gpu-kernels-rk4/main_rk4.jl:5029-5152

The RK4 combination of the driver loop (main_rk4.jl:6182-6435) lives inside
`run()` and is restated here as its four broadcast lines (mul, then add).
The fixtures are committed; the tests never read the reference at run time.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import julia_subset as js  # noqa: E402

NAMES36 = (["phi_1", "phi_2", "phi_3", "phi_4"]
           + [f"W_{a}_{i}" for a in (1, 2, 3) for i in (2, 3, 4)]
           + ["Y_2", "Y_3", "Y_4", "Gam_1", "Gam_2", "Gam_3", "Sig"]
           + [f"dphi_{a}_dt" for a in (1, 2, 3, 4)]
           + [f"dW_{a}_{i}_dt" for a in (1, 2, 3) for i in (2, 3, 4)]
           + ["dY_2_dt", "dY_3_dt", "dY_4_dt"])
OUT36 = ["k_" + n for n in NAMES36[:20]] + ["kt_" + n for n in NAMES36[:16]]

DENSITY_KERNELS = [
    "compute_PE!", "compute_KE!", "compute_GE!", "compute_EEW!", "compute_MEW!",
    "compute_EEY!", "compute_MEY!", "compute_Bx!", "compute_By!", "compute_Bz!",
    "compute_B_2_x!", "compute_B_2_y!", "compute_B_2_z!",
    "compute_Ax!", "compute_Ay!", "compute_Az!",
]


def load(ref: str) -> dict:
    base = os.path.join(ref, "gpu-kernels-rk4")
    ns = dict(js.RUNTIME)
    # module `differentiations` (6th order) is diff_scheme.jl:1-365
    js.load_functions(os.path.join(base, "diff_scheme.jl"),
                      ["dfdx", "dfdy", "dfdz", "d2fdx2", "d2fdy2", "d2fdz2"], ns, (1, 365))
    js.load_functions(os.path.join(base, "cov_derivs_temporal.jl"),
                      [f"D_{i}ϕ_{a}" for i in (2, 3, 4) for a in (1, 2, 3, 4)], ns)
    js.load_functions(os.path.join(base, "field_strengths.jl"),
                      [f"W_{a}_{p}" for a in (1, 2, 3) for p in ("xy", "xz", "yz")]
                      + ["Y_2_y", "Y_2_z", "Y_3_z"], ns)
    js.load_functions(os.path.join(base, "main_rk4.jl"),
                      ["rk4_step!", "initializer!", "J_ext", "damp"] + DENSITY_KERNELS, ns)
    # the thermal kernels divide by exp(w/T) - 1 = 0 at the w = 0 mode before
    # their branch discards it: IEEE division (inf, as in Julia), not Python's
    nth = dict(js.RUNTIME, exp=lambda x: np.float64(math.exp(x)))
    js.load_functions(os.path.join(base, "main_rk4.jl"), ["thermal_initializer_ϕ!", "thermal_initializer_gauge!"],
                      nth)
    ns["thermal_initializer_phi_b"] = nth["thermal_initializer_phi_b"]
    ns["thermal_initializer_gauge_b"] = nth["thermal_initializer_gauge_b"]
    js.load_functions(os.path.join(base, "spec_routines.jl"),
                      ["K_c_mag", "Kc_bin_nums", "convolve_1d"], ns)
    ns["_sig"] = {n: js.signature(os.path.join(base, "main_rk4.jl"), n)
                  for n in ["rk4_step!"] + DENSITY_KERNELS}
    return ns


def as_jarr(flat: np.ndarray, shape) -> js.JArr:
    return js.JArr(flat.reshape(shape, order="F"))


def call_kernel(ns, name, arrays: dict, scalars: dict, shape, out: dict):
    fn = ns[name.replace("!", "_b")]
    sig = ns["_sig"][name]
    args = []
    for a in sig:
        if a in arrays:
            args.append(arrays[a])
        elif a in scalars:
            args.append(scalars[a])
        elif a in out:
            args.append(out[a])
        else:
            raise KeyError(f"{name}: unbound argument {a}")
    nx, ny, nz = shape
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                fn(*args, i, j, k)


def rates(ns, y: np.ndarray, shape, sc: dict, Jex: float, gam: float) -> np.ndarray:
    S = int(np.prod(shape))
    arr = {n: as_jarr(y[q], shape) for q, n in enumerate(NAMES36)}
    r = np.zeros((36, S))
    out = {n: as_jarr(r[q], shape) for q, n in enumerate(OUT36)}
    scal = dict(sc, Jex=Jex, gam=gam)
    call_kernel(ns, "rk4_step!", arr, scal, shape, out)
    return r


def rk4_step(ns, y, shape, sc, dt, Jex, gam):
    """main_rk4.jl:6155-6435 (broadcasts: X_n = k.*(dt/6.) + X, ...)."""
    k = rates(ns, y, shape, sc, Jex, gam)
    yn = k * (dt / 6.) + y
    k = rates(ns, y + k * (dt / 2.), shape, sc, Jex, gam)
    yn = k * (dt / 3.) + yn
    k = rates(ns, y + k * (dt / 2.), shape, sc, Jex, gam)
    yn = k * (dt / 3.) + yn
    k = rates(ns, y + k * dt, shape, sc, Jex, gam)
    return k * (dt / 6.) + yn


def densities(ns, y, shape, sc) -> np.ndarray:
    S = int(np.prod(shape))
    arr = {n: as_jarr(y[q], shape) for q, n in enumerate(NAMES36)}
    res = np.zeros((len(DENSITY_KERNELS), S))
    for q, name in enumerate(DENSITY_KERNELS):
        sig = ns["_sig"][name]
        outs = [a for a in sig if a not in arr and a not in sc]
        assert len(outs) == 1, (name, outs)
        call_kernel(ns, name, arr, sc, shape, {outs[0]: as_jarr(res[q], shape)})
    return res


def snapshot_row(den: np.ndarray, y: np.ndarray, dx: float) -> np.ndarray:
    """Host reductions of main_rk4.jl:6451-6805 (columns 1-13 of
    total_energies) plus the total-energy sum of :6921."""
    vol = dx ** 3
    row = np.zeros(14)
    for q in range(7):
        row[q] = np.sum(den[q]) * vol
    row[7] = (0.5 * (np.sum(den[7] ** 2) + np.sum(den[8] ** 2) + np.sum(den[9] ** 2))) * vol
    row[8] = (0.5 * (np.sum(den[10] ** 2) + np.sum(den[11] ** 2) + np.sum(den[12] ** 2))) * vol
    mod = np.sqrt(y[0] ** 2 + y[1] ** 2 + y[2] ** 2 + y[3] ** 2)
    row[9] = mod.min()
    row[10] = 0.0
    row[11] = mod.sum() / mod.size
    row[12] = np.sum(den[10] * den[13] + den[11] * den[14] + den[12] * den[15]) * vol
    row[13] = row[:7].sum()
    return row


def random_state(rng, shape, phi_offset=0.6):
    S = int(np.prod(shape))
    y = rng.normal(0.0, 0.35, size=(36, S))
    y[0] += phi_offset  # keep |Phi| away from 0
    return y


def case(ns, name, shape, params, dt, Jex, gam, seed):
    rng = np.random.default_rng(seed)
    y0 = random_state(rng, shape)
    sc = dict(gw=params["gw"], gy=params["gy"], gp2=params["gp2"], beta_W=params["beta_w"],
              beta_Y=params["beta_y"], vev=params["vev"], lambda_=params["lambda"], dx=params["dx"],
              theta_w=params["theta_w"])
    r = rates(ns, y0, shape, sc, Jex, gam)
    y1 = rk4_step(ns, y0, shape, sc, dt, Jex, gam)
    den = densities(ns, y0, shape, sc)
    row = snapshot_row(den, y0, params["dx"])
    # spectrum of the B field of y0: P = |fft Bx|^2+|fft By|^2+|fft Bz|^2
    nx, ny, nz = shape
    P = np.zeros(int(np.prod(shape)))
    for q in (7, 8, 9):
        f = np.fft.fftn(den[q].reshape(shape, order="F"))
        P += (np.conj(f) * f).real.ravel(order="F")
    cut = (nx // 4, ny // 4, nz // 4)
    spec = ns["convolve_1d"](as_jarr(P.copy(), shape), nx, ny, nz, *cut).d
    out = dict(shape=np.array(shape), y0=y0, rates=r, y1=y1, dens=den, row=row,
               P=P, spec=spec, cut=np.array(cut), dt=dt, Jex=Jex, gam=gam,
               **{f"p_{k}": v for k, v in params.items()})
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
    print(name, "rates", np.abs(r).max(), "row", row)


def spectrum_case(ns, seed=7):
    rng = np.random.default_rng(seed)
    shape = (16, 16, 12)
    P = rng.random(int(np.prod(shape)))
    cut = (4, 4, 3)
    spec = ns["convolve_1d"](as_jarr(P.copy(), shape), *shape, *cut).d
    nb = ns["Kc_bin_nums"](*cut)
    np.savez_compressed(os.path.join(HERE, "ref_spectrum.npz"), shape=np.array(shape), P=P,
                        cut=np.array(cut), spec=spec, nbins=nb)
    print("spectrum bins", nb)


# modules differentiations_{8th,10th,12th,2nd}_order of diff_scheme.jl
ORDER_MODULES = {8: (370, 626), 10: (627, 932), 12: (933, 1365), 2: (1366, 1438)}


def orders_case(ref, ns):
    """rk4_step! rates with each alternative stencil module swapped in (the
    driver selects one by `using`, main_rk4.jl:33-35), on a 14^3 lattice so
    that the 12th-order branches (diff_scheme.jl:939-1403) stay distinct;
    plus the snapshot densities with the 8th-order module."""
    base = os.path.join(ref, "gpu-kernels-rk4")
    shape = (14, 14, 14)
    rng = np.random.default_rng(4321)
    y0 = random_state(rng, shape)
    tw = math.asin(math.sqrt(0.22))
    params = dict(gw=0.65, gy=0.35, gp2=0.99, vev=1.0, dx=0.3, beta_w=0.3, beta_y=0.2, theta_w=tw)
    params["lambda"] = 0.129
    sc = dict(gw=params["gw"], gy=params["gy"], gp2=params["gp2"], beta_W=params["beta_w"],
              beta_Y=params["beta_y"], vev=params["vev"], lambda_=params["lambda"], dx=params["dx"],
              theta_w=params["theta_w"])
    out = dict(shape=np.array(shape), y0=y0, Jex=0.07, gam=0.05, **{f"p_{k}": v for k, v in params.items()})
    diff_src = os.path.join(base, "diff_scheme.jl")
    # diff_scheme.jl:879: the 10th-order d2fdz2 tests `i` instead of `k` in its
    # interior branch, so on the z-boundary planes it indexes outside the
    # array; the fixture uses the intended condition (one token changed).
    with open(diff_src, encoding="utf-8") as f:
        text = f.read().split("\n")
    bad = "    if (i>5 && i<(size(A,3)-4))"
    assert text[878] == bad, text[878]
    text[878] = "    if (k>5 && k<(size(A,3)-4))"
    fixed = os.path.join(HERE, "_diff_scheme_fixed.jl")
    with open(fixed, "w", encoding="utf-8") as f:
        f.write("\n".join(text))
    for order, lines in ORDER_MODULES.items():
        nso = dict(ns)
        js.load_functions(fixed, ["dfdx", "dfdy", "dfdz", "d2fdx2", "d2fdy2", "d2fdz2"], nso, lines)
        # the kernels resolve the stencils through the namespace they were loaded into
        js.load_functions(os.path.join(base, "main_rk4.jl"), ["rk4_step!"] + DENSITY_KERNELS, nso)
        js.load_functions(os.path.join(base, "cov_derivs_temporal.jl"),
                          [f"D_{i}ϕ_{a}" for i in (2, 3, 4) for a in (1, 2, 3, 4)], nso)
        js.load_functions(os.path.join(base, "field_strengths.jl"),
                          [f"W_{a}_{p}" for a in (1, 2, 3) for p in ("xy", "xz", "yz")]
                          + ["Y_2_y", "Y_2_z", "Y_3_z"], nso)
        out[f"rates_{order}"] = rates(nso, y0, shape, sc, 0.07, 0.05)
        if order == 8:
            out["dens_8"] = densities(nso, y0, shape, sc)
        print("order", order, "rates", np.abs(out[f"rates_{order}"]).max(), flush=True)
    os.remove(fixed)
    np.savez_compressed(os.path.join(HERE, "ref_orders.npz"), **out)


def bubble_case(ns):
    shape = (8, 8, 8)
    S = int(np.prod(shape))
    phi = np.zeros((4, S))
    arr = [as_jarr(phi[q], shape) for q in range(4)]
    dx = 0.25
    lam = 0.129
    mH = 2.0 * math.sqrt(lam) * 1.0
    bubbles = [(3, 5, 2, 0.5, -0.3, 0.7, 0.1), (6, 2, 7, -0.2, 0.9, 0.1, -0.4)]
    nx, ny, nz = shape
    rkx = math.pi / ((nx - 1) * dx)
    rky = math.pi / ((ny - 1) * dx)
    rkz = math.pi / ((nz - 1) * dx)
    fn = ns["initializer_b"]
    for (ib, jb, kb, p1, p2, p3, p4) in bubbles:
        for k in range(1, nz + 1):
            for j in range(1, ny + 1):
                for i in range(1, nx + 1):
                    fn(*arr, ib, jb, kb, p1, p2, p3, p4, rkx, rky, rkz, dx, mH, i, j, k)
    its = np.arange(0, 400)
    jex = np.array([ns["J_ext"](int(i), 0.0125, mH, 2.0, thermal_init=True) for i in its])
    dmp = np.array([ns["damp"](int(i), 0.0125, mH, 2.0, thermal_init=True) for i in its])
    np.savez_compressed(os.path.join(HERE, "ref_bubble.npz"), shape=np.array(shape), phi=phi,
                        bubbles=np.array(bubbles, dtype=np.float64), dx=dx, mH=mH,
                        its=its, jex=jex, damp=dmp)


# deviate arrays of the thermal IC in the order run() draws them
# (main_rk4.jl:5348-5636): for W^1, W^2, W^3 and Y the ten arrays r_1, r_2,
# r_3, r_1_i, r_2_i, r_3_i, x_1, x_2, x_3, x_4, then phi_1_k .. phi_4_k
THERMAL_GROUPS = [("W_1_2", "W_1_3", "W_1_4"), ("W_2_2", "W_2_3", "W_2_4"), ("W_3_2", "W_3_3", "W_3_4"),
                  ("Y_2", "Y_3", "Y_4")]


def thermal_case(ns, seed=2718):
    """The reference's thermal IC on fixed deviates: each gauge group's
    arrays go through thermal_initializer_gauge! (r_1..r_3 become the real
    and r_1_i..r_3_i the imaginary part of the spectrum) and then
    real(bfft(re + i im)); the Higgs deviates through thermal_initializer_phi!
    and real(bfft(.)) (main_rk4.jl:5348-5636).  bfft is the unnormalised
    backward transform: numpy's ifftn times the number of sites.  Gamma,
    Sigma and the momenta stay zero, as in run()."""
    shape = (8, 7, 10)
    nx, ny, nz = shape
    S = nx * ny * nz
    rng = np.random.default_rng(seed)
    dev = rng.normal(0.0, math.sqrt(2.0), size=(44, S))
    gw, gy, gp2, vev, dx, T = 0.65, 0.35, 0.99, 1.0, 0.25, 1.5
    meff_sq = 8119.43 / 174.0 ** 2  # parameters.jl:37
    fields = np.zeros((36, S))
    spec = np.zeros((16, S), dtype=complex)

    def bfft(z):
        return np.fft.ifftn(z.reshape(shape, order="F")) * S

    np.seterr(divide="ignore")
    for g, names in enumerate(THERMAL_GROUPS):
        d = dev[10 * g:10 * g + 10].copy()
        arr = [as_jarr(d[q], shape) for q in range(10)]
        r1, r2, r3, r1i, r2i, r3i, x1, x2, x3, x4 = arr
        fn = ns["thermal_initializer_gauge_b"]
        for k in range(1, nz + 1):
            for j in range(1, ny + 1):
                for i in range(1, nx + 1):
                    fn(gw, gy, gp2, vev, dx, T, nx, ny, nz, r1, r2, r3, r1i, r2i, r3i, x1, x2, x3, x4, i, j, k)
        base = 4 + 3 * g
        for c in range(3):
            z = d[c] + 1j * d[3 + c]
            spec[base + c] = z
            fields[base + c] = bfft(z).real.ravel(order="F")
    d = dev[40:44].copy()
    arr = [as_jarr(d[q], shape) for q in range(4)]
    fn = ns["thermal_initializer_phi_b"]
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                fn(*arr, gw, gy, gp2, vev, dx, T, meff_sq, nx, ny, nz, i, j, k)
    for a in range(4):
        spec[a] = d[a]
        fields[a] = bfft(d[a]).real.ravel(order="F")
    np.savez_compressed(os.path.join(HERE, "ref_thermal.npz"), shape=np.array(shape), deviates=dev, fields=fields,
                        spec=spec, T=T, meff_sq=meff_sq, dx=dx)
    print("thermal max |field|", np.abs(fields).max(axis=1)[:16])


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference_root>")
    ref = sys.argv[1]
    ns = load(ref)
    # the damp() fixture needs the driver's gamma_inp global
    ns["γ_inp"] = 0.3
    ns["gam_inp"] = 0.3
    tw = math.asin(math.sqrt(0.22))
    pa = dict(gw=0.65, gy=0.35, gp2=0.99, lambda_=0.129, vev=1.0, dx=0.25,
              beta_w=0.3, beta_y=0.2, theta_w=tw)
    pa["lambda"] = pa.pop("lambda_")
    case(ns, "a", (8, 8, 8), pa, dt=0.0125, Jex=0.07, gam=0.05, seed=1234)
    pb = dict(pa, gy=0.65 * math.tan(tw), gp2=0.5, beta_w=0.0, beta_y=0.0, dx=0.5)
    case(ns, "b", (7, 8, 9), pb, dt=0.05, Jex=0.0, gam=0.0, seed=99)
    spectrum_case(ns)
    bubble_case(ns)
    thermal_case(ns)
    orders_case(ref, ns)


if __name__ == "__main__":
    main()
