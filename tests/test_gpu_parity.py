"""GPU parity: libewpt (through its C ABI) against the CPU oracle and the
golden vectors of the reference's own kernel source.

Tolerances.  FP64 work is not bit-exact (the GPU path uses FMA and
pre-divided stencil coefficients where the reference divides): per array,
max |gpu - ref| <= tol * max |ref| with tol = 1e-12 for one rate evaluation
and 1e-11 after 100 RK4 steps (the FP64 parity bar); diagnostics 1e-10
relative; spectra 1e-10 relative per shell.
"""
import os

import numpy as np
import pytest

import ewpt
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build_lib

    build_lib.build()
    orc.build()


def rel_err(a, b):
    scale = np.maximum(np.abs(b).max(axis=-1), 1e-300)
    return (np.abs(a - b).max(axis=-1) / scale).max()


def oparams(p: ewpt.Params):
    return orc.params(p.dims, p.dx, p.gw, p.gy, p.gp2, p.lam, p.vev, p.beta_w, p.beta_y, p.theta_w,
                      order=p.stencil_order)


def golden(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, f"ref_{name}.npz")))


def params_from_golden(g, **over):
    shape = tuple(int(v) for v in g["shape"])
    return ewpt.Params(shape=shape, N=shape[0], dx=float(g["p_dx"]), dt=float(g["dt"]), gw=float(g["p_gw"]),
                       gy=float(g["p_gy"]), gp2=float(g["p_gp2"]), lam=float(g["p_lambda"]),
                       vev=float(g["p_vev"]), beta_w=float(g["p_beta_w"]), beta_y=float(g["p_beta_y"]),
                       theta_w=float(g["p_theta_w"]), **over)


def perturbed_bubbles(shape, dx, nb, seed, amp=0.05):
    y = ewpt.ic.bubbles_tanh(shape, dx, nb, seed=seed)
    rng = np.random.default_rng(seed + 1)
    y[4:] += amp * rng.normal(size=y[4:].shape)  # gauge fields, aux and momenta non-zero
    return y


@pytest.mark.parametrize("case", ["a", "b"])
def test_rk4_rates_dropin_matches_golden(golden_dir, case):
    import torch

    g = golden(golden_dir, case)
    p = params_from_golden(g)
    yin = torch.tensor(g["y0"], device="cuda:0", dtype=torch.float64).contiguous()
    out = torch.zeros_like(yin)
    ewpt.rk4_rates_device(p, [yin[a].data_ptr() for a in range(36)], [out[a].data_ptr() for a in range(36)],
                          float(g["Jex"]), float(g["gam"]), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    r = out.cpu().numpy()
    assert rel_err(r, g["rates"]) < 1e-12


@pytest.mark.parametrize("case", ["a", "b"])
def test_one_step_matches_golden(golden_dir, case):
    g = golden(golden_dir, case)
    p = params_from_golden(g)
    with ewpt.Lattice(p) as lat:
        lat.set_state(g["y0"])
        lat.step(1, Jex=float(g["Jex"]), gamma=float(g["gam"]))
        y1 = lat.get_state()
    assert rel_err(y1, g["y1"]) < 1e-12


@pytest.mark.parametrize("shape,beta", [((20, 24, 16), True), ((32, 32, 32), False)])
def test_fp64_100_steps_vs_oracle(shape, beta):
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025,
                                beta_w=0.3 if beta else 0.0, beta_y=0.2 if beta else 0.0)
    y0 = perturbed_bubbles(shape, p.dx, 4, seed=11)
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        lat.step(100, Jex=0.02, gamma=0.01)
        y = lat.get_state()
    yo = orc.rk4_step(oparams(p), y0, p.dt, 0.02, 0.01, nsteps=100)
    assert np.isfinite(y).all()
    assert rel_err(y, yo) < 1e-11


def test_fp64_energy_and_gauss_history_vs_oracle():
    """The snapshot rows every 10 of 100 steps (13 energy columns, total,
    the Gauss-constraint norms and maxima) follow the oracle's history."""
    shape = (24, 20, 28)
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025, beta_w=0.2, beta_y=0.1)
    y0 = perturbed_bubbles(shape, p.dx, 4, seed=21)
    op = oparams(p)
    rows, ref = [], []
    yo = y0.copy()
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        rows.append(lat.diagnostics())
        ref.append(orc.diagnostics(op, yo))
        for _ in range(10):
            lat.step(10, Jex=0.02, gamma=0.01)
            rows.append(lat.diagnostics())
            yo = orc.rk4_step(op, yo, p.dt, 0.02, 0.01, nsteps=10)
            ref.append(orc.diagnostics(op, yo))
    rows, ref = np.array(rows), np.array(ref)
    assert np.abs(rows[:, 14:20]).min() > 0  # the constraint is violated: the columns carry signal
    np.testing.assert_allclose(rows, ref, rtol=1e-10, atol=1e-13)


@pytest.mark.parametrize("shape,beta", [((20, 24, 16), True), ((32, 32, 32), False)])
def test_df64_100_steps_vs_oracle(shape, beta):
    """The DF64 form (FP64 scheme in double-float arithmetic on the FP32
    pipes) meets the FP64 parity bar: 1e-11 relative per field after 100
    steps, with beta terms, J_ext and damping."""
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025, precision=ewpt.DF64,
                                beta_w=0.3 if beta else 0.0, beta_y=0.2 if beta else 0.0)
    y0 = perturbed_bubbles(shape, p.dx, 4, seed=11)
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        lat.step(100, Jex=0.02, gamma=0.01)
        y = lat.get_state()
        d = lat.diagnostics()
    yo = orc.rk4_step(oparams(p), y0, p.dt, 0.02, 0.01, nsteps=100)
    assert np.isfinite(y).all()
    assert rel_err(y, yo) < 1e-11
    do = orc.diagnostics(oparams(p), yo)
    np.testing.assert_allclose(d[:14], do[:14], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("prec", [ewpt.FP64, ewpt.FP32, ewpt.DF64])
def test_state_io_separate_and_packed_arrays(prec):
    """ewpt_set_state / ewpt_get_state with 36 separate host arrays (one copy
    each; some of them back to back, which the library merges into one
    copy) give the same state as the packed entry points."""
    shape = (12, 10, 14)
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025, precision=prec)
    y = perturbed_bubbles(shape, p.dx, 2, seed=4, amp=0.1)
    L = ewpt._lib
    # arrays 0-9 back to back in one block, the others separate
    block = np.ascontiguousarray(y[:10])
    sep = [np.ascontiguousarray(y[a]) for a in range(10, 36)]
    ptrs = L.DPA(*([block[a].ctypes.data_as(L.DP) for a in range(10)] + [v.ctypes.data_as(L.DP) for v in sep]))
    with ewpt.Lattice(p) as lat:
        lat._chk(lat.L.ewpt_set_state(lat.h, ptrs, 0))
        packed = lat.get_state()
        outs = [np.zeros(p.sites) for _ in range(36)]
        optr = L.DPA(*[o.ctypes.data_as(L.DP) for o in outs])
        lat._chk(lat.L.ewpt_get_state(lat.h, optr, 0))
        lat.set_state(y)
        ref = lat.get_state()
    np.testing.assert_array_equal(packed, ref)
    np.testing.assert_array_equal(np.array(outs), ref)
    if prec == ewpt.FP64:
        np.testing.assert_array_equal(ref, y)


def test_df64_state_roundtrip_and_golden_step(golden_dir):
    """set_state / get_state of a DF64 context is exact to the double-float
    split (2^-48), and one DF64 step matches the golden FP64 step to 1e-12."""
    g = golden(golden_dir, "a")
    p = params_from_golden(g)
    p.precision = ewpt.DF64
    with ewpt.Lattice(p) as lat:
        lat.set_state(g["y0"])
        back = lat.get_state()
        assert rel_err(back, g["y0"]) < 1e-14
        lat.step(1, Jex=float(g["Jex"]), gamma=float(g["gam"]))
        y1 = lat.get_state()
    assert rel_err(y1, g["y1"]) < 1e-12


def test_step_schedule_jext_damp():
    """ewpt_step applies J_ext/damp per iteration (main_rk4.jl:5154-5172)."""
    shape = (16, 16, 16)
    p = ewpt.baseline_couplings(shape=shape, N=16, dx=0.25, dt=0.05, thermal_init=True, gamma_inp=0.3,
                                mH=2.0 * np.sqrt(0.129))
    p.t_sat = 0.5  # it*dt*mH crosses t_sat at it ~ 14, inside the 30 steps
    y0 = perturbed_bubbles(shape, p.dx, 2, seed=3)
    op = oparams(p)
    yo = y0.copy()
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        lat.step(30)
        y = lat.get_state()
        assert lat.iteration == 30
    for it in range(1, 31):
        J = orc.jext(it, p.dt, p.mH, p.t_sat, True)
        G = orc.damp(it, p.dt, p.mH, p.t_sat, True, p.gamma_inp)
        yo = orc.rk4_step(op, yo, p.dt, J, G)
    assert rel_err(y, yo) < 1e-11


@pytest.mark.parametrize("shape", [(16, 16, 16), (20, 18, 22)])
def test_diagnostics_vs_oracle(shape):
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025)
    y0 = perturbed_bubbles(shape, p.dx, 3, seed=7, amp=0.2)
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        d = lat.diagnostics()
    do = orc.diagnostics(oparams(p), y0)
    np.testing.assert_allclose(d, do, rtol=1e-10, atol=1e-13)


def test_diagnostics_match_golden_row(golden_dir):
    g = golden(golden_dir, "a")
    p = params_from_golden(g)
    with ewpt.Lattice(p) as lat:
        lat.set_state(g["y0"])
        d = lat.diagnostics()
    np.testing.assert_allclose(d[:14], g["row"], rtol=1e-10)


def _oracle_power(p, y, field):
    den = orc.densities(oparams(p), y)
    if field == "B":
        comps = [den[7], den[8], den[9]]
    elif field == "B2":
        comps = [den[10], den[11], den[12]]
    else:
        comps = [y[a] - y[a].mean() for a in range(4)]
    P = np.zeros(y.shape[1])
    for f in comps:
        F = np.fft.fftn(f.reshape(p.dims[::-1]))
        P += (np.abs(F) ** 2).ravel()
    return P


@pytest.mark.parametrize("field", ["B", "B2", "higgs"])
@pytest.mark.parametrize("shape", [(16, 16, 16), (18, 16, 20)])
def test_spectrum_log_shells_vs_oracle(field, shape):
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025)
    y0 = perturbed_bubbles(shape, p.dx, 3, seed=9, amp=0.2)
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        s = lat.spectrum(field, "log", 12)
    ref = orc.shell_spectrum(oparams(p), _oracle_power(p, y0, field), 12)
    np.testing.assert_array_equal(s["count"], ref["count"])
    np.testing.assert_allclose(s["sum"], ref["sum"], rtol=1e-10)
    np.testing.assert_allclose(s["mean"], ref["mean"], rtol=1e-10)


def test_spectrum_unique_matches_convolve_1d_golden(golden_dir):
    g = golden(golden_dir, "a")
    p = params_from_golden(g)
    cut = tuple(int(v) for v in g["cut"])
    nb = ewpt.kc_bin_nums(*cut)
    with ewpt.Lattice(p) as lat:
        lat.set_state(g["y0"])
        s = lat.spectrum("B", "unique", nb)
    np.testing.assert_array_equal(s["k"], g["spec"][:, 0])
    np.testing.assert_allclose(s["mean"], g["spec"][:, 1], rtol=1e-10)


@pytest.mark.parametrize("tile", [(32, 4, 0, 0), (32, 4, 0, 1), (64, 2, 2, 1)])
def test_fp32_tilings_agree(tile):
    """Every FP32 launch shape (incl. two sites per thread with packed FP32x2
    arithmetic) gives the same evolution to FP32 round-off."""
    shape = (32, 24, 20)
    p32 = ewpt.baseline_couplings(shape=shape, N=32, dx=0.25, dt=0.025, precision=ewpt.FP32, beta_w=0.2)
    y0 = perturbed_bubbles(shape, p32.dx, 3, seed=8, amp=0.02)
    res = []
    for t in [(32, 4, 0, 0), tile]:
        with ewpt.Lattice(p32) as lat:
            lat.set_state(y0)
            lat.set_tiling(*t)
            assert lat.tiling() == t
            lat.step(20)
            res.append(lat.get_state())
    assert rel_err(res[1], res[0]) < 2e-5


@pytest.mark.parametrize("shape,beta", [((32, 24, 20), 0.2), ((64, 8, 12), 0.0), ((32, 8, 8), 0.1)])
def test_fp32_tma_tiles_match_pair_kernel(shape, beta):
    """TMA-staged shared-memory tiles (tiling mode 2) run the same packed
    FP32x2 arithmetic as the two-sites-per-thread kernel: bit-identical
    states, through the J_ext/damp schedule and with beta terms, on lattices
    with one to eight tiles per axis, so boxes at every face read their halo
    from the ghost cells."""
    p32 = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025, precision=ewpt.FP32, beta_w=beta,
                                  beta_y=0.5 * beta)
    y0 = perturbed_bubbles(shape, p32.dx, 3, seed=11, amp=0.02)
    res = []
    for t in [(32, 4, 0, 1), (32, 4, 4, 2), (32, 2, 4, 2)]:
        with ewpt.Lattice(p32) as lat:
            lat.set_state(y0)
            lat.set_tiling(*t)
            assert lat.tiling() == t
            lat.step(6, Jex=0.03, gamma=0.01)
            lat.step(6)
            res.append(lat.get_state())
            d = lat.diagnostics()
    for r in res[1:]:
        np.testing.assert_array_equal(r, res[0])
    assert np.isfinite(d).all()


def test_fp32_tma_tiles_switch_modes_midrun():
    """The three FP32 tiling modes share one state: switching mid-run gives
    the same evolution as staying in the paired mode."""
    shape = (32, 16, 16)
    p32 = ewpt.baseline_couplings(shape=shape, N=32, dx=0.25, dt=0.025, precision=ewpt.FP32)
    y0 = perturbed_bubbles(shape, p32.dx, 2, seed=5, amp=0.02)
    with ewpt.Lattice(p32) as lat:
        lat.set_state(y0)
        lat.set_tiling(32, 4, 0, 1)
        lat.step(9)
        ref = lat.get_state()
    with ewpt.Lattice(p32) as lat:
        lat.set_state(y0)
        for t in ((32, 4, 4, 2), (32, 4, 0, 1), (32, 2, 4, 2)):
            lat.set_tiling(*t)
            lat.step(3)
        got = lat.get_state()
    np.testing.assert_array_equal(got, ref)


def test_fp32_tma_tiles_reject_bad_contexts():
    p64 = ewpt.baseline_couplings(shape=(32, 8, 8), N=32, dx=0.25, dt=0.025)
    with ewpt.Lattice(p64) as lat, pytest.raises(ewpt.EwptError):
        lat.set_tiling(32, 4, 4, 2)  # FP64 context
    p32 = ewpt.baseline_couplings(shape=(24, 8, 8), N=24, dx=0.25, dt=0.025, precision=ewpt.FP32)
    with ewpt.Lattice(p32) as lat:
        with pytest.raises(ewpt.EwptError):
            lat.set_tiling(32, 4, 4, 2)  # nx not a multiple of 32
        with pytest.raises(ewpt.EwptError):
            lat.set_tiling(32, 3, 4, 2)  # tile shape not offered
        with pytest.raises(ewpt.EwptError):
            lat.set_tiling(32, 4, 2, 2)
        assert lat.tiling() == (32, 4, 0, 0)


@pytest.mark.parametrize("ic_kind", ["bubbles", "thermal"])
def test_fp32_form_tracks_fp64(ic_kind):
    """The FP32 form's bars against FP64 after 100 steps, with no floors:
    fields within 1e-4 (per array, of its largest value), the energy change
    |E(t) - E(0)| and the Gauss violation ||G_W||, ||G_Y|| within 2x of
    FP64's, and the B spectrum within 1e-4 per shell.  Both ICs move the
    FP64 energy measurably (about 2.4e-3 E0 for the bubbles and 0.13 E0 for
    the T = 1.5 thermal state over 100 steps, the constraint formulation's
    own drift), so each 2x bar can fail."""
    shape = (32, 32, 32)
    p64 = ewpt.baseline_couplings(shape=shape, N=32, dx=0.25, dt=0.025)
    p32 = ewpt.baseline_couplings(shape=shape, N=32, dx=0.25, dt=0.025, precision=ewpt.FP32)
    y0 = ewpt.ic.bubbles_tanh(shape, p64.dx, 4, seed=21)
    res = {}
    for name, p in (("64", p64), ("32", p32), ("32x2", p32), ("32tma", p32)):
        with ewpt.Lattice(p) as lat:
            if ic_kind == "thermal":
                lat.init_thermal(1.5, seed=3)
            else:
                lat.set_state(y0)
            if name == "32x2":
                lat.set_tiling(32, 4, 0, 1)
            if name == "32tma":
                lat.set_tiling(32, 4, 4, 2)
            d0 = lat.diagnostics()
            lat.step(100)
            res[name] = (lat.get_state(), d0, lat.diagnostics(), lat.spectrum("B", "log", 12))
    y64 = res["64"][0]
    e0 = res["64"][1][13]
    drift64 = abs(res["64"][2][13] - e0)
    assert drift64 > 1e-3 * abs(e0)  # the bar has something to measure
    gw64, gy64 = res["64"][2][14], res["64"][2][16]
    s64 = res["64"][3]["mean"]
    m = s64 > 1e-12 * s64.max()
    for name in ("32", "32x2", "32tma"):
        y32 = res[name][0]
        assert rel_err(y32[:20], y64[:20]) < 1e-4
        assert abs(res[name][2][13] - res[name][1][13]) <= 2.0 * drift64
        assert res[name][2][14] <= 2.0 * gw64 and res[name][2][16] <= 2.0 * gy64
        np.testing.assert_allclose(res[name][3]["mean"][m], s64[m], rtol=1e-4)


def test_fp32_compensated_mode_tracks_fp64_closer():
    """The FP32 form's compensated mode (gauge Laplacians and auxiliary
    gradients compensated, lap - grad formed before rounding) against FP64 on
    a thermal 48^3 state (T = 1.5, fields projected onto the Gauss law), 300
    steps: the B spectrum within 1e-4 per shell and at most half the plain
    FP32 form's error there, fields closer than the plain form's, energy
    drift and Gauss violation within 2x of FP64's."""
    shape = (48, 48, 48)
    p64 = ewpt.baseline_couplings(shape=shape, N=48, dx=0.25, dt=0.025)
    p32 = ewpt.baseline_couplings(shape=shape, N=48, dx=0.25, dt=0.025, precision=ewpt.FP32)
    y0 = ewpt.ic.thermal(shape, 0.25, T=1.5, seed=7, gauss_iters=20)
    res = {}
    for name, p, comp in (("64", p64, False), ("32", p32, False), ("32c", p32, True)):
        with ewpt.Lattice(p) as lat:
            lat.set_state(y0)
            if p is p32:
                lat.set_tiling(8, 16, 2, 1)
            if comp:
                lat.set_fp32_compensated(True)
                assert lat.fp32_compensated()
            d0 = lat.diagnostics()
            lat.step(300)
            res[name] = (lat.get_state(), d0, lat.diagnostics(), lat.spectrum("B", "log", 40)["mean"])
    y64, d064, d64, s64 = res["64"]
    m = s64 > 1e-12 * s64.max()
    drift64 = abs(d64[13] - d064[13])
    assert drift64 > 1e-3 * abs(d064[13])  # the 2x bar has something to measure

    def errs(name):
        y, d0, d, sp = res[name]
        assert np.isfinite(y).all() and np.isfinite(sp).all()
        field = max(float(np.abs(y[q] - y64[q]).max() / np.abs(y64[q]).max()) for q in range(36))
        spec = float((np.abs(sp - s64)[m] / s64[m]).max())
        assert abs(d[13] - d0[13]) <= 2.0 * drift64
        assert d[14] <= 2.0 * d64[14] and d[16] <= 2.0 * d64[16]
        return field, spec

    f32, sp32 = errs("32")
    f32c, sp32c = errs("32c")
    assert sp32c < 1e-4 and sp32c <= 0.5 * sp32, (sp32c, sp32)
    assert f32c < f32, (f32c, f32)


def test_fp32_compensated_mode_rejections():
    p64 = ewpt.baseline_couplings(shape=(16, 16, 16), N=16, dx=0.25, dt=0.025)
    with ewpt.Lattice(p64) as lat, pytest.raises(ewpt.EwptError):
        lat.set_fp32_compensated(True)  # FP64 context
    p32 = ewpt.baseline_couplings(shape=(16, 16, 16), N=16, dx=0.25, dt=0.025, precision=ewpt.FP32)
    with ewpt.Lattice(p32) as lat:
        with pytest.raises(ewpt.EwptError):
            lat.set_fp32_compensated(True)  # the default tiling has one site per thread
        lat.set_tiling(32, 4, 2, 1)
        lat.set_fp32_compensated(True)
        for t in ((32, 4, 0, 0), (32, 4, 4, 2)):
            with pytest.raises(ewpt.EwptError):
                lat.set_tiling(*t)  # the compensated mode keeps two sites per thread
        lat.set_tiling(16, 8, 0, 1)
        lat.set_state(perturbed_bubbles((16, 16, 16), 0.25, 2, seed=3, amp=0.02))  # |Phi| > 0 (the damping's 0/0)
        lat.step(2)
        assert np.isfinite(lat.get_state()).all()
        lat.set_fp32_compensated(False)
        lat.set_tiling(32, 4, 0, 0)
        assert not lat.fp32_compensated()


@pytest.mark.parametrize("prec", [ewpt.FP64, ewpt.FP32])
def test_device_bubble_ic_matches_host(prec):
    shape = (24, 20, 18)
    p = ewpt.baseline_couplings(shape=shape, N=24, dx=0.25, dt=0.025, precision=prec)
    bl = ewpt.ic.tanh_bubble_list(shape, p.dx, 5, seed=12)
    R, w = ewpt.ic.tanh_profile_params(p.lam, p.vev)
    host = ewpt.ic.bubbles_tanh(shape, p.dx, 5, lam=p.lam, vev=p.vev, seed=12)
    with ewpt.Lattice(p) as lat:
        lat.set_state(np.ones((36, p.sites)))  # must be overwritten everywhere
        lat.init_bubbles(bl, "tanh", R, w)
        dev = lat.get_state()
    np.testing.assert_allclose(dev, host, rtol=0, atol=1e-14)


def test_device_reference_bubble_ic_matches_oracle():
    shape = (20, 20, 20)
    p = ewpt.baseline_couplings(shape=shape, N=20, dx=0.5, dt=0.05)
    bl = np.array([[3, 5, 2, 0.5, -0.3, 0.7, 0.1], [16, 12, 7, -0.2, 0.9, 0.1, -0.4]], dtype=np.float64)
    op = oparams(p)
    yo = np.zeros((36, p.sites))
    for b in bl:
        orc.bubble_rmag(op, yo, b[:3], b[3:], p.mH)
    with ewpt.Lattice(p) as lat:
        lat.init_bubbles(bl, "reference")
        dev = lat.get_state()
    np.testing.assert_allclose(dev, yo, rtol=1e-13, atol=1e-15)


def test_driver_energy_table_matches_oracle(tmp_path):
    """ewpt.run (the run() driver mirror): the energy table every dsnaps steps
    equals the oracle evolving the same reference-placement bubble IC."""
    from ewpt import run as drv

    args = ["0.0", "4", "20", "0.25", "10", "32", "0.99", "4", "0.0", "0.0", "0.0", "2"]
    p = ewpt.Params.from_args(args)
    res = drv.run(p, out_dir=str(tmp_path), nshell=12, verbose=False)
    assert res["energies"].shape == (5, 13) and res["iterations"] == 20
    assert (tmp_path / "energies.npy").exists()
    op = oparams(p)
    y = np.zeros((36, p.sites))
    for b in drv.reference_bubble_list(p):
        orc.bubble_rmag(op, y, b[:3], b[3:], p.mH)
    rows = [orc.diagnostics(op, y)]
    for _ in range(4):
        y = orc.rk4_step(op, y, p.dt, 0.0, 0.0, nsteps=p.dsnaps)
        rows.append(orc.diagnostics(op, y))
    ref = np.array(rows)
    np.testing.assert_allclose(res["energies"], ref[:, :13], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(res["total"], ref[:, 13], rtol=1e-9)


@pytest.mark.parametrize("prec", [ewpt.FP64, ewpt.FP32, ewpt.DF64])
def test_fields_match_oracle_densities(prec):
    """ewpt_fields: the energy densities, B and B_2 per site equal the
    oracle's site densities (the E_t arrays of compute_PE! .. compute_B_2_z!),
    the Higgs field is the stored state, and the sums times dx^3 are the
    diagnostics row."""
    shape = (18, 16, 20)
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025, precision=prec)
    y0 = perturbed_bubbles(shape, p.dx, 3, seed=5, amp=0.2)
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        y = lat.get_state()  # the state as this form holds it
        dens, B, B2, H = (lat.fields(f) for f in ("density", "B", "B2", "higgs"))
        row = lat.diagnostics()
        with pytest.raises(ewpt.EwptError):
            lat._chk(lat.L.ewpt_fields(lat.h, 9, B.ctypes.data_as(ewpt._lib.DP), 0))
    den = orc.densities(oparams(p), y)
    assert dens.shape == (7, p.sites) and B.shape == B2.shape == (3, p.sites) and H.shape == (4, p.sites)
    assert rel_err(dens, den[:7]) < 1e-12
    assert rel_err(B, den[7:10]) < 1e-12
    assert rel_err(B2, den[10:13]) < 1e-12
    np.testing.assert_array_equal(H, y[:4])
    np.testing.assert_allclose(dens.sum(axis=1) * p.dx ** 3, row[:7], rtol=1e-11)
    np.testing.assert_allclose(0.5 * (B ** 2).sum() * p.dx ** 3, row[7], rtol=1e-11)


def test_driver_reference_outputs(tmp_path):
    """ewpt.run writes the datasets of data.h5 and 3d-fft-data-<it>.h5 as
    .npz: y_slices_snaps are the y = Ny/2 planes of the oracle's densities
    and B sums times dx^3 (main_rk4.jl:5700-5960), and the FFT dump is
    fft(E_t) of the oracle's B and B_2 over the Julia axes."""
    from ewpt import run as drv
    from ewpt.lattice import julia_array

    args = ["0.0", "4", "20", "0.25", "10", "32", "0.99", "4", "0.0", "0.0", "0.0", "2"]
    p = ewpt.Params.from_args(args, nsnaps_fft=2)
    res = drv.run(p, out_dir=str(tmp_path), nshell=12, verbose=False, fft_dumps=True)
    z = np.load(tmp_path / "data.npz")
    for k in ("Nx", "gp2", "dx", "dt", "nte", "gamma", "T", "meff_sq", "t_sat_jex", "nsnaps", "dsnaps",
              "no_bubbles", "bubble_locations", "Hoft_angles", "energies", "y_slices_snaps"):
        assert k in z.files, k
    nx, ny, nz = p.dims
    assert z["energies"].shape == (5, 13) and z["y_slices_snaps"].shape == (5, 7, nx, nz)
    assert z["bubble_locations"].shape == (4, 3) and z["Hoft_angles"].shape == (4, 3)
    np.testing.assert_array_equal(z["energies"], res["energies"])
    # snapshot 0 against the oracle's densities of the same IC
    op = oparams(p)
    y = np.zeros((36, p.sites))
    for b in drv.reference_bubble_list(p):
        orc.bubble_rmag(op, y, b[:3], b[3:], p.mH)
    den = orc.densities(op, y)
    vol = p.dx ** 3
    j = ny // 2 - 1

    def plane(q):
        return julia_array(den[q], p.dims)[:, j, :] * vol

    s0 = z["y_slices_snaps"][0]
    scale = np.abs(s0).max()
    for q, ref in enumerate([plane(0), plane(1), plane(2), plane(4) + plane(3) + plane(6) + plane(5),
                             plane(7) + plane(8) + plane(9), plane(10) + plane(11) + plane(12)]):
        assert np.abs(s0[q] - ref).max() <= 1e-11 * scale, q
    assert not s0[6].any()
    # FFT dumps at iteration 0 and every dsnaps_fft = 10 steps at snapshots (5, 10, 15, 20)
    assert list(res["fft_dump_iterations"]) == [0, 10, 20]
    f0 = np.load(tmp_path / "3d-fft-data-0.npz")
    assert sorted(f0.files) == sorted(["3D_fft_x", "3D_fft_y", "3D_fft_z", "3D_fft_x2", "3D_fft_y2", "3D_fft_z2"])
    for name, q in (("3D_fft_x", 7), ("3D_fft_z", 9), ("3D_fft_y2", 11)):
        ref = np.fft.fftn(julia_array(den[q], p.dims))
        assert f0[name].shape == (nx, ny, nz) and f0[name].dtype == np.complex128
        assert np.abs(f0[name] - ref).max() <= 1e-10 * np.abs(ref).max(), name
    assert (tmp_path / "3d-fft-data-20.npz").exists()


# ------------------------------------------------------------ stencil orders
@pytest.mark.parametrize("order", [8, 10, 12])
def test_alternative_order_rates_match_golden(golden_dir, order):
    """ewpt_rk4_rates with stencil_order 8/10/12 against rk4_step! run with
    the reference's own 8th/10th/12th-order modules (14^3, beta, Jex, gamma)."""
    import torch

    g = golden(golden_dir, "orders")
    p = params_from_golden(dict(g, dt=0.01), stencil_order=order)
    yin = torch.tensor(g["y0"], device="cuda:0", dtype=torch.float64).contiguous()
    out = torch.zeros_like(yin)
    ewpt.rk4_rates_device(p, [yin[a].data_ptr() for a in range(36)], [out[a].data_ptr() for a in range(36)],
                          float(g["Jex"]), float(g["gam"]), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rel_err(out.cpu().numpy(), g[f"rates_{order}"]) < 1e-12


def test_second_order_rates_match_oracle(golden_dir):
    """stencil_order 2 is the periodic 2nd-order stencil everywhere (the
    reference's module misses the planes i = 2 and N-1; see the oracle tests)."""
    import torch

    g = golden(golden_dir, "orders")
    p = params_from_golden(dict(g, dt=0.01), stencil_order=2)
    yin = torch.tensor(g["y0"], device="cuda:0", dtype=torch.float64).contiguous()
    out = torch.zeros_like(yin)
    ewpt.rk4_rates_device(p, [yin[a].data_ptr() for a in range(36)], [out[a].data_ptr() for a in range(36)],
                          float(g["Jex"]), float(g["gam"]), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ref = orc.rates(oparams(p), g["y0"], float(g["Jex"]), float(g["gam"]))
    assert rel_err(out.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("order", [2, 8, 10, 12])
def test_alternative_order_20_steps_and_diagnostics_vs_oracle(order):
    shape = (16, 18, 14)
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.3, dt=0.02, beta_w=0.3, beta_y=0.2,
                                stencil_order=order)
    y0 = perturbed_bubbles(shape, p.dx, 3, seed=17)
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        lat.step(20, Jex=0.02, gamma=0.01)
        y = lat.get_state()
        d = lat.diagnostics()
    yo = orc.rk4_step(oparams(p), y0, p.dt, 0.02, 0.01, nsteps=20)
    assert rel_err(y, yo) < 1e-11
    do = orc.diagnostics(oparams(p), yo)
    np.testing.assert_allclose(d[:14], do[:14], rtol=1e-9, atol=1e-12)


def test_alternative_orders_rejected_where_not_offered():
    with pytest.raises(ewpt.EwptError):
        ewpt.Lattice(ewpt.baseline_couplings(shape=(16, 16, 16), N=16, precision=ewpt.FP32, stencil_order=8))
    with pytest.raises(ewpt.EwptError):
        ewpt.Lattice(ewpt.baseline_couplings(shape=(12, 16, 16), N=12, stencil_order=12))  # nx < 13
    with pytest.raises(ewpt.EwptError):
        ewpt.Lattice(ewpt.baseline_couplings(shape=(16, 16, 16), N=16, stencil_order=4))


# ------------------------------------------------------------ largest lattice
def test_largest_lattice_forms_agree():
    """512^3 (36 S = 4.8e9 > 2^31 array elements; FP64 context 155 GB):
    the same device bubble IC stepped twice by the FP64, DF64 and FP32 forms
    gives the same snapshot row (DF64 to the FP64 bar, FP32 to its
    round-off), so the 64-bit array offsets, the ghosted FP32 layout and the
    autotuned launch shapes hold at the largest size the GPU takes."""
    from ewpt import autotune

    N = 512
    rows = {}
    for name, prec in (("fp64", ewpt.FP64), ("df64", ewpt.DF64), ("fp32", ewpt.FP32)):
        p = ewpt.baseline_couplings(N=N, dx=0.25, dt=0.025, precision=prec)
        R, w = ewpt.ic.tanh_profile_params(p.lam, p.vev)
        # the sweep runs on its own scratch lattice: pick the shape first
        tile = autotune.best_tiling(p, steps=1) if prec == ewpt.FP32 else None
        with ewpt.Lattice(p) as lat:
            lat.init_bubbles(ewpt.ic.tanh_bubble_list(p.dims, p.dx, 64, seed=3), "tanh", R, w)
            if tile:
                lat.set_tiling(*tile)
            lat.step(2)
            rows[name] = lat.diagnostics()
    for r in rows.values():
        assert np.isfinite(r).all()
    cols = [0, 1, 2, 3, 4, 7, 11, 13]  # PE KE GE EEW MEW EB mean|phi| total
    np.testing.assert_allclose(rows["df64"][cols], rows["fp64"][cols], rtol=1e-10)
    np.testing.assert_allclose(rows["fp32"][cols], rows["fp64"][cols], rtol=1e-4)
