"""Device thermal initial condition (ewpt_init_thermal, ewpt_ensemble_init_thermal).

The construction is thermal_initializer_phi!/gauge! (main_rk4.jl:5029-5152,
5348-5636): each field is real(bfft(amp (a + i b))) with a, b ~ N(0, sqrt 2).
The device draws its own deviates (a counter-based hash of the seed), so
the checks are the ones a random field allows:
- the power of every Fourier mode, divided by its expectation (2 S^2 amp_k^2
  per scalar component, 4 S^2 amp_k^2 summed over a polarised triplet),
  averages to 1 within five standard errors, for the device state and for
  the host restatement (ewpt.ic.thermal without momenta);
- Gamma^a and Sigma are the stencil divergences of W^a and Y (the
  constraint columns of the snapshot row vanish);
- momenta are zero;
- a seed fixes the state (any form, any member of an ensemble).
Besides: the reference's own construction from given deviates
(ewpt_init_thermal_deviates) against the transpiled reference kernels; the
device Gauss projection (ewpt_gauss_project) against the host one; and the
projected thermal IC (ewpt_init_thermal_gauss) against the constraint bars.
"""
import dataclasses
import math

import numpy as np
import pytest

import ewpt
from ewpt import ic

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 32)
T = 1.5


@pytest.fixture(scope="module", autouse=True)
def built():
    import build_lib

    build_lib.build()


def _amps(shape, dx, T, lam=0.129, gw=0.65, vev=1.0):
    """amp_k of the Higgs, W and Y spectra on the FFT grid (ic.thermal's)."""
    nx, ny, nz = shape
    th = ic._kgrid((nz, ny, nx), dx)
    TZ, TY, TX = np.meshgrid(*th, indexing="ij")
    k2 = 2.0 * ((1 - np.cos(TX)) + (1 - np.cos(TY)) + (1 - np.cos(TZ))) / dx ** 2
    vol = nx * ny * nz * dx ** 3

    def amp(m, empty_k0):
        w = np.sqrt(k2 + m * m)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            a = np.where(w > 0, np.sqrt(1.0 / np.expm1(w / T) / (w * vol)), 0.0)
        if empty_k0:
            a = np.where(k2 == 0, 0.0, a)
        return a

    return amp(math.sqrt(2 * lam) * vev, False), amp(gw * vev / 2, True), amp(0.0, True)


def _check_power(y, shape, dx):
    """Per-mode power over its expectation: for f = real(bfft(c)) with
    c_k = amp_k (a + i b), E|fft(f)_k|^2 = 2 S^2 amp_k^2 (scalar) and
    E sum_i |fft(f_i)_k|^2 = 4 S^2 amp_k^2 (two unit polarisations).  The
    mean ratio over the modes is 1 within sqrt(2 / modes) (scalar) or
    sqrt(1 / modes) (polarised); five of those are allowed."""
    nx, ny, nz = shape
    S = nx * ny * nz
    aH, aW, aY = _amps(shape, dx, T)

    def power(a):
        return np.abs(np.fft.fftn(y[a].reshape(nz, ny, nx))) ** 2

    live = aH > 0
    r = np.mean([power(a)[live] / (2 * S * S * aH[live] ** 2) for a in range(4)])
    assert abs(r - 1) < 5 * math.sqrt(2 / live.sum()) / 2, r  # four components
    for base, amp in [(4, aW), (7, aW), (10, aW), (13, aY)]:
        live = amp > 0
        pw = sum(power(base + i) for i in range(3))
        r = np.mean(pw[live] / (4 * S * S * amp[live] ** 2))
        assert abs(r - 1) < 5 * math.sqrt(1 / live.sum()), (base, r)


def test_thermal_ic_statistics_and_constraints():
    p = ewpt.baseline_couplings(shape=SHAPE, N=SHAPE[0], dx=0.25, dt=0.025)
    with ewpt.Lattice(p) as lat:
        lat.init_thermal(T, seed=12345)
        y = lat.get_state()
        d = lat.diagnostics()
        assert lat.iteration == 0
    assert np.isfinite(y).all()
    assert not y[20:].any()  # momenta zero
    _check_power(y, SHAPE, p.dx)
    # Gamma / Sigma: the divergence of W / Y with the evolution's stencil
    g_norm = math.sqrt((y[16:19] ** 2).sum() * p.dx ** 3)
    s_norm = math.sqrt((y[19] ** 2).sum() * p.dx ** 3)
    assert g_norm > 0 and s_norm > 0
    assert d[18] < 1e-12 * g_norm and d[19] < 1e-12 * s_norm
    # the host restatement of the same construction meets the same statistics
    yh = ic.thermal(SHAPE, p.dx, T=T, seed=3, with_momenta=False)
    _check_power(yh, SHAPE, p.dx)


def test_thermal_ic_seed_forms_and_members():
    shapes = [(16, 16, 16), (20, 24, 18)]
    ps = [ewpt.baseline_couplings(shape=s, N=s[0], dx=0.25, dt=0.025) for s in shapes]
    states = {}
    for p in ps:
        for prec, name in ((ewpt.FP64, "fp64"), (ewpt.FP32, "fp32"), (ewpt.DF64, "df64")):
            q = dataclasses.replace(p, precision=prec)
            with ewpt.Lattice(q) as lat:
                lat.init_thermal(T, seed=77)
                states[(p.dims, name)] = lat.get_state()
    for p in ps:
        ref = states[(p.dims, "fp64")]
        scale = np.abs(ref).max(axis=1, keepdims=True) + 1e-300
        for name in ("fp32", "df64"):  # the forms store the same state (hi/lo or double-float split)
            assert (np.abs(states[(p.dims, name)] - ref) / scale).max() < 1e-13, name
    with ewpt.Lattice(ps[0]) as lat:  # the seed fixes the state
        lat.init_thermal(T, seed=77)
        np.testing.assert_array_equal(lat.get_state(), states[(ps[0].dims, "fp64")])
        lat.init_thermal(T, seed=78)
        assert not np.array_equal(lat.get_state(), states[(ps[0].dims, "fp64")])
    # ensemble members: the single FP32 context's state, bit for bit
    ms = [dataclasses.replace(p, precision=ewpt.FP32) for p in ps]
    with ewpt.Ensemble(ms) as ens:
        for m in range(len(ms)):
            ens.init_thermal(m, T, seed=77)
        got = [ens.get_state(m) for m in range(len(ms))]
    for m, p in enumerate(ps):
        np.testing.assert_array_equal(got[m], states[(p.dims, "fp32")])


def test_thermal_ic_rejects_bad_arguments():
    p = ewpt.baseline_couplings(N=16, dx=0.25, dt=0.025)
    with ewpt.Lattice(p) as lat:
        for args in [(0.0,), (-1.0,), (float("nan"),)]:
            with pytest.raises(ewpt.EwptError):
                lat.init_thermal(*args)
        with pytest.raises(ewpt.EwptError):
            lat.init_thermal(1.5, mH=-1.0)


def test_thermal_ic_uses_the_context_stencil():
    """Gamma and Sigma are the divergences with the context's stencil order:
    with the 8th-order stencil the constraint columns of the (8th-order)
    snapshot row vanish too."""
    p = ewpt.baseline_couplings(shape=(20, 18, 22), N=20, dx=0.25, dt=0.025, stencil_order=8)
    with ewpt.Lattice(p) as lat:
        lat.init_thermal(T, seed=5)
        y = lat.get_state()
        d = lat.diagnostics()
    g_norm = math.sqrt((y[16:19] ** 2).sum() * p.dx ** 3)
    s_norm = math.sqrt((y[19] ** 2).sum() * p.dx ** 3)
    assert d[18] < 1e-12 * g_norm and d[19] < 1e-12 * s_norm


@pytest.mark.parametrize("prec", [ewpt.FP64, ewpt.FP32, ewpt.DF64])
def test_device_thermal_from_deviates_matches_reference_kernels(golden_dir, prec):
    """ewpt_init_thermal_deviates with the reference's conventions (1-based
    mode indices, massless gauge modes, mH^2 = meff_sq) against the
    reference's own thermal_initializer_gauge!/phi! + bfft evaluated on the
    same deviates (tests/golden/ref_thermal.npz): every field to 1e-12 of its
    largest value (cuFFT against numpy's FFT); Gamma, Sigma and the momenta
    zero, as in run()."""
    import math
    import os

    g = dict(np.load(os.path.join(golden_dir, "ref_thermal.npz")))
    shape = tuple(int(v) for v in g["shape"])
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=float(g["dx"]), dt=0.025, precision=prec)
    with ewpt.Lattice(p) as lat:
        lat.set_state(np.ones((36, p.sites)))  # overwritten everywhere
        lat.init_thermal_deviates(float(g["T"]), g["deviates"], mH=math.sqrt(float(g["meff_sq"])), mW=0.0)
        y = lat.get_state()
    ref = g["fields"]
    scale = np.abs(ref[:16]).max(axis=1, keepdims=True)
    assert (np.abs(y[:16] - ref[:16]) / scale).max() < 1e-12
    assert np.abs(y[16:]).max() == 0.0


@pytest.mark.parametrize("shape", [(16, 14, 18), (15, 16, 17)])
def test_device_gauss_projection_matches_host(shape):
    """ewpt_gauss_project against ewpt/ic.py gauss_project on the same
    unprojected thermal state (fields and momenta drawn, no projection):
    after 6 iterations the Higgs momenta and electric fields agree to 1e-9 of
    each array's largest value (cuFFT D2Z/Z2D and a Jacobi SVD against
    numpy's complex FFT and lstsq); every other array is untouched."""
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025)
    y0 = ic.thermal(shape, p.dx, T=1.5, gw=p.gw, gy=p.gy, seed=12, gauss_iters=0, with_momenta=True)
    yh = ic.gauss_project(y0.copy(), shape, p.dx, p.gw, p.gy, iters=6)
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        lat.gauss_project(6)
        yd = lat.get_state()
    np.testing.assert_array_equal(yd[:20], y0[:20])
    scale = np.abs(yh[20:]).max(axis=1, keepdims=True)
    assert (np.abs(yd[20:] - yh[20:]) / scale).max() < 1e-9


@pytest.mark.parametrize("prec", [ewpt.FP64, ewpt.FP32, ewpt.DF64])
def test_init_thermal_gauss_meets_the_constraints(prec):
    """ewpt_init_thermal_gauss: 20 projection iterations leave the U(1)
    Gauss violation below 1e-10 and the SU(2) one below 1e-6 of the
    unprojected state's (the host projection's bars); Gamma = div W holds
    and the momenta are the thermal ones, not zero."""
    shape = (32, 32, 32)
    p = ewpt.baseline_couplings(shape=shape, N=32, dx=0.25, dt=0.025, precision=prec)
    with ewpt.Lattice(p) as lat:
        lat.init_thermal_gauss(1.5, seed=21, gauss_iters=0)
        d0 = lat.diagnostics()
        lat.init_thermal_gauss(1.5, seed=21, gauss_iters=20)
        d1 = lat.diagnostics()
        y = lat.get_state()
    assert d0[14] > 1.0 and d0[16] > 1.0
    assert d1[16] < 1e-10 * d0[16]
    assert d1[14] < 1e-6 * d0[14]
    assert d1[18] < 1e-9 and d1[19] < 1e-9  # Gamma = div W, Sigma = div Y
    assert np.abs(y[20:]).max() > 0.0
