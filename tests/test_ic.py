"""Initial conditions (CPU): the thermal IC satisfies the discrete Gauss law
and the auxiliary-field definitions as the oracle's own stencils measure
them; bubble ICs have the documented shape."""
import math

import numpy as np
import pytest

import ewpt
from oracle import oracle as orc


def _op(shape, dx, p):
    return orc.params(shape, dx, p.gw, p.gy, p.gp2, p.lam, p.vev, 0.0, 0.0, p.theta_w)


@pytest.mark.parametrize("shape", [(16, 16, 16), (20, 14, 18), (15, 16, 17)])
def test_thermal_gauss_projected(shape):
    p = ewpt.baseline_couplings(N=shape[0])
    y = ewpt.ic.thermal(shape, 0.25, T=1.5, gw=p.gw, gy=p.gy, seed=5)
    d = orc.diagnostics(_op(shape, 0.25, p), y)
    y0 = ewpt.ic.thermal(shape, 0.25, T=1.5, gw=p.gw, gy=p.gy, seed=5, gauss_iters=0)
    d0 = orc.diagnostics(_op(shape, 0.25, p), y0)
    assert d0[14] > 1.0 and d0[16] > 1.0            # unprojected: violated
    assert d[16] < 1e-10 * d0[16] + 1e-12           # U(1): one linear projection
    assert d[14] < 1e-6 * d0[14]                    # SU(2): fixed-point iteration
    assert d[18] < 1e-10 and d[19] < 1e-10          # Gamma = div W, Sigma = div Y
    assert np.isfinite(y).all()


def test_thermal_is_seeded_and_bose_einstein_scaled():
    shape = (16, 16, 16)
    a = ewpt.ic.thermal(shape, 0.25, T=1.5, seed=1)
    b = ewpt.ic.thermal(shape, 0.25, T=1.5, seed=1)
    c = ewpt.ic.thermal(shape, 0.25, T=1.0, seed=1)
    np.testing.assert_array_equal(a, b)
    assert np.std(c[0]) < np.std(a[0])  # colder -> smaller Higgs fluctuations


def test_bubbles_tanh_profile():
    shape = (64, 64, 64)  # box 16 > bubble diameter 2R = 11.1
    y = ewpt.ic.bubbles_tanh(shape, 0.25, 1, seed=2)
    mod = np.sqrt((y[:4] ** 2).sum(axis=0))
    assert abs(mod.max() - 1.0) < 0.02          # broken phase |Phi| -> v inside
    assert mod.min() < 0.02                     # symmetric phase outside
    R = 2 / math.sqrt(0.129)
    frac = (mod > 0.5).mean()                   # volume inside the wall
    assert abs(frac - 4 / 3 * math.pi * R ** 3 / (64 * 0.25) ** 3) < 0.01


def test_bubbles_reference_profile_matches_oracle():
    p = ewpt.Params(N=24, dx=0.5, no_bubbles=3, base_seed=7)
    y = ewpt.ic.bubbles_reference(p)
    op = orc.params(p.dims, p.dx, p.gw, p.gy, p.gp2, p.lam, p.vev)
    rng = np.random.default_rng(7)
    bd = p.bub_diam
    coords = [(a, b, c) for a in range(bd, 25, bd) for b in range(bd, 25, bd) for c in range(bd, 25, bd)]
    pick = rng.choice(len(coords), size=3, replace=False)
    hoft = rng.random((3, 3))
    signs = rng.choice([-1.0, 1.0], size=3)
    yo = np.zeros_like(y)
    for b in range(3):
        orc.bubble_rmag(op, yo, coords[pick[b]], ewpt.ic.gen_phi(*hoft[b], signs[b]), p.mH)
    np.testing.assert_allclose(y[:4], yo[:4], rtol=1e-13, atol=1e-15)


def test_thermal_from_deviates_matches_reference_kernels(golden_dir):
    """The host twin of ewpt_init_thermal_deviates against the reference's
    thermal_initializer_gauge!/phi! + bfft run on the same deviates
    (tests/golden/ref_thermal.npz, made by make_golden.py from the
    reference's source): with the reference's 1-based mode indices, massless
    gauge modes and mH^2 = meff_sq, every field agrees to 1e-12."""
    import math
    import os

    g = dict(np.load(os.path.join(golden_dir, "ref_thermal.npz")))
    shape = tuple(int(v) for v in g["shape"])
    y = ewpt.ic.thermal_from_deviates(shape, float(g["dx"]), float(g["T"]), math.sqrt(float(g["meff_sq"])), 0.0,
                                 g["deviates"], one_based=True)
    ref = g["fields"]
    scale = np.abs(ref[:16]).max(axis=1, keepdims=True)
    assert (np.abs(y[:16] - ref[:16]) / scale).max() < 1e-12
    assert not y[16:].any() and not ref[16:].any()
    # with FFT-frequency modes the spectrum moves by one mode per axis: not the reference's
    y0 = ewpt.ic.thermal_from_deviates(shape, float(g["dx"]), float(g["T"]), math.sqrt(float(g["meff_sq"])), 0.0,
                                  g["deviates"], one_based=False)
    assert (np.abs(y0[:16] - ref[:16]) / scale).max() > 1e-3
