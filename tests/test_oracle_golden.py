"""The CPU oracle against golden vectors computed from the reference's own
Julia source text (tests/golden/make_golden.py).  Integer-free FP64 work in
the reference's evaluation order: rates, the RK4 step and per-site densities
must match bit for bit; host reductions (whose summation order is Julia's
pairwise `sum`) to 1e-12 relative."""
import os

import numpy as np
import pytest

from oracle import oracle as orc


def load(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, f"ref_{name}.npz")))


def mkparams(g):
    return orc.params(tuple(int(v) for v in g["shape"]), float(g["p_dx"]), float(g["p_gw"]),
                      float(g["p_gy"]), float(g["p_gp2"]), float(g["p_lambda"]), float(g["p_vev"]),
                      float(g["p_beta_w"]), float(g["p_beta_y"]), float(g["p_theta_w"]))


@pytest.mark.parametrize("case", ["a", "b"])
def test_rates_bitwise(golden_dir, case):
    g = load(golden_dir, case)
    r = orc.rates(mkparams(g), g["y0"], float(g["Jex"]), float(g["gam"]))
    np.testing.assert_array_equal(r, g["rates"])


@pytest.mark.parametrize("case", ["a", "b"])
def test_rk4_step_bitwise(golden_dir, case):
    g = load(golden_dir, case)
    y1 = orc.rk4_step(mkparams(g), g["y0"], float(g["dt"]), float(g["Jex"]), float(g["gam"]))
    np.testing.assert_array_equal(y1, g["y1"])


@pytest.mark.parametrize("case", ["a", "b"])
def test_densities_bitwise(golden_dir, case):
    g = load(golden_dir, case)
    d = orc.densities(mkparams(g), g["y0"])
    np.testing.assert_array_equal(d[:16], g["dens"])


@pytest.mark.parametrize("case", ["a", "b"])
def test_snapshot_row(golden_dir, case):
    g = load(golden_dir, case)
    diag = orc.diagnostics(mkparams(g), g["y0"])
    np.testing.assert_allclose(diag[:14], g["row"], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("case", ["a", "b"])
def test_convolve_1d_case(golden_dir, case):
    g = load(golden_dir, case)
    spec = orc.convolve_1d(mkparams(g), g["P"], tuple(int(v) for v in g["cut"]))
    assert spec.shape == g["spec"].shape
    np.testing.assert_array_equal(spec[:, 0], g["spec"][:, 0])
    np.testing.assert_allclose(spec[:, 1], g["spec"][:, 1], rtol=1e-13)


def test_convolve_1d_random(golden_dir):
    g = load(golden_dir, "spectrum")
    shape = tuple(int(v) for v in g["shape"])
    p = orc.params(shape, 1.0, 0.65, 0.35, 0.99, 0.129, 1.0)
    cut = tuple(int(v) for v in g["cut"])
    assert orc.lib().or_kc_bin_nums(*cut) == int(g["nbins"])
    spec = orc.convolve_1d(p, g["P"], cut)
    np.testing.assert_array_equal(spec[:, 0], g["spec"][:, 0])
    np.testing.assert_allclose(spec[:, 1], g["spec"][:, 1], rtol=1e-13)


def test_bubble_and_schedules(golden_dir):
    g = load(golden_dir, "bubble")
    shape = tuple(int(v) for v in g["shape"])
    S = int(np.prod(shape))
    p = orc.params(shape, float(g["dx"]), 0.65, 0.35, 0.99, 0.129, 1.0)
    y = np.zeros((36, S))
    for b in g["bubbles"]:
        orc.bubble_rmag(p, y, b[:3], b[3:], float(g["mH"]))
    np.testing.assert_array_equal(y[:4], g["phi"])
    for it, je, dm in zip(g["its"], g["jex"], g["damp"]):
        assert orc.jext(it, 0.0125, float(g["mH"]), 2.0, True) == je
        assert orc.damp(it, 0.0125, float(g["mH"]), 2.0, True, 0.3) == dm
