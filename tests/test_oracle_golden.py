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


# ------------------------------------------------------------ stencil orders
ORDERS = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_orders.npz"))


def _orders_params(order):
    g = ORDERS
    shape = tuple(int(v) for v in g["shape"])
    return orc.params(shape, float(g["p_dx"]), float(g["p_gw"]), float(g["p_gy"]), float(g["p_gp2"]),
                      float(g["p_lambda"]), float(g["p_vev"]), float(g["p_beta_w"]), float(g["p_beta_y"]),
                      float(g["p_theta_w"]), order=order)


@pytest.mark.parametrize("order", [8, 10, 12])
def test_oracle_alternative_stencil_orders_bit_exact(order):
    """rk4_step! with each alternative module of diff_scheme.jl swapped in
    (8th, 10th, 12th order, diff_scheme.jl:370-1365), 14^3, beta, Jex, gamma."""
    r = orc.rates(_orders_params(order), ORDERS["y0"], float(ORDERS["Jex"]), float(ORDERS["gam"]))
    np.testing.assert_array_equal(r, ORDERS[f"rates_{order}"])


def test_oracle_second_order_module_as_written():
    """The 2nd-order module (diff_scheme.jl:1366-1438) misses the planes
    i = 2 and N-1 in its branches and returns the caller's 0 there; the
    oracle's order -2 reproduces it bit for bit, order 2 is the intended
    periodic stencil and differs exactly on those planes."""
    g = ORDERS
    shape = tuple(int(v) for v in g["shape"])
    r_ref = orc.rates(_orders_params(-2), g["y0"], float(g["Jex"]), float(g["gam"]))
    np.testing.assert_array_equal(r_ref, g["rates_2"])
    r = orc.rates(_orders_params(2), g["y0"], float(g["Jex"]), float(g["gam"]))
    nx, ny, nz = shape
    i = np.arange(nx * ny * nz) % nx
    j = (np.arange(nx * ny * nz) // nx) % ny
    k = np.arange(nx * ny * nz) // (nx * ny)
    gap = np.isin(i, (1, nx - 2)) | np.isin(j, (1, ny - 2)) | np.isin(k, (1, nz - 2))
    assert np.array_equal(r[:, ~gap], r_ref[:, ~gap])
    assert not np.array_equal(r[:, gap], r_ref[:, gap])


def test_oracle_eighth_order_densities_bit_exact():
    d = orc.densities(_orders_params(8), ORDERS["y0"])
    np.testing.assert_array_equal(d[:16], ORDERS["dens_8"])
