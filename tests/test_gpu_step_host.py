"""ewpt_step_host: host state in, n RK4 steps, host state out.

With page-locked buffers an FP64 context overlaps the upload with stage 1
of the first step and the download with stage 4 of the last step, over
windows of z planes.  Every test here holds the call to the result of
ewpt_set_state_packed + ewpt_step + ewpt_get_state_packed bit for bit (the
same kernels on the same sites), and one test holds it to the oracle at the
FP64 parity bar (1e-11 relative per array after 20 steps).
"""
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


def state(shape, dx, seed):
    y = ewpt.ic.bubbles_tanh(shape, dx, 3, seed=seed)
    rng = np.random.default_rng(seed + 1)
    y[4:] += 0.05 * rng.normal(size=y[4:].shape)
    return y


def schedule_params(shape, prec=ewpt.FP64, beta=False):
    """J_ext switches off and the damping on at it ~ 3: the per-iteration
    drive of the reference loop (main_rk4.jl:5154-5172) is exercised."""
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025, precision=prec, thermal_init=True,
                                gamma_inp=0.2, mH=2.0 * np.sqrt(0.129), beta_w=0.3 if beta else 0.0,
                                beta_y=0.2 if beta else 0.0)
    p.t_sat = 0.05
    return p


def three_calls(p, y0, n, tiling=None):
    with ewpt.Lattice(p) as lat:
        if tiling:
            lat.set_tiling(*tiling)
        lat.set_state(y0)
        lat.step(n)
        return lat.get_state(), lat.iteration


def pinned(a):
    import torch

    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
    t.numpy()[:] = a
    return t


@pytest.mark.parametrize("shape,n,beta", [((24, 20, 48), 1, False), ((16, 18, 37), 3, True),
                                          ((32, 32, 128), 2, False), ((16, 16, 16), 1, False)])
def test_overlapped_matches_three_calls(shape, n, beta):
    """nz = 48, 37, 128, 16: 3, 2 (ragged), 8 and 2 plane windows."""
    import torch

    p = schedule_params(shape, beta=beta)
    y0 = state(shape, p.dx, seed=shape[2])
    ref, it_ref = three_calls(p, y0, n, tiling=(64, 2, 2, 0))
    with ewpt.Lattice(p) as lat:
        lat.set_tiling(64, 2, 2, 0)
        src, dst = pinned(y0), torch.zeros((36, p.sites), dtype=torch.float64, pin_memory=True)
        lat.step_host(src, dst, n)
        assert lat.iteration == it_ref == n
        on_device = lat.get_state()  # the new state also stays on the device
    np.testing.assert_array_equal(dst.numpy(), ref)
    np.testing.assert_array_equal(on_device, ref)
    np.testing.assert_array_equal(src.numpy(), y0)  # the input is not written


def test_overlapped_in_place_and_continued():
    """state_in == state_out, and two calls of 2 steps equal one of 4 (the
    iteration counter carries the drive schedule across calls)."""
    shape = (20, 16, 40)
    p = schedule_params(shape)
    y0 = state(shape, p.dx, seed=5)
    ref, _ = three_calls(p, y0, 4)
    with ewpt.Lattice(p) as lat:
        buf = pinned(y0)
        lat.step_host(buf, buf, 2)
        lat.step_host(buf, buf, 2)
        assert lat.iteration == 4
    np.testing.assert_array_equal(buf.numpy(), ref)


def test_overlapped_vs_oracle():
    """20 steps through ewpt_step_host against the oracle: the FP64 bar."""
    shape = (16, 20, 32)
    p = schedule_params(shape, beta=True)
    y0 = state(shape, p.dx, seed=9)
    with ewpt.Lattice(p) as lat:
        out = pinned(np.zeros_like(y0))
        lat.step_host(pinned(y0), out, 20)
    op = orc.params(p.dims, p.dx, p.gw, p.gy, p.gp2, p.lam, p.vev, p.beta_w, p.beta_y, p.theta_w)
    yo = y0.copy()
    for it in range(1, 21):
        J = orc.jext(it, p.dt, p.mH, p.t_sat, True)
        G = orc.damp(it, p.dt, p.mH, p.t_sat, True, p.gamma_inp)
        yo = orc.rk4_step(op, yo, p.dt, J, G)
    y = out.numpy()
    scale = np.maximum(np.abs(yo).max(axis=-1), 1e-300)
    assert (np.abs(y - yo).max(axis=-1) / scale).max() < 1e-11


@pytest.mark.parametrize("prec,tiling", [(ewpt.FP64, None), (ewpt.FP32, (64, 2, 2, 1)), (ewpt.DF64, None)])
def test_sequential_forms(prec, tiling):
    """Pageable buffers (any form), and the FP32 and DF64 forms, take the
    three calls in turn: same result, same counter."""
    shape = (16, 16, 24)
    p = schedule_params(shape, prec=prec)
    y0 = state(shape, p.dx, seed=2)
    ref, it_ref = three_calls(p, y0, 2, tiling=tiling)
    bufs = [(y0, np.zeros_like(y0))]
    if prec != ewpt.FP64:
        bufs.append((pinned(y0), pinned(np.zeros_like(y0))))
    for src, dst in bufs:
        with ewpt.Lattice(p) as lat:
            if tiling:
                lat.set_tiling(*tiling)
            lat.step_host(src, dst, 2)
            assert lat.iteration == it_ref
        np.testing.assert_array_equal(np.asarray(dst), ref)


def test_rejections():
    shape = (16, 16, 16)
    p = schedule_params(shape)
    with ewpt.Lattice(p) as lat:
        L = lat.L
        y = np.zeros((36, p.sites))
        assert L.ewpt_step_host(lat.h, None, y.ctypes.data, 1) != 0
        assert "NULL" in L.ewpt_last_error(lat.h).decode()
        assert L.ewpt_step_host(lat.h, y.ctypes.data, y.ctypes.data, -1) != 0
        with pytest.raises(ValueError):
            lat.step_host(y[:, :-1], y, 1)
        with pytest.raises(ValueError):
            lat.step_host(y.astype(np.float32), y, 1)
        lat.step_host(y, y, 0)  # zero steps: a round trip of the state
        assert lat.iteration == 0
