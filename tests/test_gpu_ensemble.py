"""Batched ensemble (FP32 form): each member of a mixed-size ensemble is a
single-lattice FP32 context stepped from one CUDA graph with a concurrent
branch per member, so it evolves bit for bit like a single lattice with the
same tiling (ensemble-wide or per member); diagnostics and spectra of members
match single contexts."""
import numpy as np
import pytest

import ewpt

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16, 16), (20, 24, 14), (24, 18, 20), (32, 16, 24)]


@pytest.fixture(scope="module", autouse=True)
def built():
    import build_lib

    build_lib.build()


def _members(beta=0.0):
    ps = []
    for n, shp in enumerate(SHAPES):
        dx = 0.25 if n % 2 == 0 else 0.3
        ps.append(ewpt.baseline_couplings(shape=shp, N=shp[0], dx=dx, dt=dx / 10, precision=ewpt.FP32,
                                          lam=0.129 + 0.01 * n, beta_w=beta))
    return ps


def _states(ps):
    out = []
    for n, p in enumerate(ps):
        y = ewpt.ic.bubbles_tanh(p.dims, p.dx, 2, seed=40 + n)
        y[4:] += 0.02 * np.random.default_rng(n).normal(size=y[4:].shape)
        out.append(y)
    return out


@pytest.mark.parametrize("pair", [1, 0])
def test_members_match_single_lattices(pair):
    ps = _members(beta=0.1)
    ys = _states(ps)
    with ewpt.Ensemble(ps) as ens:
        assert len(ens) == len(ps) and ens.sites == sum(p.sites for p in ps)
        ens.set_tiling(32, 4, pair)
        for m, y in enumerate(ys):
            ens.set_state(m, y)
        ens.set_drive(1, 0.05, 0.02)
        ens.step(12)
        got = [ens.get_state(m) for m in range(len(ps))]
        dg = [ens.diagnostics(m) for m in range(len(ps))]
        sp = ens.spectrum(2, "B", "log", 8)
    for m, (p, y) in enumerate(zip(ps, ys)):
        with ewpt.Lattice(p) as lat:
            lat.set_state(y)
            lat.set_tiling(32, 4, 2, pair)  # the ensemble runs member tilings with <= 168 registers
            if m == 1:
                lat.step(12, Jex=0.05, gamma=0.02)
            else:
                lat.step(12, Jex=0.0, gamma=0.0)
            ref = lat.get_state()
            dref = lat.diagnostics()
            if m == 2:
                sref = lat.spectrum("B", "log", 8)
        np.testing.assert_array_equal(got[m], ref)
        np.testing.assert_allclose(dg[m], dref, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(sp["mean"], sref["mean"], rtol=1e-12)


def test_member_tilings_and_redrive_between_steps():
    """Per-member launch shapes (as the autotuner sets them), a drive changed
    between steps (the step graph is captured again) and state set between
    steps: every member equals a single lattice run the same way."""
    ps = _members()
    ys = _states(ps)
    tiles = [(8, 16, 2, 1), (16, 8, 0, 1), (32, 4, 2, 0), (64, 2, 2, 1)]
    with ewpt.Ensemble(ps) as ens:
        for m, (y, t) in enumerate(zip(ys, tiles)):
            ens.set_state(m, y)
            ens.set_member_tiling(m, *t)
        ens.step(4)
        ens.set_drive(0, 0.04, 0.01)
        ens.step(3)
        ens.set_state(3, ys[3])
        ens.step(2)
        got = [ens.get_state(m) for m in range(len(ps))]
    for m, (p, y, t) in enumerate(zip(ps, ys, tiles)):
        with ewpt.Lattice(p) as lat:
            lat.set_state(y)
            lat.set_tiling(*t)
            lat.step(4, Jex=0.0, gamma=0.0)
            lat.step(3, Jex=0.04 if m == 0 else 0.0, gamma=0.01 if m == 0 else 0.0)
            if m == 3:
                lat.set_state(y)
            lat.step(2, Jex=0.04 if m == 0 else 0.0, gamma=0.01 if m == 0 else 0.0)
            np.testing.assert_array_equal(got[m], lat.get_state())


def test_ensemble_rejects_bad_members():
    p = ewpt.baseline_couplings(N=16, precision=ewpt.FP64)
    with pytest.raises(ewpt.EwptError):
        ewpt.Ensemble([p])
    with pytest.raises(ewpt.EwptError):
        ewpt.Ensemble([ewpt.baseline_couplings(N=16, precision=ewpt.FP32), p])


def test_ensemble_rejects_bad_tiling():
    ps = [ewpt.baseline_couplings(N=n, precision=ewpt.FP32) for n in (16, 20)]
    with ewpt.Ensemble(ps) as ens:
        # (bx, by, pair): partial warp, more than 128 threads, pair 2
        for t in [(8, 3, 1), (32, 8, 1), (32, 4, 2)]:
            with pytest.raises(ewpt.EwptError):
                ens.set_tiling(*t)
        for m, t in [(0, (32, 4, 4, 2)), (1, (16, 8, 3, 1)), (2, (16, 8, 2, 1))]:
            with pytest.raises(ewpt.EwptError):
                ens.set_member_tiling(m, *t)  # TMA tiles, register variant 3, member out of range
        ens.set_tiling(16, 8, 1)
        ens.set_member_tiling(1, 8, 16, 2, 1)
        ens.step(1)
        ens.sync()
