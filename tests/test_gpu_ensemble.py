"""Batched ensemble (FP32 form): each member of a mixed-size ensemble evolves
like a single FP32-form lattice with the same packed/scalar mode (bit for
bit in packed mode, FP32 round-off in scalar mode), diagnostics and spectra
of members match single contexts."""
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
            lat.set_tiling(32, 4, 0, pair)
            if m == 1:
                lat.step(12, Jex=0.05, gamma=0.02)
            else:
                lat.step(12, Jex=0.0, gamma=0.0)
            ref = lat.get_state()
            dref = lat.diagnostics()
            if m == 2:
                sref = lat.spectrum("B", "log", 8)
        if pair:
            np.testing.assert_array_equal(got[m], ref)
        else:
            # one site per thread: the two kernels contract a*b + c into FMAs
            # at different places, so FP32 round-off differs (and grows)
            scale = np.maximum(np.abs(ref).max(axis=1, keepdims=True), 1e-30)
            assert (np.abs(got[m] - ref) / scale).max() < 1e-4
        np.testing.assert_allclose(dg[m], dref, rtol=1e-5 if not pair else 1e-12, atol=1e-12)
    np.testing.assert_allclose(sp["mean"], sref["mean"], rtol=1e-5 if not pair else 1e-12)


def test_ensemble_rejects_bad_members():
    p = ewpt.baseline_couplings(N=16, precision=ewpt.FP64)
    with pytest.raises(ewpt.EwptError):
        ewpt.Ensemble([p])
    # members index their [36][S] block with 32-bit offsets: 36 S < 2^31
    big = ewpt.baseline_couplings(N=392, precision=ewpt.FP32)
    with pytest.raises(ewpt.EwptError, match="2\\^31"):
        ewpt.Ensemble([ewpt.baseline_couplings(N=16, precision=ewpt.FP32), big])


def test_ensemble_rejects_bad_tiling():
    ps = [ewpt.baseline_couplings(N=n, precision=ewpt.FP32) for n in (16, 20)]
    with ewpt.Ensemble(ps) as ens:
        # (bx, by, pair): partial warp, more than 128 threads, pair 2
        for t in [(8, 3, 1), (32, 8, 1), (32, 4, 2)]:
            with pytest.raises(ewpt.EwptError):
                ens.set_tiling(*t)
        ens.set_tiling(16, 8, 1)
        ens.step(1)
        ens.sync()
