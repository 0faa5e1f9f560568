"""The bounded device-side waits run out safely.

Every mbarrier wait in libewpt's kernels has an iteration limit.  These
tests set the limit to zero polls, so the first wait in the TMA-staged FP32
stage kernel (its copy ring) and in the MLP's tensor-core GEMM (the MMA
commit) gives up at once: the kernels stop their copies or MMAs, wait for
what is already in flight with the full limit, and return; the host sees
EWPT_ERR_TIMEOUT.  The same context or net then runs normally and matches
its reference (the paired FP32 kernel bit for bit; the MLP oracle).  No
fault, trap or hang is involved: the limit is a host-set number."""
import numpy as np
import pytest

import ewpt
from ewpt import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build_lib

    build_lib.build()


def test_tma_ring_wait_runs_out_and_context_recovers():
    shape = (64, 32, 32)
    p = ewpt.baseline_couplings(shape=shape, N=64, dx=0.25, dt=0.025, precision=ewpt.FP32)
    y0 = ewpt.ic.bubbles_tanh(shape, p.dx, 4, seed=3)
    y0[20:] = 0.05 * np.random.default_rng(2).normal(size=(16, y0.shape[1]))
    with ewpt.Lattice(p) as ref:
        ref.set_state(y0)
        ref.set_tiling(32, 4, 0, 1)  # the paired kernel: the TMA kernel's arithmetic
        ref.step(3)
        y_ref = ref.get_state()
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        lat.set_tiling(32, 4, 4, 2)
        lat.set_wait_limit(0)
        lat.step(1)
        with pytest.raises(_lib.EwptError) as ei:
            lat.sync()
        assert ei.value.code == _lib.ERR_TIMEOUT
        # the context is usable again: default limit, fresh state, same result as the paired kernel
        lat.set_wait_limit(-1)
        lat.set_state(y0)
        lat.step(3)
        lat.sync()
        np.testing.assert_array_equal(lat.get_state(), y_ref)


def test_mlp_tensor_core_wait_runs_out_and_net_recovers():
    from ewpt.surrogate import MLP
    from oracle import mlp_oracle as mo

    n_in, width, n_out, B = 84, 256, 40, 37
    rng = np.random.default_rng(9)
    x = rng.normal(size=(B, n_in)).astype(np.float32)
    net = MLP(n_in, width, n_out, max_batch=64, seed=4)
    try:
        p = net.get_params()
        net.set_wait_limit(0)
        with pytest.raises(_lib.EwptError) as ei:
            net.forward(x)
        assert ei.value.code == _lib.ERR_TIMEOUT
        net.set_wait_limit(-1)
        got = net.forward(x)
        ref = mo.forward(p.astype(np.float64), x.astype(np.float64), n_in, width, n_out)["z3"]
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 2e-3
    finally:
        net.close()
