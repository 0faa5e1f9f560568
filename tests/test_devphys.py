"""The stage kernels' own per-site arithmetic (csrc/physics.cuh over
csrc/accessors.cuh), compiled for the host by oracle/devphys.cu, against
the golden rates of the reference's rk4_step! and against the oracle; and
the exact FP64 operation count that bench.py's compute roofline uses.

These run on the CPU: a change to the physics is checked here before it
reaches a GPU, where tests/test_gpu_parity.py repeats the comparison through
the C ABI with FMA contraction."""
import os

import numpy as np
import pytest

from oracle import devphys
from oracle import oracle as orc

TOL = 1e-12  # relative to max |rate| per array, as the GPU rates test


def _coef(g):
    return (float(g["p_gw"]), float(g["p_gy"]), float(g["p_gp2"]), float(g["p_lambda"]), float(g["p_vev"]),
            float(g["p_beta_w"]), float(g["p_beta_y"]), float(g["p_dx"]))


def _close(r, ref):
    scale = np.maximum(np.abs(ref).max(axis=1, keepdims=True), 1e-300)
    return float((np.abs(r - ref) / scale).max())


@pytest.mark.parametrize("case", ["a", "b"])
def test_kernel_physics_matches_golden_rates(golden_dir, case):
    g = dict(np.load(os.path.join(golden_dir, f"ref_{case}.npz")))
    shape = tuple(int(v) for v in g["shape"])
    r = devphys.rates(shape, _coef(g), g["y0"], float(g["Jex"]), float(g["gam"]))
    assert _close(r, g["rates"]) < TOL


@pytest.mark.parametrize("beta", [False, True])
def test_kernel_physics_matches_oracle(beta):
    shape = (12, 10, 14)
    S = int(np.prod(shape))
    rng = np.random.default_rng(11)
    y = rng.normal(size=(36, S))
    y[:4] += 1.0  # |Phi| away from 0 (the damping term divides by it)
    bw, by = (0.3, -0.2) if beta else (0.0, 0.0)
    coef = (0.65, 0.35, 0.99, 0.129, 1.0, bw, by, 0.25)
    op = orc.params(shape, 0.25, 0.65, 0.35, 0.99, 0.129, 1.0, bw, by)
    ref = orc.rates(op, y, 0.7, 0.05)
    r = devphys.rates(shape, coef, y, 0.7, 0.05)
    assert _close(r, ref) < TOL


def test_operation_count_is_the_bench_figure():
    import bench

    c = devphys.count(beta=False)
    assert c["div_per_site_update"] == 4
    assert c["flops_per_site_update"] == bench.FLOPS_FP64
    assert c["fp64_inst_est_per_site_update"] == bench.FP64_INST_EST
    # the stencils: 16 gradient+Laplacians, 4 gradients, 4 divergences per site
    assert c["stencil_flops_per_stage"] == 16 * 46 + 4 * 24 + 4 * 26
