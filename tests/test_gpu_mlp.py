"""The surrogate's tensor-core MLP kernels against the CPU FP64 oracle
(oracle/mlp_oracle.py, bfloat16 rounding emulated at the GPU's points):
forward outputs and every parameter gradient, then a training run."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

N_IN, WIDTH, N_OUT = 84, 256, 40


@pytest.fixture(scope="module")
def net():
    import build_lib

    build_lib.build()
    from ewpt.surrogate import MLP

    m = MLP(N_IN, WIDTH, N_OUT, max_batch=256, seed=3)
    yield m
    m.close()


def _data(B, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(B, N_IN)).astype(np.float32)
    y = rng.normal(size=(B, N_OUT)).astype(np.float32)
    return x, y


def _blocks(v):
    sizes = [WIDTH * N_IN, WIDTH, WIDTH * WIDTH, WIDTH, N_OUT * WIDTH, N_OUT]
    out, o = [], 0
    for s in sizes:
        out.append(v[o:o + s])
        o += s
    return out


@pytest.mark.parametrize("B", [1, 37, 200])
def test_forward_matches_oracle(net, B):
    x, _ = _data(B, B)
    p = net.init_params(seed=B)
    net.set_params(p)
    got = net.forward(x)
    ref = mo.forward(p.astype(np.float64), x.astype(np.float64), N_IN, WIDTH, N_OUT)["z3"]
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 2e-3


@pytest.mark.parametrize("B", [16, 129])
def test_gradients_match_oracle(net, B):
    x, y = _data(B, 100 + B)
    p = net.init_params(seed=7 + B)
    net.set_params(p)
    g, loss = net.gradients(x, y)
    gr, lr_ = mo.gradients(p.astype(np.float64), x.astype(np.float64), y.astype(np.float64), N_IN, WIDTH, N_OUT)
    assert abs(loss - lr_) < 1e-3 * lr_
    for name, a, b in zip(["W1", "b1", "W2", "b2", "W3", "b3"], _blocks(g), _blocks(gr)):
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err < 2e-2, (name, err)


def test_training_reduces_loss(net):
    rng = np.random.default_rng(5)
    x = rng.normal(size=(256, N_IN)).astype(np.float32)
    w = rng.normal(size=(N_IN, N_OUT)) / np.sqrt(N_IN)
    y = np.tanh(x @ w).astype(np.float32)
    net.set_params(net.init_params(seed=1))
    losses = [net.train_step(x, y, 2e-3, 0.0) for _ in range(300)]
    assert losses[-1] < 0.1 * losses[0]
    assert np.isfinite(net.get_params()).all()
