"""CPU FP64 restatement of the surrogate MLP's forward and backward pass.

TEST INFRASTRUCTURE ONLY (the checker of ewpt_mlp_gradients /
ewpt_mlp_forward).  Rounds to bfloat16 at exactly the points where the GPU
path feeds the tensor cores (inputs, weights, activations, back-propagated
gradients) and accumulates in FP64, so the GPU result differs from this one
only by FP32 accumulation order and the rare bfloat16 rounding flip that
order causes.

Network: x -> Linear(n_in, width) -> GELU -> Linear(width, width) -> GELU ->
Linear(width, n_out); loss = mean((z3 - y)^2).  Parameters flattened as
W1 [width][n_in], b1, W2 [width][width], b2, W3 [n_out][width], b3.
"""
from __future__ import annotations

import math

import numpy as np


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    if nan.any():
        out[nan] = np.nan
    return out


def _erf(x):
    v = np.vectorize(math.erf)
    return v(x)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def unpack(params, n_in, width, n_out):
    p = np.asarray(params, dtype=np.float64)
    o = 0
    out = []
    for shape in [(width, n_in), (width,), (width, width), (width,), (n_out, width), (n_out,)]:
        n = int(np.prod(shape))
        out.append(p[o:o + n].reshape(shape))
        o += n
    return out


def forward(params, x, n_in, width, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(params, n_in, width, n_out)
    x0 = bf16(x)
    z1 = x0 @ bf16(W1).T + b1
    a1 = bf16(gelu(z1))
    z2 = a1 @ bf16(W2).T + b2
    a2 = bf16(gelu(z2))
    z3 = a2 @ bf16(W3).T + b3
    return dict(x0=x0, z1=z1, a1=a1, z2=z2, a2=a2, z3=z3)


def gradients(params, x, y, n_in, width, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(params, n_in, width, n_out)
    f = forward(params, x, n_in, width, n_out)
    B = x.shape[0]
    d3 = 2.0 * (f["z3"] - y) / (B * n_out)
    loss = float(np.mean((f["z3"] - y) ** 2))
    d3b = bf16(d3)
    gW3 = d3b.T @ f["a2"]
    gb3 = d3.sum(axis=0)
    da2 = d3b @ bf16(W3)
    d2 = da2 * gelu_grad(f["z2"])
    d2b = bf16(d2)
    gW2 = d2b.T @ f["a1"]
    gb2 = d2.sum(axis=0)
    da1 = d2b @ bf16(W2)
    d1 = da1 * gelu_grad(f["z1"])
    d1b = bf16(d1)
    gW1 = d1b.T @ f["x0"]
    gb1 = d1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return g, loss
