"""Initial conditions (host side, seeded with numpy's PCG64 generator).

The reference draws its initial conditions from Julia's global RNG with
unpinned package versions (gpu-kernels-rk4/main_rk4.jl:5348-5697), so its
random streams cannot be reproduced; these generators keep the reference's
construction with the project's own seeded RNG and write the full 36-array
state that every implementation (CPU oracle, FP64 and FP32 GPU forms) then
evolves from identical inputs.

  bubbles_reference  placement on the bub_diam sub-lattice sampled without
                     replacement (main_rk4.jl:5638-5658), direction from
                     gen_phi (convenients.jl:8-14), profile rmag(rb) with the
                     reference's sin-distance rb (initializer!, :4930-4946)
  bubbles_tanh       the benchmark configurations' IC: seeded uniform centres,
                     tanh wall 0.5*(1 - tanh((r - R)/w)) with R = 2/sqrt(lambda)
                     and w = 1/(sqrt(lambda) vev) (the kink width of
                     lambda(|Phi|^2 - v^2)^2), direction uniform on S^3
                     (Haar measure of the unit doublet), minimum-image r
"""
from __future__ import annotations

import math

import numpy as np

from .params import Params


def _grid(shape, dx):
    nx, ny, nz = shape
    i = np.arange(nx, dtype=np.float64)
    j = np.arange(ny, dtype=np.float64)
    k = np.arange(nz, dtype=np.float64)
    return i, j, k


def empty_state(shape) -> np.ndarray:
    return np.zeros((36, int(np.prod(shape))))


def gen_phi(a, b, c, sign):
    """gen_phi (convenients.jl:8-14) with the random sign drawn by the caller."""
    alpha = 0.5 * math.acos(sign * a)
    beta = b * 2.0 * math.pi
    gamma = c * 2.0 * math.pi
    z1 = complex(math.cos(alpha) * math.cos(beta), math.cos(alpha) * math.sin(beta))
    z2 = complex(math.sin(alpha) * math.cos(gamma), math.sin(alpha) * math.sin(gamma))
    return [z1.real, z1.imag, z2.real, z2.imag]


def rmag(rb, mH):
    """Bubble profile of initializer! (main_rk4.jl:4936)."""
    s2 = math.sqrt(2.0)
    return (1.0 + (s2 - 1.0) ** 2) * np.exp(-mH * rb / s2) / (1.0 + ((s2 - 1.0) ** 2) * np.exp(-s2 * mH * rb))


def bubble_reference_field(shape, dx, centre, direction, mH) -> np.ndarray:
    """phi contribution (4, S) of one bubble, initializer! (main_rk4.jl:4930-4946);
    centre is the reference's 1-based (ib, jb, kb)."""
    nx, ny, nz = shape
    rkx, rky, rkz = (math.pi / ((n - 1) * dx) for n in shape)
    i, j, k = _grid(shape, dx)
    sx = np.sin(rkx * (i - (centre[0] - 0.5)) * dx) ** 2 / rkx ** 2
    sy = np.sin(rky * (j - (centre[1] - 0.5)) * dx) ** 2 / rky ** 2
    sz = np.sin(rkz * (k - (centre[2] - 0.5)) * dx) ** 2 / rkz ** 2
    rb = np.sqrt(sz[:, None, None] + sy[None, :, None] + sx[None, None, :]).ravel()
    r = rmag(rb, mH)
    return np.stack([r * d for d in direction])


def bubbles_reference(p: Params, nbub: int | None = None, seed: int | None = None) -> np.ndarray:
    """Reference bubble-nucleation IC (main_rk4.jl:5638-5697) with a numpy RNG."""
    shape = p.dims
    nbub = p.no_bubbles if nbub is None else nbub
    rng = np.random.default_rng(p.base_seed if seed is None else seed)
    bd = p.bub_diam
    xs = range(bd, shape[0] + 1, bd)
    ys = range(bd, shape[1] + 1, bd)
    zs = range(bd, shape[2] + 1, bd)
    coords = [(a, b, c) for a in xs for b in ys for c in zs]
    if nbub > len(coords):
        raise ValueError(f"{nbub} bubbles do not fit the {len(coords)}-point placement sub-lattice")
    pick = rng.choice(len(coords), size=nbub, replace=False)
    hoft = rng.random((nbub, 3))
    signs = rng.choice([-1.0, 1.0], size=nbub)
    y = empty_state(shape)
    for b in range(nbub):
        d = gen_phi(*hoft[b], signs[b])
        y[:4] += bubble_reference_field(shape, p.dx, coords[pick[b]], d, p.mH)
    return y


def bubbles_tanh(shape, dx, nbub, lam=0.129, vev=1.0, seed=0, radius=None, width=None):
    """Benchmark bubble IC: nbub seeded bubbles, tanh core of radius 2/sqrt(lam)."""
    rng = np.random.default_rng(seed)
    R = 2.0 / math.sqrt(lam) if radius is None else radius
    w = 1.0 / (math.sqrt(lam) * vev) if width is None else width
    nx, ny, nz = shape
    L = np.array([nx * dx, ny * dx, nz * dx])
    centres = rng.random((nbub, 3)) * L
    dirs = rng.normal(size=(nbub, 4))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    x = np.arange(nx) * dx
    yv = np.arange(ny) * dx
    z = np.arange(nz) * dx
    y = empty_state(shape)
    for b in range(nbub):
        ddx = x - centres[b, 0]
        ddx -= L[0] * np.round(ddx / L[0])
        ddy = yv - centres[b, 1]
        ddy -= L[1] * np.round(ddy / L[1])
        ddz = z - centres[b, 2]
        ddz -= L[2] * np.round(ddz / L[2])
        r = np.sqrt(ddz[:, None, None] ** 2 + ddy[None, :, None] ** 2 + ddx[None, None, :] ** 2).ravel()
        prof = vev * 0.5 * (1.0 - np.tanh((r - R) / w))
        for a in range(4):
            y[a] += dirs[b, a] * prof
    return y
