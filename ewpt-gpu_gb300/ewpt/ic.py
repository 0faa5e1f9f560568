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

try:  # multithreaded FFTs when scipy is present (same pocketfft algorithm)
    import scipy.fft as _sfft

    def _fftn(a):
        return _sfft.fftn(a, workers=-1)

    def _ifftn(a):
        return _sfft.ifftn(a, workers=-1)
except ImportError:  # pragma: no cover
    _fftn, _ifftn = np.fft.fftn, np.fft.ifftn


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


def tanh_bubble_list(shape, dx, nbub, seed=0) -> np.ndarray:
    """(nbub, 7): seeded uniform centres (physical units) and directions
    uniform on S^3 -- the draws of bubbles_tanh, for ewpt_init_bubbles."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    L = np.array([nx * dx, ny * dx, nz * dx])
    centres = rng.random((nbub, 3)) * L
    dirs = rng.normal(size=(nbub, 4))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    return np.ascontiguousarray(np.hstack([centres, dirs]))


def tanh_profile_params(lam=0.129, vev=1.0, radius=None, width=None):
    """(R, w) of the benchmark bubble profile: R = 2/sqrt(lam), w = 1/(sqrt(lam) vev)."""
    R = 2.0 / math.sqrt(lam) if radius is None else radius
    w = 1.0 / (math.sqrt(lam) * vev) if width is None else width
    return R, w


def bubbles_tanh(shape, dx, nbub, lam=0.129, vev=1.0, seed=0, radius=None, width=None):
    """Benchmark bubble IC: nbub seeded bubbles, tanh core of radius 2/sqrt(lam)."""
    R, w = tanh_profile_params(lam, vev, radius, width)
    nx, ny, nz = shape
    L = np.array([nx * dx, ny * dx, nz * dx])
    bl = tanh_bubble_list(shape, dx, nbub, seed)
    centres, dirs = bl[:, :3], bl[:, 3:]
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


# ----------------------------------------------------------------- thermal
def _kgrid(shape, dx):
    """Per-axis lattice wave numbers theta = 2 pi n / N (n the wrapped FFT index)."""
    return [2.0 * np.pi * np.fft.fftfreq(n) for n in shape]


def _deriv_symbol(theta, dx):
    """Fourier symbol s(theta) of the 6th-order first derivative
    (diff_scheme.jl:157-233): d/dx e^{i k x} = i s e^{i k x}."""
    return (90.0 * np.sin(theta) - 18.0 * np.sin(2 * theta) + 2.0 * np.sin(3 * theta)) / (60.0 * dx)


def _real_field(rng, amp, shape):
    """real(bfft(amp * (r + i r')))/1 with r, r' ~ N(0, sqrt 2) per mode, the
    construction of main_rk4.jl:5352-5600 (unnormalised backward FFT)."""
    z = amp * (rng.normal(0.0, math.sqrt(2.0), amp.shape) + 1j * rng.normal(0.0, math.sqrt(2.0), amp.shape))
    return np.real(_ifftn(z) * z.size)


def _grad(f, sym):
    F = _fftn(f)
    return [np.real(_ifftn(1j * s * F)) for s in sym]


def _div(fx, fy, fz, sym):
    out = 0
    for f, s in zip((fx, fy, fz), sym):
        out = out + _fftn(f) * (1j * s)
    return np.real(_ifftn(out))


def thermal(shape, dx, T=1.5, lam=0.129, gw=0.65, gy=0.35, vev=1.0, seed=0, mH=None, mW=None,
            gauss_iters=20, with_momenta=True):
    """Thermal initial condition of the precision configuration (thermal IC, T = 1.5 vev).

    Gaussian random Higgs and gauge modes with Bose-Einstein occupation
    n(w) = 1/(exp(w/T) - 1): Higgs w^2 = k^2 + mH^2 (mH = sqrt(2 lambda) vev),
    gauge w^2 = k^2 + mW^2 (mW = g vev/2) with two transverse polarisations
    (thermal_initializer_phi!/gauge!, main_rk4.jl:5029-5152: field amplitude
    sqrt(n/(w V)), real part of the unnormalised backward FFT), with
    k^2 = sum_i 2(1 - cos(k_i dx))/dx^2.  Momenta get amplitude sqrt(n w / V)
    (the reference leaves them zero) and the electric fields are then
    projected onto the discrete Gauss law d_i E^a_i = rho^a,
    d_i E_i(Y) = rho_Y, with the 6th-order derivative's Fourier symbol and a
    fixed-point iteration over the E-dependent SU(2) charge.  Gamma_a =
    d_i W^a_i and Sigma = d_i Y_i.  The zero mode of rho (total charge)
    cannot be projected out on a periodic box and remains."""
    rng = np.random.default_rng(seed)
    shape = tuple(shape)
    nx, ny, nz = shape
    mH = math.sqrt(2.0 * lam) * vev if mH is None else mH
    mW = gw * vev / 2.0 if mW is None else mW
    # numpy arrays in (z, y, x) order so that ravel() is the Julia layout
    th = _kgrid((nz, ny, nx), dx)
    TZ, TY, TX = np.meshgrid(*th, indexing="ij")
    k2 = 2.0 * ((1 - np.cos(TX)) + (1 - np.cos(TY)) + (1 - np.cos(TZ))) / dx ** 2
    vol = nx * ny * nz * dx ** 3

    def occ(w):
        with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
            n = 1.0 / np.expm1(w / T)
        return np.where(w > 0, n, 0.0)

    wH = np.sqrt(k2 + mH ** 2)
    wW = np.sqrt(k2 + mW ** 2)
    nH, nW = occ(wH), occ(wW)
    aH = np.sqrt(nH / (wH * vol))
    pH = np.sqrt(nH * wH / vol)
    with np.errstate(divide="ignore", invalid="ignore"):
        aW = np.where(wW > 0, np.sqrt(nW / (wW * vol)), 0.0)
        pW = np.sqrt(nW * wW / vol)
    zero = (k2 == 0)
    aW[zero] = 0.0
    pW[zero] = 0.0
    # transverse polarisations from the lattice momentum (2 sin(theta/2)/dx)
    kv = [2.0 * np.sin(0.5 * t) / dx for t in (TX, TY, TZ)]

    def transverse(amp):
        r = [rng.normal(0.0, math.sqrt(2.0), amp.shape) for _ in range(3)]
        e1 = [r[1] * kv[2] - r[2] * kv[1], r[2] * kv[0] - r[0] * kv[2], r[0] * kv[1] - r[1] * kv[0]]
        n1 = np.sqrt(sum(c * c for c in e1))
        n1[n1 == 0] = 1.0
        e1 = [c / n1 for c in e1]
        e2 = [e1[1] * kv[2] - e1[2] * kv[1], e1[2] * kv[0] - e1[0] * kv[2], e1[0] * kv[1] - e1[1] * kv[0]]
        n2 = np.sqrt(sum(c * c for c in e2))
        n2[n2 == 0] = 1.0
        e2 = [c / n2 for c in e2]
        xs = [rng.normal(0.0, math.sqrt(2.0), amp.shape) + 1j * rng.normal(0.0, math.sqrt(2.0), amp.shape)
              for _ in range(2)]
        comps = []
        for i in range(3):
            z = amp * (e1[i] * xs[0] + e2[i] * xs[1])
            comps.append(np.real(_ifftn(z) * z.size))
        return comps

    S = nx * ny * nz
    y = np.zeros((36, S))
    for a in range(4):
        y[a] = _real_field(rng, aH, (nz, ny, nx)).ravel()
        if with_momenta:
            y[20 + a] = _real_field(rng, pH, (nz, ny, nx)).ravel()
    for a in range(3):
        W = transverse(aW)
        for i in range(3):
            y[4 + 3 * a + i] = W[i].ravel()
        if with_momenta:
            E = transverse(pW)
            for i in range(3):
                y[24 + 3 * a + i] = E[i].ravel()
    aY = np.sqrt(np.where(k2 > 0, occ(np.sqrt(k2)) / np.where(k2 > 0, np.sqrt(k2) * vol, 1.0), 0.0))
    pY = np.sqrt(np.where(k2 > 0, occ(np.sqrt(k2)) * np.sqrt(k2) / vol, 0.0))
    Yc = transverse(aY)
    for i in range(3):
        y[13 + i] = Yc[i].ravel()
    if with_momenta:
        Ec = transverse(pY)
        for i in range(3):
            y[33 + i] = Ec[i].ravel()
    sym = [_deriv_symbol(t, dx) for t in (TX, TY, TZ)]
    # auxiliaries consistent with the gauge fields
    for a in range(3):
        y[16 + a] = _div(*[y[4 + 3 * a + i].reshape(nz, ny, nx) for i in range(3)], sym).ravel()
    y[19] = _div(*[y[13 + i].reshape(nz, ny, nx) for i in range(3)], sym).ravel()
    if with_momenta:
        gauss_project(y, shape, dx, gw, gy, iters=gauss_iters, sym=sym)
    return y


def thermal_from_deviates(shape, dx, T, mH, mW, deviates, one_based=True) -> np.ndarray:
    """The reference's thermal IC from given random draws (run()'s thermal
    branch, main_rk4.jl:5348-5636, with thermal_initializer_gauge! and
    thermal_initializer_phi!, :5029-5152); the host twin of
    ewpt_init_thermal_deviates.  deviates: (44, S) in run()'s draw order --
    for W^1, W^2, W^3, Y the arrays r_1, r_2, r_3, r_1_i, r_2_i, r_3_i, x_1..x_4,
    then phi_1_k .. phi_4_k.  one_based: theta = 2 pi (index + 1) / N per axis
    as the reference indexes its modes (else the FFT frequency).  Gamma,
    Sigma and the momenta stay zero, as in run()."""
    nx, ny, nz = shape
    S = nx * ny * nz
    dv = np.asarray(deviates, dtype=np.float64).reshape(44, nz, ny, nx)
    idx = [np.arange(n) for n in (nz, ny, nx)]
    if one_based:
        th = [2.0 * math.pi * (i + 1) / n for i, n in zip(idx, (nz, ny, nx))]
    else:
        th = [2.0 * math.pi * np.where(i < (n + 1) // 2, i, i - n) / n for i, n in zip(idx, (nz, ny, nx))]
    TZ, TY, TX = np.meshgrid(*th, indexing="ij")
    k2 = 2.0 * ((1 - np.cos(TX)) + (1 - np.cos(TY)) + (1 - np.cos(TZ))) / dx ** 2
    kv = [2.0 * np.sin(0.5 * t) / dx for t in (TX, TY, TZ)]
    vol = S * dx ** 3

    def amp(m, empty_k0):
        w = np.sqrt(k2 + m * m)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            a = np.where(w > 0, np.sqrt(1.0 / np.expm1(w / T) / (w * vol)), 0.0)
        if empty_k0:
            a = np.where(k2 == 0, 0.0, a)
        return a

    y = np.zeros((36, S))
    for g in range(4):
        d = dv[10 * g:10 * g + 10]
        r, x = d[0:3], d[6:10]
        e1 = [r[1] * kv[2] - r[2] * kv[1], r[2] * kv[0] - r[0] * kv[2], r[0] * kv[1] - r[1] * kv[0]]
        n1 = np.sqrt(sum(c * c for c in e1))
        n1[n1 == 0] = 1.0
        e1 = [c / n1 for c in e1]
        e2 = [e1[1] * kv[2] - e1[2] * kv[1], e1[2] * kv[0] - e1[0] * kv[2], e1[0] * kv[1] - e1[1] * kv[0]]
        n2 = np.sqrt(sum(c * c for c in e2))
        n2[n2 == 0] = 1.0
        e2 = [c / n2 for c in e2]
        a = amp(0.0 if g == 3 else mW, True)
        base = 13 if g == 3 else 4 + 3 * g
        for c in range(3):
            z = a * (e1[c] * x[0] + e2[c] * x[1]) + 1j * a * (e1[c] * x[2] + e2[c] * x[3])
            y[base + c] = np.real(_ifftn(z) * S).ravel()
    aH = amp(mH, False)
    for c in range(4):
        y[c] = np.real(_ifftn(aH * dv[40 + c]) * S).ravel()
    return y


def gauss_charges(y, gw, gy):
    """SU(2) and U(1) charge densities of main_rk4.jl:603-655 (the terms
    multiplying gp2 in k_Gamma_a and k_Sigma)."""
    p1, p2, p3, p4 = y[0], y[1], y[2], y[3]
    t1, t2, t3, t4 = y[20], y[21], y[22], y[23]
    W = [[y[4 + 3 * a + i] for i in range(3)] for a in range(3)]
    E = [[y[24 + 3 * a + i] for i in range(3)] for a in range(3)]
    hig = [p1 * t4 - p4 * t1 + p3 * t2 - p2 * t3, p3 * t1 - p1 * t3 + p4 * t2 - p2 * t4,
           p1 * t2 - p2 * t1 + p4 * t3 - p3 * t4]
    rho = []
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        q = -sum(W[b][i] * E[c][i] - W[c][i] * E[b][i] for i in range(3))
        rho.append(gw * q + gw * hig[a])
    rhoY = gy * (p1 * t2 - p2 * t1 + p3 * t4 - p4 * t3)
    return rho, rhoY


# phi^T M pi of the Higgs charges of k_Gamma_1..3 and k_Sigma (main_rk4.jl:603-655)
_CHARGE_PAIRS = [[(0, 3), (2, 1)], [(2, 0), (3, 1)], [(0, 1), (3, 2)], [(0, 1), (2, 3)]]


def _charge_matrix(a):
    M = np.zeros((4, 4))
    for i, j in _CHARGE_PAIRS[a]:
        M[i, j] = 1.0
        M[j, i] = -1.0
    return M


def _null_patterns(shape):
    """Staggered patterns (-1)^(e.x), e in {0,1}^3 (only e_i = 1 on even axes):
    the modes that the central-difference divergence cannot produce."""
    nx, ny, nz = shape
    i = np.arange(nx)
    j = np.arange(ny)
    k = np.arange(nz)
    pats = []
    for ez in (0, 1) if nz % 2 == 0 else (0,):
        for ey in (0, 1) if ny % 2 == 0 else (0,):
            for ex in (0, 1) if nx % 2 == 0 else (0,):
                P = ((-1.0) ** (ez * k))[:, None, None] * ((-1.0) ** (ey * j))[None, :, None] * \
                    ((-1.0) ** (ex * i))[None, None, :]
                pats.append(P.ravel())
    return pats


def _class_sums(f, shape):
    """Sums of f over the 8 parity classes (k % 2, j % 2, i % 2) of the sites."""
    nx, ny, nz = shape
    a = f.reshape(nz, ny, nx)
    return np.array([[[a[pz::2, py::2, px::2].sum() for px in (0, 1)] for py in (0, 1)] for pz in (0, 1)])


def _null_vectors(shape):
    """The e in {0,1}^3 (e_i = 1 only on even axes) of the staggered null
    patterns (-1)^(e.x), in the order of _null_patterns."""
    nx, ny, nz = shape
    return [(ez, ey, ex) for ez in ((0, 1) if nz % 2 == 0 else (0,)) for ey in ((0, 1) if ny % 2 == 0 else (0,))
            for ex in ((0, 1) if nx % 2 == 0 else (0,))]


def _moment(s, e):
    """sum_x (-1)^(e.x) f(x) from the parity-class sums s of f."""
    return sum((-1.0) ** (e[0] * pz + e[1] * py + e[2] * px) * s[pz, py, px]
               for pz in (0, 1) for py in (0, 1) for px in (0, 1))


def neutralize_charges(y, gw, gy, shape):
    """Shift the Higgs momenta along the four charge generators so that the
    charges have no component in the null modes of the central-difference
    divergence (the zero mode and the Nyquist corners, where d_i E_i is 0
    whatever E is): Gauss's law can only hold for such a charge density.

    Unknowns alpha[b, e]: pi += sum_b (sum_e alpha[b,e] (-1)^(e.x)) M_b^T phi.
    Since (-1)^(e.x) (-1)^(e'.x) = (-1)^((e^e').x), every coefficient of the
    linear system is a parity-class moment of one site field, so the system
    costs 16 + 4 passes over the lattice."""
    nx, ny, nz = shape
    rho, rhoY = gauss_charges(y, gw, gy)
    dens = list(rho) + [rhoY]
    coup = [gw, gw, gw, gy]
    es = _null_vectors(shape)
    ne = len(es)
    phi = y[0:4]
    Ms = [_charge_matrix(a) for a in range(4)]
    MT_phi = [M.T @ phi for M in Ms]
    n = 4 * ne
    A = np.zeros((n, n))
    Q = np.zeros(n)
    for a in range(4):
        sq = _class_sums(dens[a], shape)
        for pi_, e in enumerate(es):
            Q[a * ne + pi_] = _moment(sq, e)
        for b in range(4):
            g = coup[a] * np.sum(phi * (Ms[a] @ MT_phi[b]), axis=0)  # per-site phi^T M_a M_b^T phi
            sg = _class_sums(g, shape)
            for pi_, e in enumerate(es):
                for pj, e2 in enumerate(es):
                    A[a * ne + pi_, b * ne + pj] = _moment(sg, tuple(u ^ v for u, v in zip(e, e2)))
    alpha = np.linalg.lstsq(A, -Q, rcond=None)[0]
    # coefficient field of generator b: constant on each parity class
    cls = ((np.arange(nz) % 2)[:, None, None] * 4 + (np.arange(ny) % 2)[None, :, None] * 2 +
           (np.arange(nx) % 2)[None, None, :]).ravel()
    for b in range(4):
        table = np.zeros(8)
        for c in range(8):
            pz, py, px = c >> 2, (c >> 1) & 1, c & 1
            table[c] = sum(alpha[b * ne + pj] * (-1.0) ** (e[0] * pz + e[1] * py + e[2] * px)
                           for pj, e in enumerate(es))
        y[20:24] += table[cls] * MT_phi[b]
    return y


def gauss_project(y, shape, dx, gw, gy, iters=12, sym=None):
    """Project the electric fields onto d_i E_i = rho (in place), iterating
    over the E-dependent part of the SU(2) charge; each iteration first
    neutralises the total charges (neutralize_charges)."""
    nx, ny, nz = shape
    if sym is None:
        th = _kgrid((nz, ny, nx), dx)
        TZ, TY, TX = np.meshgrid(*th, indexing="ij")
        sym = [_deriv_symbol(t, dx) for t in (TX, TY, TZ)]
    s2 = sym[0] ** 2 + sym[1] ** 2 + sym[2] ** 2
    ok = s2 > 1e-12 * s2.max()
    for _ in range(iters):
        neutralize_charges(y, gw, gy, shape)
        rho, rhoY = gauss_charges(y, gw, gy)
        groups = [(24 + 3 * a, rho[a]) for a in range(3)] + [(33, rhoY)]
        for base, r in groups:
            Ex, Ey, Ez = (y[base + i].reshape(nz, ny, nx) for i in range(3))
            F = [_fftn(Ex), _fftn(Ey), _fftn(Ez)]
            res = 1j * (sym[0] * F[0] + sym[1] * F[1] + sym[2] * F[2]) - _fftn(r.reshape(nz, ny, nx))
            chi = np.where(ok, res / np.where(ok, -s2, 1.0), 0.0)
            for i in range(3):
                y[base + i] = np.real(_ifftn(F[i] - 1j * sym[i] * chi)).ravel()
    return y
