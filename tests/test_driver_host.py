"""Host logic of the driver's reference-format outputs (ewpt.run), with a
stand-in for the device lattice: the y-slices follow main_rk4.jl:5700-5960
(plane j = Ny/2 in Julia's 1-based numbering, PE, KE, GE, MEW+EEW+MEY+EEY,
B_x+B_y+B_z, B2_x+B2_y+B2_z, zeros, times dx^3), the FFT dump holds fft(E_t)
over the Julia axes, and the cadence parameters follow parameters.jl."""
import numpy as np

import ewpt
from ewpt import run as drv
from ewpt.lattice import julia_array


class FakeLattice:
    def __init__(self, p, seed=0):
        rng = np.random.default_rng(seed)
        self.f = {"density": rng.normal(size=(7, p.sites)), "B": rng.normal(size=(3, p.sites)),
                  "B2": rng.normal(size=(3, p.sites))}

    def fields(self, name):
        return self.f[name]


def test_y_slices_follow_the_reference_layout():
    p = ewpt.Params(shape=(6, 8, 5), N=6, dx=0.5)
    lat = FakeLattice(p)
    s = drv.y_slices(lat, p)
    assert s.shape == (7, 6, 5)
    nx, ny, nz = p.dims
    vol = p.dx ** 3
    d, b, b2 = lat.f["density"], lat.f["B"], lat.f["B2"]

    def ref_plane(row):  # E_t[:, Ny÷2, :] with Julia's 1-based index Ny÷2 = 4
        a = np.asarray(row).reshape(nz, ny, nx)  # [k, j, i], x fastest
        return a[:, ny // 2 - 1, :].T * vol  # -> [i, k]

    np.testing.assert_array_equal(s[0], ref_plane(d[0]))
    np.testing.assert_array_equal(s[2], ref_plane(d[2]))
    np.testing.assert_array_equal(s[3], ((ref_plane(d[4]) + ref_plane(d[3])) + ref_plane(d[6])) + ref_plane(d[5]))
    np.testing.assert_array_equal(s[4], (ref_plane(b[0]) + ref_plane(b[1])) + ref_plane(b[2]))
    np.testing.assert_array_equal(s[5], (ref_plane(b2[0]) + ref_plane(b2[1])) + ref_plane(b2[2]))
    assert not s[6].any()


def test_fft_dump_is_the_julia_axes_fft():
    p = ewpt.Params(shape=(6, 4, 5), N=6)
    lat = FakeLattice(p, seed=3)
    out = drv.b_fft_dump(lat, p)
    assert sorted(out) == sorted(["3D_fft_x", "3D_fft_y", "3D_fft_z", "3D_fft_x2", "3D_fft_y2", "3D_fft_z2"])
    for name, field, c in (("3D_fft_y", "B", 1), ("3D_fft_z2", "B2", 2)):
        a = out[name]
        assert a.shape == p.dims and a.flags["F_CONTIGUOUS"]
        # F[kx, ky, kz] = sum_{x,y,z} f[x, y, z] exp(-2 pi i (kx x / nx + ...))
        f = julia_array(lat.f[field][c], p.dims)
        x, y, z = (np.arange(n) for n in p.dims)
        kx, ky, kz = 1, 2, 3
        ph = np.exp(-2j * np.pi * (kx * x[:, None, None] / p.dims[0] + ky * y[None, :, None] / p.dims[1]
                                   + kz * z[None, None, :] / p.dims[2]))
        assert abs(a[kx, ky, kz] - (f * ph).sum()) < 1e-10 * np.abs(f).sum()


def test_julia_array_is_column_major():
    row = np.arange(24.0)
    a = julia_array(row, (2, 3, 4))
    assert a[1, 0, 0] == 1.0 and a[0, 1, 0] == 2.0 and a[0, 0, 1] == 6.0


def test_cadence_parameters():
    p = ewpt.Params.from_args(["0.0", "10", "2000", "0.25", "10", "256", "0.99", "20", "0.0", "0.0", "0.0", "1"])
    assert p.dsnaps == 100 and p.dsnaps_fft == 40 and p.spec_cut == (64, 64, 64)
    q = ewpt.Params.from_args(["0.0", "10", "30", "0.25", "10", "32", "0.99", "4", "0.0", "0.0", "0.0", "1"])
    assert q.dsnaps == 7 and q.dsnaps_fft == 1  # floor(30/50) = 0 -> every snapshot


def test_surrogate_parameter_draws():
    """Seeded draws: features (lambda, g, g', bubble count[, T][, log2 N]);
    thermal runs carry bubble count 0 and T in [1, 2]; a single size keeps
    the four-feature layout."""
    import numpy as np

    from ewpt import surrogate

    ps, prm, nb = surrogate.draw_members(200, [64, 96, 128], seed=3, thermal_fraction=0.5)
    assert prm.shape == (200, 6) and len(ps) == 200
    th = prm[:, 4] > 0
    assert 60 < th.sum() < 140
    assert (prm[th, 3] == 0).all() and (nb[th] == 0).all() and ((prm[th, 4] >= 1) & (prm[th, 4] <= 2)).all()
    assert (prm[~th, 3] >= 4).all() and (prm[~th, 3] <= 16).all()
    assert set(prm[:, 5]) <= {6.0, np.log2(96), 7.0}
    assert [p.dims[0] for p in ps] == [int(round(2 ** v)) for v in prm[:, 5]]
    ps2, prm2, _ = surrogate.draw_members(200, [64, 96, 128], seed=3, thermal_fraction=0.5)
    np.testing.assert_array_equal(prm, prm2)
    _, prm1, _ = surrogate.draw_members(10, 24, seed=1)
    assert prm1.shape == (10, 4)


def test_step_host_buffer_checks():
    """Lattice.step_host takes (36, S) C-contiguous float64 host buffers,
    numpy or CPU torch, and refuses anything else before any library call."""
    import pytest
    import torch

    from ewpt.lattice import Lattice

    lat = Lattice.__new__(Lattice)  # no device context: only the checks run
    lat.S = 12
    good = [np.zeros((36, 12)), torch.zeros((36, 12), dtype=torch.float64)]
    for buf in good:
        assert Lattice._host_state_ptr(lat, buf, "state_in") != 0
    bad = [np.zeros((36, 12), np.float32), np.zeros((36, 11)), np.zeros((12, 36)).T,
           torch.zeros((36, 12)), torch.zeros((36, 24), dtype=torch.float64)[:, ::2], [0.0] * 432]
    for buf in bad:
        with pytest.raises(ValueError, match="state_in"):
            Lattice._host_state_ptr(lat, buf, "state_in")
    ro = np.zeros((36, 12))
    ro.flags.writeable = False
    with pytest.raises(ValueError, match="writeable"):
        lat.step_host(np.zeros((36, 12)), ro, 1)
