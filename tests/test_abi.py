"""CPU-only checks of the C ABI boundary: the library loads, exports every
symbol include/ewpt.h declares, and validates arguments before touching a
device (no compute calls here)."""
import ctypes as C
import math

import pytest

import ewpt
from ewpt import _lib


@pytest.fixture(scope="module")
def L():
    import build_lib

    build_lib.build()
    return _lib.load()


def test_exports_every_declared_symbol(L):
    names = _lib.declared_symbols()
    assert "ewpt_rk4_rates" in names and "ewpt_step" in names
    for n in names:
        assert hasattr(L, n), f"libewpt.so does not export {n}"


def test_params_default_matches_parameters_jl(L):
    p = _lib.EwptParams()
    assert L.ewpt_params_default(C.byref(p), 64) == 0
    assert (p.nx, p.ny, p.nz) == (64, 64, 64)
    assert p.gw == 0.65 and p.lam == 0.129 and p.vev == 1.0 and p.gp2 == 0.99
    assert abs(p.gy - 0.65 * math.tan(math.asin(math.sqrt(0.22)))) < 1e-15
    assert abs(p.mH - 2 * math.sqrt(0.129)) < 1e-15
    assert p.t_sat == 2.0


@pytest.mark.parametrize("field,val", [("nx", 6), ("nz", 0), ("dx", float("nan")), ("dt", -1.0),
                                       ("gw", float("inf")), ("precision", 7)])
def test_create_rejects_bad_params(L, field, val):
    p = _lib.EwptParams()
    L.ewpt_params_default(C.byref(p), 16)
    setattr(p, field, val)
    h = C.c_void_p()
    rc = L.ewpt_create(C.byref(p), C.byref(h))
    assert rc == _lib.ERR_ARG
    assert not h.value
    assert len(L.ewpt_last_error(None)) > 0


def test_null_pointers_rejected(L):
    assert L.ewpt_create(None, None) == _lib.ERR_ARG
    assert L.ewpt_step(None, 1) == _lib.ERR_ARG
    assert L.ewpt_diagnostics(None, None) == _lib.ERR_ARG
    assert L.ewpt_sync(None) == _lib.ERR_ARG
    assert L.ewpt_iteration(None) == -1
    assert L.ewpt_destroy(None) == 0
    p = _lib.EwptParams()
    L.ewpt_params_default(C.byref(p), 16)
    assert L.ewpt_rk4_rates(C.byref(p), None, None, 0.0, 0.0, None) == _lib.ERR_ARG


def test_kc_bin_nums_host(L):
    # spec_routines.jl:32-43 restated: distinct |K| on a c^3 wrapped index lattice
    from oracle import oracle as orc

    for c in [(2, 2, 2), (4, 4, 3), (8, 8, 8), (16, 16, 16)]:
        assert L.ewpt_kc_bin_nums(*c) == orc.lib().or_kc_bin_nums(*c)
    assert L.ewpt_kc_bin_nums(0, 1, 1) == -1


def test_field_components_host(L):
    assert [L.ewpt_field_components(f) for f in range(4)] == [3, 3, 4, 7]
    assert L.ewpt_field_components(4) == -1 and L.ewpt_field_components(-1) == -1
    assert L.ewpt_fields(None, 0, None, 0) == _lib.ERR_ARG


def test_h5_layout_reverses_julia_axes():
    """HDF5.jl writes a Julia array with reversed dimensions and the same
    memory; the converter writes the transpose of each Julia-axes array."""
    import numpy as np

    from ewpt import h5convert

    a = np.asfortranarray(np.arange(24.0).reshape(2, 3, 4))  # Julia A[x, y, z], column-major
    h = h5convert.julia_layout(a)
    assert h.shape == (4, 3, 2) and h.flags["C_CONTIGUOUS"]
    assert np.shares_memory(h, a) or np.array_equal(h.ravel(), a.ravel(order="F"))
    assert h[3, 2, 1] == a[1, 2, 3]
    s = np.float64(0.25)
    assert h5convert.julia_layout(s) == s


def test_h5convert_writes_reference_datasets(tmp_path):
    h5py = pytest.importorskip("h5py")
    import numpy as np

    from ewpt import h5convert

    e = np.asfortranarray(np.random.default_rng(0).normal(size=(5, 13)))
    np.savez(tmp_path / "data.npz", Nx=np.int64(8), energies=e)
    np.savez(tmp_path / "3d-fft-data-0.npz", **{"3D_fft_x": np.asfortranarray(np.ones((4, 4, 4), complex))})
    out = h5convert.convert_dir(str(tmp_path))
    assert sorted(map(str, out)) == sorted([str(tmp_path / "data.h5"), str(tmp_path / "3d-fft-data-0.h5")])
    with h5py.File(tmp_path / "data.h5") as f:
        assert f["energies"].shape == (13, 5) and int(f["Nx"][()]) == 8
        np.testing.assert_array_equal(f["energies"][()].T, e)


def test_params_from_reference_args():
    p = ewpt.Params.from_args(["0.0", "10", "200", "0.25", "20", "64", "0.99", "20", "0.0", "0.0", "0.0", "1"])
    assert p.N == 64 and p.dt == 0.25 / 20 and p.dsnaps == 10 and p.base_seed == 123456
    assert p.bub_diam == 12 and p.spec_cut == (16, 16, 16)
    c = p.to_c()
    assert c.nx == 64 and c.dt == 0.0125
