"""ewpt_diagnostics_noalloc: the diagnostics entry point for callers that
cannot let the library allocate device memory (for example a process whose
device memory is already owned by another allocator's pool).  It must give
the same snapshot row as ewpt_diagnostics, call after call, although its
scratch array keeps whatever the previous call left in it.

The lattices cover the small case (one reduction block per x-y tile and z
plane), lattices whose z planes fold into each block's loop (256x256x64:
512 tiles, each block walks ~21 planes; 512x512x10 with the 8th-order
stencil: 2048 tiles, one block per tile walks all 10 planes), and the
largest accepted x-y extent (1024x512: exactly 4096 tiles).

This file is named so that pytest collects it last; it passes both alone in
a fresh process and after the other tests."""
import ctypes as C

import numpy as np
import pytest

import ewpt
from ewpt import _lib

pytestmark = pytest.mark.gpu

RTOL = 1e-10  # the diagnostics tolerance of the parity tests


def _noalloc(p, ptr, stream=0):
    L = _lib.load()
    out = np.zeros(_lib.NDIAG)
    cp = p.to_c()
    rc = L.ewpt_diagnostics_noalloc(C.byref(cp), C.c_void_p(ptr), out.ctypes.data_as(_lib.DP), C.c_void_p(stream))
    _lib.check(rc)
    return out


def _state(shape, seed):
    y = ewpt.ic.bubbles_tanh(shape, 0.25, 3, seed=seed)
    y[4:] += 0.1 * np.random.default_rng(seed).normal(size=y[4:].shape)
    return y


@pytest.fixture(scope="module", autouse=True)
def built():
    import build_lib

    build_lib.build()


@pytest.mark.parametrize("shape,order,side_stream", [
    ((40, 36, 24), 6, False),
    ((256, 256, 64), 6, True),
    ((512, 512, 10), 8, False),
    ((1024, 512, 8), 6, True),
])
def test_noalloc_matches_diagnostics_on_two_calls_in_a_row(shape, order, side_stream):
    import torch

    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025, stencil_order=order)
    states = [_state(shape, 3), _state(shape, 4)]
    refs = []
    with ewpt.Lattice(p) as lat:
        for y in states:
            lat.set_state(y)
            refs.append(lat.diagnostics())
    stream = torch.cuda.Stream() if side_stream else torch.cuda.current_stream()
    dev_before = torch.cuda.current_device()
    for y, ref in zip(states, refs):
        with torch.cuda.stream(stream):
            dev = torch.tensor(y, dtype=torch.float64, device="cuda:0").contiguous()
        got = _noalloc(p, dev.data_ptr(), stream.cuda_stream)
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=1e-13)
        del dev
    assert torch.cuda.current_device() == dev_before
    assert not np.allclose(refs[0], refs[1])


def test_noalloc_rejects_lattices_beyond_its_scratch():
    import torch

    p = ewpt.baseline_couplings(shape=(1024, 1024, 8), N=1024, dx=0.25, dt=0.025)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    L = _lib.load()
    out = np.zeros(_lib.NDIAG)
    cp = p.to_c()
    rc = L.ewpt_diagnostics_noalloc(C.byref(cp), C.c_void_p(dummy.data_ptr()), out.ctypes.data_as(_lib.DP), None)
    assert rc == _lib.ERR_ARG
    assert "4096" in L.ewpt_last_error(None).decode()
