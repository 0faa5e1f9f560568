"""z-slab decomposition on the GPU, through the C ABI: a lattice cut into
z-slabs (ghost planes filled from the neighbouring slabs before every
stage) evolves to the same bits as the undecomposed lattice, with the
stage kernels of the whole lattice reading their z neighbours from the
ghost planes.  Covered: one-process slab groups of 1, 2 and 3 slabs (even
and uneven), the J_ext/damp schedule, two slab contexts driven only by
ewpt_slab_pack/unpack/stage, and DistributedSlab on a one-rank process
group.  (Two ranks on one GPU would make NCCL ranks share a device; the
multi-rank exchange schedule is tested on CPU ranks in
tests/test_slabs_cpu.py.)"""
import socket

import numpy as np
import pytest

import ewpt
from ewpt.slabs import CSlab, DistributedSlab, SlabGroup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import build_lib

    build_lib.build()


def _state(shape, seed):
    y = ewpt.ic.bubbles_tanh(shape, 0.25, 3, seed=seed)
    y[4:] += 0.05 * np.random.default_rng(seed).normal(size=y[4:].shape)
    return y


def _whole(p, y0, steps, Jex=None, gamma=None):
    with ewpt.Lattice(p) as lat:
        lat.set_state(y0)
        lat.step(steps, Jex=Jex, gamma=gamma) if Jex is not None else lat.step(steps)
        return lat.get_state()


@pytest.mark.parametrize("shape,n,nzl", [((32, 24, 20), 1, None), ((32, 24, 20), 2, None),
                                         ((32, 24, 20), 3, [7, 6, 7]), ((24, 20, 18), 3, [3, 12, 3])])
def test_slab_group_bit_identical_to_whole_lattice(shape, n, nzl):
    p = ewpt.baseline_couplings(shape=shape, N=shape[0], dx=0.25, dt=0.025, beta_w=0.3, beta_y=0.2)
    y0 = _state(shape, 5)
    ref = _whole(p, y0, 10, Jex=0.03, gamma=0.02)
    with SlabGroup(p, n, nz_local=nzl) as g:
        assert g.count == n
        g.set_state(y0)
        g.step(10, Jex=0.03, gamma=0.02)
        y = g.get_state()
    np.testing.assert_array_equal(y, ref)


def test_slab_group_schedule_and_tiling():
    shape = (32, 16, 24)
    p = ewpt.baseline_couplings(shape=shape, N=32, dx=0.25, dt=0.025, thermal_init=True, gamma_inp=0.1)
    y0 = _state(shape, 8)
    with ewpt.Lattice(p) as lat:
        lat.set_tiling(32, 2, 0, 0)
        lat.set_state(y0)
        lat.step(12)
        ref = lat.get_state()
    with SlabGroup(p, 2) as g:
        g.set_tiling(32, 2, 0)
        g.set_state(y0)
        g.step(12)
        np.testing.assert_array_equal(g.get_state(), ref)


def test_two_slab_contexts_by_pack_and_unpack():
    import torch

    shape = (24, 16, 16)
    p = ewpt.baseline_couplings(shape=shape, N=24, dx=0.25, dt=0.025)
    y0 = _state(shape, 9)
    ref = _whole(p, y0, 6, Jex=0.0, gamma=0.0)
    nx, ny, nz = shape
    slabs = [CSlab(p, 0, 9), CSlab(p, 9, 7)]
    try:
        g = y0.reshape(36, nz, ny * nx)
        slabs[0].set_state(np.ascontiguousarray(g[:, :9]).reshape(36, -1))
        slabs[1].set_state(np.ascontiguousarray(g[:, 9:]).reshape(36, -1))
        for _ in range(6):
            for s in (1, 2, 3, 4):
                faces = [sl.pack(s) for sl in slabs]
                for sl in slabs:
                    sl.sync()
                faces = [(lo.clone(), hi.clone()) for lo, hi in faces]
                torch.cuda.synchronize()  # the slab streams do not wait for torch's stream
                for m, sl in enumerate(slabs):
                    below = faces[(m - 1) % 2][1]
                    above = faces[(m + 1) % 2][0]
                    sl.unpack(s, below, above)
                    sl.stage(s, 0.0, 0.0)
                for sl in slabs:
                    sl.sync()
        y = np.concatenate([sl.get_state().reshape(36, -1, ny * nx) for sl in slabs], axis=1).reshape(36, -1)
    finally:
        for sl in slabs:
            sl.close()
    np.testing.assert_array_equal(y, ref)


def test_distributed_slab_one_rank():
    import torch.distributed as dist

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        shape = (32, 16, 12)
        p = ewpt.baseline_couplings(shape=shape, N=32, dx=0.25, dt=0.025, beta_w=0.1)
        y0 = _state(shape, 4)
        ref = _whole(p, y0, 5, Jex=0.01, gamma=0.0)
        d = DistributedSlab(p)
        try:
            d.set_state(y0)
            d.step(5, Jex=0.01, gamma=0.0)
            d.sync()
            np.testing.assert_array_equal(d.get_state(), ref)
        finally:
            d.close()
    finally:
        dist.destroy_process_group()


def test_slab_rejections():
    p = ewpt.baseline_couplings(shape=(16, 16, 16), N=16, dx=0.25, dt=0.025)
    with pytest.raises(ewpt.EwptError):
        SlabGroup(p, 2, nz_local=[10, 2])  # a slab thinner than the halo
    with pytest.raises(ewpt.EwptError):
        SlabGroup(p, 2, nz_local=[8, 7])  # planes do not add up
    q = ewpt.baseline_couplings(shape=(16, 16, 16), N=16, dx=0.25, dt=0.025, precision=ewpt.FP32)
    with pytest.raises(ewpt.EwptError):
        SlabGroup(q, 2)
