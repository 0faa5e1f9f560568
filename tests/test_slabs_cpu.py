"""The z-slab decomposition's host logic on CPU ranks (gloo): every rank
owns planes slab_extent(nz, world, rank) of the lattice, exchanges its
bottom and top 3 interior planes with the ranks below and above (periodic
in z) before every RK4 stage, and evolves its slab.  The slab operations run
here on a CPU stand-in built on the oracle: a slab's padded box (interior
plus 3 ghost planes per z face) is evolved with the oracle's rates, which
are exact on the interior once the ghost planes hold the neighbours'
planes.  The decomposed evolution must equal the oracle's RK4 step on the
whole lattice bit for bit, which checks the exchange schedule (who sends
which face to whom, including two ranks whose neighbours coincide), the
plane bookkeeping of pack/unpack and the stage order."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SHAPE = (8, 7, 10)
COUP = dict(dx=0.25, gw=0.65, gy=0.35, gp2=0.99, lam=0.129, vev=1.0, bw=0.3, by=0.2)
DT, JEX, GAM, NSTEPS = 0.025, 0.04, 0.02, 3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _state():
    S = int(np.prod(SHAPE))
    rng = np.random.default_rng(17)
    y = rng.normal(0.0, 0.3, size=(36, S))
    y[0] += 0.7
    return y


class OracleSlab:
    """CPU stand-in for one slab context: FP64 buffers y, yn and the two
    stage inputs over the padded box, the stage combination in the
    oracle's rounding order (or_rk4_step)."""

    def __init__(self, z0, nzl):
        from oracle import oracle as orc

        self.orc = orc
        nx, ny, _ = SHAPE
        self.pl, self.nzl = nx * ny, nzl
        shape_p = (nx, ny, nzl + 6)
        P = nx * ny * (nzl + 6)
        self.y, self.yn, self.xa, self.xb = (np.zeros((36, P)) for _ in range(4))
        c = COUP
        self.op = orc.params(shape_p, c["dx"], c["gw"], c["gy"], c["gp2"], c["lam"], c["vev"], c["bw"], c["by"])

    def _inp(self, s):
        return {1: self.y, 2: self.xa, 3: self.xb, 4: self.xa}[s]

    def _int(self):
        return slice(3 * self.pl, (3 + self.nzl) * self.pl)

    def set_state(self, y):
        self.y[:, self._int()] = y

    def get_state(self):
        return self.y[:, self._int()].copy()

    def pack(self, s):
        import torch

        b, pl = self._inp(s), self.pl
        lo = b[:, 3 * pl:6 * pl].copy()
        hi = b[:, self.nzl * pl:(self.nzl + 3) * pl].copy()
        return torch.from_numpy(lo.ravel()), torch.from_numpy(hi.ravel())

    def unpack(self, s, below, above):
        b, pl = self._inp(s), self.pl
        b[:, 0:3 * pl] = below.numpy().reshape(36, 3 * pl)
        b[:, (self.nzl + 3) * pl:(self.nzl + 6) * pl] = above.numpy().reshape(36, 3 * pl)

    def stage(self, s, J, G):
        k = self.orc.rates(self.op, self._inp(s), J, G)
        I = self._int()
        y, yn = self.y[:, I], self.yn[:, I]
        if s == 1:
            self.yn[:, I] = k[:, I] * (DT / 6.) + y
            self.xa[:, I] = y + k[:, I] * (DT / 2.)
        elif s == 2:
            self.yn[:, I] = k[:, I] * (DT / 3.) + yn
            self.xb[:, I] = y + k[:, I] * (DT / 2.)
        elif s == 3:
            self.yn[:, I] = k[:, I] * (DT / 3.) + yn
            self.xa[:, I] = y + k[:, I] * DT
        else:
            self.y[:, I] = k[:, I] * (DT / 6.) + yn


def _worker(rank, ws, port, q):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "ewpt-gpu_gb300"))
    import torch.distributed as dist

    from ewpt import Params
    from ewpt.slabs import DistributedSlab, slab_extent

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    p = Params(shape=SHAPE, N=SHAPE[0], dx=COUP["dx"], dt=DT, gw=COUP["gw"], gy=COUP["gy"], gp2=COUP["gp2"],
               lam=COUP["lam"], vev=COUP["vev"], beta_w=COUP["bw"], beta_y=COUP["by"])
    z0, nzl = slab_extent(SHAPE[2], ws, rank)
    d = DistributedSlab(p, backend=OracleSlab(z0, nzl))
    d.set_state(_state())
    d.step(NSTEPS, Jex=JEX, gamma=GAM)
    q.put((rank, z0, nzl, d.get_state()))
    dist.destroy_process_group()


@pytest.mark.parametrize("ws", [2, 3])
def test_distributed_slabs_match_whole_lattice_gloo(ws):
    import torch.multiprocessing as mp

    from oracle import oracle as orc

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    parts = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    nx, ny, nz = SHAPE
    y = np.zeros((36, nz, ny * nx))
    for _, z0, nzl, loc in parts:
        y[:, z0:z0 + nzl] = loc.reshape(36, nzl, ny * nx)
    c = COUP
    op = orc.params(SHAPE, c["dx"], c["gw"], c["gy"], c["gp2"], c["lam"], c["vev"], c["bw"], c["by"])
    ref = orc.rk4_step(op, _state(), DT, JEX, GAM, nsteps=NSTEPS)
    np.testing.assert_array_equal(y.reshape(36, -1), ref)


def test_even_split():
    from ewpt.slabs import even_split, slab_extent

    assert even_split(10, 3) == [4, 3, 3]
    assert [slab_extent(10, 3, m) for m in range(3)] == [(0, 4), (4, 3), (7, 3)]
    assert sum(even_split(256, 7)) == 256
