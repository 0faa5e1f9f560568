"""z-slab domain decomposition: the host side of libewpt's slab API.

The reference decomposes its lattice over MPI ranks and refreshes 3-plane
ghost layers with MPI.Sendrecv! after every stage (update_halo!,
boundary_x/y/z, gpu-kernels-rk4/main_rk4_multiple.jl:69-212).  Here:

SlabGroup        one process drives n z-slabs of one lattice, on one GPU or
                 several (ewpt_slabs_*); the exchanges are device copies.
DistributedSlab  one slab per rank of a torch.distributed process group:
                 before every RK4 stage each rank packs the bottom and top 3
                 interior planes of the stage's input, sends them to the
                 slab below and above (periodic in z) and unpacks what it
                 receives into its ghost planes (NCCL between GPUs; any
                 backend whose tensors the slab backend can read).
halo_exchange    that send/receive pattern on its own.

A decomposed step gives the same bits as the undecomposed one: the slab
kernels are the whole lattice's, reading z neighbours from ghost planes.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .params import Params

GHOST = 3  # ghost planes per z face


def even_split(nz: int, n: int) -> list[int]:
    """Planes per slab: nz // n each, the first nz % n slabs one more."""
    return [nz // n + (1 if m < nz % n else 0) for m in range(n)]


def slab_extent(nz: int, n: int, m: int) -> tuple[int, int]:
    """(first plane, planes) of slab m of an even split."""
    sizes = even_split(nz, n)
    return sum(sizes[:m]), sizes[m]


def _jext(p: Params, it: int) -> float:
    return p.mH * p.mH if (it * p.dt * p.mH <= p.t_sat and p.thermal_init) else 0.0


def _damp(p: Params, it: int) -> float:
    return 0.0 if (it * p.dt * p.mH < p.t_sat and p.thermal_init) else p.gamma_inp


class SlabGroup:
    """n z-slabs of one lattice in this process (ewpt_slabs_create)."""

    def __init__(self, params: Params, n: int, nz_local=None, devices=None):
        self.params = params
        self.L = _lib.load()
        self._cp = params.to_c()
        nzl = (C.c_int32 * n)(*nz_local) if nz_local is not None else None
        dev = (C.c_int32 * n)(*devices) if devices is not None else None
        h = C.c_void_p()
        self._chk(self.L.ewpt_slabs_create(C.byref(self._cp), int(n), nzl, dev, C.byref(h)), None)
        self.h = h
        self.S = params.sites

    def _chk(self, rc, h=-1):
        if rc != _lib.OK:
            hh = self.h if h == -1 else h
            raise _lib.EwptError(rc, self.L.ewpt_slabs_last_error(hh).decode())

    def close(self):
        if self.h:
            self.L.ewpt_slabs_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def count(self) -> int:
        return int(self.L.ewpt_slabs_count(self.h))

    def set_state(self, y: np.ndarray):
        y = np.ascontiguousarray(y, dtype=np.float64)
        assert y.shape == (36, self.S)
        self._chk(self.L.ewpt_slabs_set_state(self.h, C.c_void_p(y.ctypes.data), 0))

    def get_state(self) -> np.ndarray:
        y = np.empty((36, self.S))
        self._chk(self.L.ewpt_slabs_get_state(self.h, C.c_void_p(y.ctypes.data), 0))
        return y

    def set_tiling(self, bx: int, by: int, reg: int = 0):
        self._chk(self.L.ewpt_slabs_set_tiling(self.h, int(bx), int(by), int(reg)))

    def step(self, n: int = 1, Jex: float | None = None, gamma: float | None = None):
        if Jex is None and gamma is None:
            self._chk(self.L.ewpt_slabs_step(self.h, int(n)))
        else:
            self._chk(self.L.ewpt_slabs_step_explicit(self.h, int(n), float(Jex or 0.0), float(gamma or 0.0)))

    def sync(self):
        self._chk(self.L.ewpt_slabs_sync(self.h))


def halo_exchange(lo, hi, group=None):
    """Send this rank's bottom planes `lo` to the rank below and its top
    planes `hi` to the rank above (periodic over the group's ranks); return
    (below, above): the rank below's `hi` and the rank above's `lo`.  With
    two ranks both neighbours are the same peer: the sends go out top face
    first and the receives are posted below first, so the in-order matching
    of point-to-point operations pairs each face with the right ghost."""
    import torch
    import torch.distributed as dist

    ws = dist.get_world_size(group)
    r = dist.get_rank(group)
    if ws == 1:
        return hi.clone(), lo.clone()
    down, up = (r - 1) % ws, (r + 1) % ws
    if group is not None:
        down, up = dist.get_global_rank(group, down), dist.get_global_rank(group, up)
    below, above = torch.empty_like(hi), torch.empty_like(lo)
    ops = [dist.P2POp(dist.isend, hi, up, group, tag=1), dist.P2POp(dist.isend, lo, down, group, tag=2),
           dist.P2POp(dist.irecv, below, down, group, tag=1), dist.P2POp(dist.irecv, above, up, group, tag=2)]
    for req in dist.batch_isend_irecv(ops):
        req.wait()
    return below, above


class CSlab:
    """One slab context of libewpt (ewpt_create_slab) with device face buffers."""

    def __init__(self, params: Params, z0: int, nz_local: int):
        import torch

        self.params = params
        self.L = _lib.load()
        self._cp = params.to_c()
        h = C.c_void_p()
        _lib.check(self.L.ewpt_create_slab(C.byref(self._cp), int(z0), int(nz_local), C.byref(h)))
        self.h = h
        nx, ny, _ = params.dims
        self.n = nx * ny * nz_local
        self.face = 36 * GHOST * nx * ny
        dev = torch.device("cuda", params.device)
        self.lo = torch.empty(self.face, dtype=torch.float64, device=dev)
        self.hi = torch.empty(self.face, dtype=torch.float64, device=dev)
        self.stream = torch.cuda.ExternalStream(self.L.ewpt_stream(self.h), device=dev)

    def _chk(self, rc):
        return _lib.check(rc, self.h)

    def close(self):
        if self.h:
            self.L.ewpt_destroy(self.h)
            self.h = None

    def set_state(self, y: np.ndarray):
        y = np.ascontiguousarray(y, dtype=np.float64)
        assert y.shape == (36, self.n)
        self._chk(self.L.ewpt_set_state_packed(self.h, C.c_void_p(y.ctypes.data), 0))

    def get_state(self) -> np.ndarray:
        y = np.empty((36, self.n))
        self._chk(self.L.ewpt_get_state_packed(self.h, C.c_void_p(y.ctypes.data), 0))
        return y

    def pack(self, stage: int):
        self._chk(self.L.ewpt_slab_pack(self.h, int(stage), C.c_void_p(self.lo.data_ptr()),
                                        C.c_void_p(self.hi.data_ptr())))
        return self.lo, self.hi

    def unpack(self, stage: int, below, above):
        self._chk(self.L.ewpt_slab_unpack(self.h, int(stage), C.c_void_p(below.data_ptr()),
                                          C.c_void_p(above.data_ptr())))

    def stage(self, stage: int, Jex: float, gamma: float):
        self._chk(self.L.ewpt_slab_stage(self.h, int(stage), float(Jex), float(gamma)))

    def stream_ctx(self):
        import torch

        return torch.cuda.stream(self.stream)

    def sync(self):
        self._chk(self.L.ewpt_sync(self.h))


class DistributedSlab:
    """This rank's slab of a lattice decomposed over a process group: planes
    slab_extent(nz, world, rank).  `backend` performs the slab operations
    (default: a libewpt slab context on params.device; the exchange then
    runs on its stream, NCCL ordering against the kernels)."""

    def __init__(self, params: Params, group=None, backend=None):
        import torch.distributed as dist

        self.params = params
        self.group = group
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        self.z0, self.nz = slab_extent(params.dims[2], self.world, self.rank)
        if self.nz < GHOST:
            raise ValueError(f"slab of {self.nz} planes: each rank needs >= {GHOST}")
        self.b = backend if backend is not None else CSlab(params, self.z0, self.nz)
        self.it = 0

    def close(self):
        close = getattr(self.b, "close", None)
        if close:
            close()

    def local(self, y_global: np.ndarray) -> np.ndarray:
        """This rank's planes of a packed global state."""
        nx, ny, nz = self.params.dims
        g = y_global.reshape(36, nz, ny * nx)
        return np.ascontiguousarray(g[:, self.z0:self.z0 + self.nz]).reshape(36, -1)

    def set_state(self, y_global: np.ndarray):
        self.b.set_state(self.local(y_global))
        self.it = 0

    def get_state(self) -> np.ndarray:
        return self.b.get_state()

    def step(self, n: int = 1, Jex: float | None = None, gamma: float | None = None):
        ctx = getattr(self.b, "stream_ctx", None)
        for _ in range(int(n)):
            it = self.it + 1
            J = _jext(self.params, it) if Jex is None else Jex
            G = _damp(self.params, it) if gamma is None else gamma
            for s in (1, 2, 3, 4):
                if ctx is not None:
                    with ctx():
                        lo, hi = self.b.pack(s)
                        below, above = halo_exchange(lo, hi, self.group)
                        self.b.unpack(s, below, above)
                else:
                    lo, hi = self.b.pack(s)
                    below, above = halo_exchange(lo, hi, self.group)
                    self.b.unpack(s, below, above)
                self.b.stage(s, J, G)
            self.it = it

    def sync(self):
        sync = getattr(self.b, "sync", None)
        if sync:
            sync()
