"""Tile-shape autotuner for the stage kernels.

Times every candidate launch shape (block bx x by over x-y, register-budget
variant reg; see ewpt_set_tiling in include/ewpt.h) on a scratch lattice of
the same size and precision, with CUDA events on the library's stream, and
caches the fastest per (lattice shape, precision, beta on/off, GPU name) in a
JSON file (default ~/.cache/ewpt/autotune.json, or $EWPT_AUTOTUNE_CACHE).
The result does not change any number the kernels compute, only their speed.
"""
from __future__ import annotations

import json
import os

from . import _lib, ic
from .lattice import Lattice
from .params import Params

CANDIDATES = [(32, 4, 0, 0), (64, 2, 0, 0), (32, 2, 0, 0), (16, 8, 0, 0), (128, 1, 0, 0),
              (32, 4, 1, 0), (64, 2, 1, 0), (32, 2, 1, 0), (16, 8, 1, 0),
              (32, 4, 2, 0), (64, 2, 2, 0), (32, 2, 2, 0), (16, 8, 2, 0)]
# FP32 form only: two sites per thread (needs even nx)
PAIR_CANDIDATES = [(32, 4, 0, 1), (64, 2, 0, 1), (32, 2, 0, 1), (16, 4, 0, 1), (32, 1, 0, 1), (64, 1, 0, 1),
                   (32, 4, 1, 1), (64, 2, 1, 1), (32, 2, 1, 1), (32, 4, 2, 1), (64, 2, 2, 1), (32, 2, 2, 1),
                   # narrow blocks for lattices of 48-160 sites per row (ensemble members)
                   (16, 8, 2, 1), (8, 16, 2, 1), (16, 8, 0, 1)]
# FP32 form only: TMA-staged tiles of 32 x by x bz sites, (bx, by, bz, 2)
TMA_CANDIDATES = [(32, 4, 4, 2), (32, 2, 4, 2)]


def cache_path() -> str:
    return os.environ.get("EWPT_AUTOTUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "ewpt",
                                                               "autotune.json"))


def _key(p: Params) -> str:
    import torch

    nx, ny, nz = p.dims
    beta = int(p.beta_w != 0.0 or p.beta_y != 0.0)
    return f"{nx}x{ny}x{nz}:p{int(p.precision)}:b{beta}:{torch.cuda.get_device_name(p.device)}"


def _load_cache() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _save_cache(d: dict):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def time_tiling(lat: Lattice, tile, steps: int = 2) -> float:
    """Seconds per RK4 step with the given tiling (CUDA events on the lattice's stream)."""
    import torch

    lat.set_tiling(*tile)
    st = torch.cuda.ExternalStream(lat.stream)
    lat.step(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    lat.step(steps)
    e1.record(st)
    lat.sync()
    return e0.elapsed_time(e1) / 1e3 / steps


def candidates_for(p: Params) -> list:
    """The launch shapes offered for this lattice and form: the one-site
    shapes always; for the FP32 form the paired shapes (even nx) and the
    TMA-staged tiles (nx a multiple of 32, ny and nz multiples of the tile)."""
    candidates = list(CANDIDATES)
    nx, ny, nz = p.dims
    if int(p.precision) == _lib.FP32 and nx % 2 == 0:
        candidates += PAIR_CANDIDATES
    if int(p.precision) == _lib.FP32 and nx % 32 == 0:
        candidates += [t for t in TMA_CANDIDATES if ny % t[1] == 0 and nz % t[2] == 0]
    return candidates


def sweep(p: Params, steps: int = 2, candidates=None) -> list:
    """(tiling, seconds per step) for every candidate on a scratch lattice."""
    if candidates is None:
        candidates = candidates_for(p)
    res = []
    with Lattice(p) as lat:
        R, w = ic.tanh_profile_params(p.lam, p.vev)
        lat.init_bubbles(ic.tanh_bubble_list(p.dims, p.dx, 4, seed=0), "tanh", R, w)  # device IC: no host state
        for t in candidates:
            try:
                res.append((t, time_tiling(lat, t, steps)))
            except _lib.EwptError:
                continue
    return res


def best_tiling(p: Params, steps: int = 2, use_cache: bool = True) -> tuple:
    key = _key(p)
    cache = _load_cache() if use_cache else {}
    if key in cache:
        return tuple(cache[key]["tile"])
    res = sweep(p, steps)
    tile, t = min(res, key=lambda r: r[1])
    cache[key] = {"tile": list(tile), "s_per_step": t, "sweep": [[list(a), b] for a, b in res]}
    if use_cache:
        _save_cache(cache)
    return tile


def tune(lat: Lattice, steps: int = 2) -> tuple:
    """Apply the cached (or freshly measured) best tiling to `lat`.  A sweep
    runs on a second lattice of the same size: for lattices that fill most
    of the GPU, call best_tiling(params) before creating the lattice."""
    tile = best_tiling(lat.params, steps)
    lat.set_tiling(*tile)
    return tile


# (bx, by, pair); narrow blocks (8 or 16 pair-threads = 16 or 32 sites in x)
# waste fewer threads on members of 48 / 96 / 160 sites per row
ENSEMBLE_CANDIDATES = [(8, 8, 1), (8, 16, 1), (16, 8, 1), (16, 4, 1), (8, 4, 1), (32, 4, 1), (32, 2, 1), (64, 2, 1),
                       (32, 4, 0), (16, 8, 0), (32, 2, 0)]


def member_tilings(members, steps: int = 2, use_cache: bool = True) -> list:
    """The fastest single-lattice launch shape (one site or two sites per
    thread; the ensemble's graph branches run those kernels) for each member,
    timed once per distinct member size and couplings switch and cached."""
    out, seen = [], {}
    for p in members:
        even = p.dims[0] % 2 == 0
        cands = list(CANDIDATES) + (list(PAIR_CANDIDATES) if even else [])
        key = "member:" + _key(p)
        if key not in seen:
            cache = _load_cache() if use_cache else {}
            if key in cache:
                seen[key] = tuple(cache[key]["tile"])
            else:
                res = sweep(p, steps, cands)
                tile, t = min(res, key=lambda r: r[1])
                cache[key] = {"tile": list(tile), "s_per_step": t, "sweep": [[list(a), b] for a, b in res]}
                if use_cache:
                    _save_cache(cache)
                seen[key] = tile
        out.append(seen[key])
    return out


def tune_ensemble(ens, steps: int = 2) -> list:
    """Apply member_tilings to a live ensemble (the sweeps run on scratch
    lattices of the members' sizes); returns the shapes."""
    tiles = member_tilings(ens.members, steps)
    for m, t in enumerate(tiles):
        ens.set_member_tiling(m, *t)
    return tiles


def best_ensemble_tiling(members, steps: int = 2, use_cache: bool = True) -> tuple:
    """Fastest (bx, by, pair) for an ensemble of these members, timed on a
    scratch ensemble (so no live state is touched) and cached by the member
    shapes, couplings switches and GPU name."""
    import hashlib

    import torch

    from .ensemble import Ensemble

    shapes = ",".join(f"{p.dims[0]}x{p.dims[1]}x{p.dims[2]}" for p in members)
    beta = int(any(p.beta_w != 0.0 or p.beta_y != 0.0 for p in members))
    key = "ens:" + hashlib.sha1(shapes.encode()).hexdigest()[:16] + f":b{beta}:{torch.cuda.get_device_name(0)}"
    cache = _load_cache() if use_cache else {}
    if key in cache:
        return tuple(cache[key]["tile"])
    even = all(p.dims[0] % 2 == 0 for p in members)
    res = []
    with Ensemble(members) as ens:
        for m, p in enumerate(members):
            R, w = ic.tanh_profile_params(p.lam, p.vev)
            ens.init_bubbles(m, ic.tanh_bubble_list(p.dims, p.dx, 4, seed=m), "tanh", R, w)
        st = torch.cuda.ExternalStream(ens.stream)
        for t in ENSEMBLE_CANDIDATES:
            if t[2] and not even:
                continue
            ens.set_tiling(*t)
            ens.step(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            ens.step(steps)
            e1.record(st)
            ens.sync()
            res.append((t, e0.elapsed_time(e1) / 1e3 / steps))
    tile, s = min(res, key=lambda r: r[1])
    cache[key] = {"tile": list(tile), "s_per_step": s, "sweep": [[list(a), b] for a, b in res]}
    if use_cache:
        _save_cache(cache)
    return tile
