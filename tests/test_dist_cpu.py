"""The N > 1 path of bench.py on CPU (gloo, world size 2): the barrier, the
max over ranks of the timed region, the whole-job value (replicas x units
/ slowest rank), and the reference arm that only rank 0 runs."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    import argparse

    import torch.distributed as dist

    import bench

    args = argparse.Namespace(impl="reference")
    ws, r, local = bench.dist_init(args)  # gloo for the reference arm
    bench.barrier(ws)
    t = bench.allmax(ws, 1.0 + rank)  # rank 1 is the slower one
    sites, steps = 1000, 4
    value = ws * sites * steps / t
    skipped = bench.run_reference(args, ws, r) if r != 0 else None  # returns at once off rank 0
    q.put((r, ws, t, value, skipped))
    dist.destroy_process_group()


def test_two_rank_aggregation_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, ws, t, value, skipped in out:
        assert ws == 2 and t == 2.0  # max over ranks
        assert value == pytest.approx(2 * 1000 * 4 / 2.0)
        assert skipped is None
