"""Replica-mode multi-process plumbing of bench.py on CPU (gloo, world size 2).

Each rank runs an independent replica; the only cross-rank traffic is a
barrier and the max of the per-rank times (no data-path collective).
"""
from __future__ import annotations

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(float(rank + 1) * 1.5)
    d.close()
    q.put((rank, d.ws, m))


def test_dist_max_and_barrier_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 2, 3.0), (1, 2, 3.0)]
