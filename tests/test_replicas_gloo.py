"""Multi-GPU runs are replicas only (one independent slab per rank, no
data-path collective): the whole-job rate is the units all ranks processed
over the slowest rank's time. Checked with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r processes 1000 * (r + 1) units in 1 + r seconds
    rate, slowest, units = bench.replica_rate(dist, 1000.0 * (rank + 1), 1.0 + rank, "cpu")
    out.put((rank, rate, slowest, units))
    dist.destroy_process_group()


def test_replica_rate_two_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, rate, slowest, units in res:
        assert slowest == 2.0 and units == 3000.0 and rate == 1500.0
