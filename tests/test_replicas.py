"""The N-GPU bench path on the CPU: two gloo ranks each time their own replica;
the job's time is the slowest rank's and its throughput counts every rank's
evaluations (bench.py replica_max_ms / replica_throughput)."""

from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
    max_ms = bench.replica_max_ms(local_ms, dist, "cpu")
    out.put((rank, max_ms, bench.replica_throughput(world, 10, max_ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [150.0, 150.0]
    assert all(abs(r[2] - 2 * 10 / 0.150) < 1e-9 for r in res)


def test_single_replica_needs_no_collective():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_max_ms(123.0, None, "cpu") == 123.0
    assert abs(bench.replica_throughput(1, 5, 500.0) - 10.0) < 1e-12
