"""The multi-GPU path of bench.py is replicas only: each rank advances its own bodies, the
ranks meet at a barrier, and the job's time is the slowest rank's.  This checks that host
logic with two gloo ranks on the CPU (no GPU involved)."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, q):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    my_time = 2.0 + rank  # rank 1 is the slow one
    bench.barrier(world)
    t_max = bench.max_over_ranks(world, my_time)
    value = bench.replica_value(world, 1000, 10, t_max)
    q.put((rank, t_max, value))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [3.0, 3.0]
    assert out[0][2] == pytest.approx(2 * 1000 * 10 / 3.0)
    assert out[0][2] == out[1][2]
