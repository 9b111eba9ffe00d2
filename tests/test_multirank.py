"""Two-rank host logic of bench.py on CPU (gloo): the slowest rank's time is
the job's time, and the whole-job throughput counts every rank's replica.
The render path itself has no collective (replicas only)."""

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


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank 1 is the slow one for the first value, rank 0 for the second
        mine = [1.0 + rank, 5.0 - rank]
        got = bench.max_over_ranks(mine)
        value = bench.aggregate_gsamples(2_000_000_000, world, 4, got[0])
        dist.barrier()
        q.put((rank, got, value))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, value in out:
        assert got == [2.0, 5.0]
        # 2e9 samples x 2 replicas x 4 steps in 2 s
        assert value == pytest.approx(8.0)


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks([3.5, 1.25]) == [3.5, 1.25]
    assert bench.aggregate_gsamples(1e9, 1, 2, 1.0) == pytest.approx(2.0)
