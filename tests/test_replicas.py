"""Replica aggregation of bench.py under torch.distributed (gloo, two CPU
ranks): every rank learns the slowest rank's step time and the whole-job
throughput counts the units of all ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_setup() == (world, rank, rank)
        ms, value = bench.replica_throughput(1.0 + rank, 2_000_000, world)  # rank 1 is slower
        q.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(world))
    for rank, ms, value in got:
        assert ms == 2.0  # max over ranks
        assert value == pytest.approx(world * 2_000_000 / 2e-3 / 1e6)  # 2,000 M/s


def test_one_replica_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.replica_throughput(4.0, 1_000_000, 1) == (4.0, 250.0)
