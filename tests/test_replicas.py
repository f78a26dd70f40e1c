"""The N > 1 path of bench.py: independent replicas, no data-path collective; the timed region
is the slowest rank's and the value counts every rank's cells. Checked with world size 2 over
gloo on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        own_ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
        total = bench.max_over_ranks(own_ms)
        q.put((rank, total, bench.replica_value(1000, 10, world, total), bench.dist_info()))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
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
    for rank, total, value, info in out:
        assert total == 150.0
        assert value == pytest.approx(1000 * 10 * 2 / 0.150)
        assert info == (rank, 2, 0)


def test_without_a_process_group_the_rank_time_stands():
    import bench
    assert bench.max_over_ranks(42.0) == 42.0
    assert bench.replica_value(10, 2, 1, 1000.0) == 20.0
