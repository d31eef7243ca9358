"""Multi-rank host logic of bench.py on CPU: two gloo ranks (replicas) take
the slowest rank's time and sum the units all ranks processed."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slowest = bench.reduce_over_ranks(dist, 1.5 + rank, "max", "cpu")
        units = bench.reduce_over_ranks(dist, 1000 * (rank + 1), "sum", "cpu")
        out.put((rank, slowest, units))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_replicas_take_the_slowest_rank_and_sum_the_units():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert res == [(0, 2.5, 3000.0), (1, 2.5, 3000.0)]


def test_one_rank_keeps_its_own_numbers():
    import bench

    assert bench.reduce_over_ranks(None, 4.25, "max", "cpu") == 4.25
    assert bench.reduce_over_ranks(None, 7, "sum", "cpu") == 7.0
