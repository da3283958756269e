"""Replica aggregation of bench.py on CPU: two gloo ranks, as torchrun would
start them.  Each rank brings its own timed region and units; the job's
number is the slowest rank's time and the sum of the units, with no other
exchange."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        t_ms, units = bench.aggregate(10.0 + 5.0 * rank, 1000.0 * (rank + 1), world, "cpu")
        q.put((rank, t_ms, units))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_sum_units():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for _, t_ms, units in got:
        assert t_ms == 15.0      # the slowest rank's time
        assert units == 3000.0   # the whole job's units


def test_single_process_is_identity():
    import bench

    assert bench.aggregate(12.5, 77.0, 1) == (12.5, 77.0)
