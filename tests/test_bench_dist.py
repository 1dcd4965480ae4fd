"""The multi-rank path of bench.py on CPU: two gloo ranks, each sliding its
own stream (no data-path collective), combine into one whole-job number from
the slowest rank's time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_ms = 100.0 * (rank + 1)  # rank 1 is the slowest
    value, total_ms = bench.weak_scaling_value(local_ms, steps=10, stride=1_000, world=world)
    out[rank] = (value, total_ms)
    dist.destroy_process_group()


def test_weak_scaling_value_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    world, port = 2, _free_port()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    for r in range(world):
        value, total_ms = out[r]
        assert total_ms == 200.0                  # MAX over ranks
        assert value == pytest.approx(2 * 10 * 1_000 / 0.2)


def test_weak_scaling_value_single_rank():
    import bench

    value, total_ms = bench.weak_scaling_value(50.0, steps=5, stride=2_000, world=1)
    assert total_ms == 50.0 and value == pytest.approx(5 * 2_000 / 0.05)


def _shard_rank(rank, world, port, out):
    """One rank of the sharded batched/serving legs: it takes its share of
    the 256-stream mix and reports its slid points and time."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from rtdbstream_gb300 import workloads as wl

    streams = wl.mixed_streams(256)
    mine = bench.partition_streams([s.window for s in streams], world, rank)
    points = float(sum(streams[i].stride for i in mine))
    ms = 10.0 + rank                                   # rank 1 is the slowest
    value, total, max_ms = bench.combine_ranks(points, ms, world)
    out[rank] = (mine, value, total, max_ms)
    dist.destroy_process_group()


def test_streams_shard_across_two_gloo_ranks():
    """The 256 streams split across two ranks with no stream lost or shared,
    even work, and the whole-job rate = all slid points / slowest rank."""
    from rtdbstream_gb300 import workloads as wl

    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    world, port = 2, _free_port()
    mp.start_processes(_shard_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    streams = wl.mixed_streams(256)
    owned = sorted(out[0][0] + out[1][0])
    assert owned == list(range(256))
    loads = [sum(streams[i].window for i in out[r][0]) for r in range(world)]
    assert max(loads) / min(loads) < 1.05
    total = float(sum(s.stride for s in streams))
    for r in range(world):
        _, value, got_total, max_ms = out[r]
        assert got_total == total and max_ms == 11.0
        assert value == pytest.approx(total / 0.011)


def test_partition_single_rank_and_balance():
    import bench

    costs = [5, 1, 9, 3, 3, 7, 2]
    assert bench.partition_streams(costs, 1, 0) == list(range(len(costs)))
    parts = [bench.partition_streams(costs, 3, r) for r in range(3)]
    assert sorted(sum(parts, [])) == list(range(len(costs)))
    sums = [sum(costs[i] for i in p) for p in parts]
    assert max(sums) - min(sums) <= max(costs)
