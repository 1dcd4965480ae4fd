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
