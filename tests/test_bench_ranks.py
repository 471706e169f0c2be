"""The multi-rank bookkeeping of bench.py on CPU: two gloo ranks each time a
different amount of work; the job time is the slowest rank's on every rank,
and the whole-job rate counts every rank's replica (weak scaling).  No GPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = 100.0 + 37.5 * rank
    out[rank] = bench.max_over_ranks(mine, world, "cpu")
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_job_time_is_the_slowest_rank(world):
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert dict(out) == {r: 100.0 + 37.5 * (world - 1) for r in range(world)}


def test_single_rank_and_rate():
    assert bench.max_over_ranks(12.5, 1) == 12.5
    # 2 replicas of 1 Mi cells, 10000 steps per run, 3 runs in 450 ms
    assert bench.job_rate(2, 1 << 20, 10000, 3, 450.0) == pytest.approx(2 * (1 << 20) * 30000 / 0.45 / 1e9)
