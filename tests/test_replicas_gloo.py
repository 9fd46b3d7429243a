"""The multi-GPU path of bench.py is replicas only (one independent solve per
GPU, no data-path collective): its host logic -- barrier, max-over-ranks
timing and the whole-job value -- checked with world_size 2 on the gloo
backend, on CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    import bench
    bench.barrier(world)
    ms = bench.max_over_ranks(world, 10.0 + 5.0 * rank)       # rank 1 is the slow replica
    out[rank] = (ms, bench.replica_value(world, 1_000_000_000, 7, ms))
    bench.barrier(world)
    dist.destroy_process_group()


def test_replicas_time_by_the_slowest_and_sum_the_work():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    ms, value = out[0]
    assert ms == 15.0
    assert value == pytest.approx(2 * 1e9 * 7 / 0.015 / 1e9)
