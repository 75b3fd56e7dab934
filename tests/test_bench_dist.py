"""Replica timing helpers of bench.py over a 2-rank gloo process group (CPU).

bench.py runs one replica per GPU under torchrun; the ranks share nothing but the
barrier around the timed region and the max-over-ranks of the step time.  Both
helpers are exercised here with two CPU processes, which is the multi-process path
without any GPU.
"""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["RANK"] = str(rank)
    os.environ["WORLD_SIZE"] = str(world)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (world, rank, int(os.environ.get("LOCAL_RANK", "0")))
        bench.barrier()
        # each rank reports a different step time; everyone must see the maximum
        got = bench.reduce_max(10.0 + 5.0 * rank)
        bench.barrier()
        results[rank] = got
    finally:
        dist.destroy_process_group()


def test_reduce_max_and_barrier_two_ranks():
    if not dist.is_available():
        pytest.skip("torch.distributed unavailable")
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    results = ctx.Manager().dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, results)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    assert dict(results) == {0: 15.0, 1: 15.0}


def test_reduce_max_without_process_group_is_identity():
    import bench

    assert not dist.is_initialized()
    assert bench.reduce_max(3.5) == 3.5
    bench.barrier()  # no-op without a group
    assert torch.tensor(1).item() == 1
