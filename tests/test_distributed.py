"""Multi-rank host logic on CPU (gloo, world size 2): shards cover the
instances exactly once, the step time is the max over ranks, and results
gather on rank 0 in rank order."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from tyxonq_gb300.distributed import cost_balanced_shards, gather_results, max_over_ranks, shard_range


def test_shard_range_partitions():
    for count in (0, 1, 7, 4096):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in shard_range(count, r, world)]
            assert got == list(range(count))
            sizes = [len(shard_range(count, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1


def test_cost_balanced_shards():
    costs = [2 ** n for n in np.random.default_rng(0).integers(8, 21, 200)]
    shards = cost_balanced_shards(costs, 4)
    assert sorted(i for s in shards for i in s) == list(range(200))
    loads = [sum(costs[i] for i in s) for s in shards]
    assert max(loads) / min(loads) < 1.3


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ids = list(shard_range(10, rank, world))
        local = np.array([float(i) ** 2 for i in ids])
        t = max_over_ranks(1.5 if rank == 0 else 2.5)
        allr = gather_results(local)
        if rank == 0:
            out.put((t, allr.tolist()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_sharded_evaluation():
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    t, vals = q.get()
    assert t == 2.5
    assert vals == [float(i) ** 2 for i in range(10)]


@pytest.mark.parametrize("world", [1])
def test_single_rank_passthrough(world):
    assert max_over_ranks(3.0) == 3.0
    np.testing.assert_array_equal(gather_results(np.array([1.0, 2.0])), [1.0, 2.0])
