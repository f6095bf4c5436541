"""Multi-rank host logic on CPU (gloo, world size 2): shards cover the
instances exactly once, the step time is the max over ranks, and a
strong-scaling split of one VQE workload (cost-balanced shards, evaluated per
rank) gathers energies and gradients on rank 0 in instance order, equal to a
serial evaluation."""
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


def _oracle_eval(inst):
    from oracle import sv

    gates = [(nm, list(qs), p, 1.0) for nm, qs, p in inst.structure()]
    return sv.grad_adjoint(inst.n, gates, inst.theta, inst.H.codes, inst.H.coeffs)


def _worker(rank, world, port, out):
    """One rank of a strong-scaling split: evaluate this rank's cost-balanced
    shard of one VQE workload (the oracle stands in for the device engine on
    CPU), then gather energies and gradients in instance order on rank 0."""
    from tyxonq_gb300.distributed import gather_instances, shard_instances
    from tyxonq_gb300.workloads import batched_vqe

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        insts = batched_vqe(14, seed=11, n_range=(3, 8), depth_range=(1, 3), terms_range=(5, 30))
        ids = shard_instances(insts, rank, world)
        res = [_oracle_eval(insts[i]) for i in ids]
        t = max_over_ranks(1.5 if rank == 0 else 2.5)
        got = gather_instances(ids, [e for e, _ in res], [g for _, g in res], len(insts))
        if rank == 0:
            E, G = got
            out.put((t, sorted(ids), E.tolist(), [g.tolist() for g in G]))
        else:
            assert got is None
            out.put(("ids", sorted(ids)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_strong_scaling_evaluation():
    from tyxonq_gb300.workloads import batched_vqe

    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    msgs = [q.get(), q.get()]
    root = [m for m in msgs if m[0] != "ids"][0]
    other = [m for m in msgs if m[0] == "ids"][0]
    t, ids0, E, G = root
    assert t == 2.5
    # the two shards partition the workload
    assert sorted(ids0 + other[1]) == list(range(14)) and ids0 and other[1]
    insts = batched_vqe(14, seed=11, n_range=(3, 8), depth_range=(1, 3), terms_range=(5, 30))
    for k, inst in enumerate(insts):
        e, g = _oracle_eval(inst)
        assert E[k] == e
        np.testing.assert_array_equal(G[k], g)


@pytest.mark.parametrize("world", [1])
def test_single_rank_passthrough(world):
    assert max_over_ranks(3.0) == 3.0
    np.testing.assert_array_equal(gather_results(np.array([1.0, 2.0])), [1.0, 2.0])


def test_multi_rank_report_line(capsys):
    """The report line of a multi-rank benchmark run: rank 0 prints one JSON
    line with the scaled headline, e2e and the contract's keys; other ranks
    print nothing."""
    import json
    import sys
    from pathlib import Path
    from types import SimpleNamespace

    import torch

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench

    from tyxonq_gb300.batch import Schedule

    args = SimpleNamespace(steps=5, warmup=3, scaling="weak", count=4096)
    bv = SimpleNamespace(sched=Schedule.builtin(torch.complex64), kernel_launches=lambda: 100)
    clk = SimpleNamespace(summary=lambda: {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 3})
    prof = {"adjoint": {"gbs": 1200.0, "frac_of_l2_copy": 0.18}}
    bench._print_scaled_line(args, 1, 2, 1.0, 2.0, 3.0, 8, 16, bv, [0] * 4096, 1.0, clk, prof, 6800.0)
    assert capsys.readouterr().out == ""
    bench._print_scaled_line(args, 0, 2, 35000.0, 234.0, 34900.0, 8, 16, bv, [0] * 4096, 1.0, clk, prof, 6800.0)
    line = json.loads(capsys.readouterr().out.strip())
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "clocks", "gpu_launches"):
        assert k in line, k
    assert line["n_gpus"] == 2 and line["value"] == 35000.0 and line["gpu_launches"] == 500
