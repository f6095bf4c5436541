"""Instance sharding across ranks (one process per GPU).

VQE instances are independent, so N GPUs evaluate disjoint shards with no
data-path collective: each rank builds and runs its own BatchedVQE; the only
communication is a barrier, the MAX of the step time, and (optionally) a
gather of energies / gradients to rank 0 on the host.  A single statevector
is not sharded (replicas only).  Works with NCCL on GPUs and gloo on CPU.

Two splits: weak scaling (every rank evaluates its own workload of fixed
size) and strong scaling (one workload split by estimated cost with
``cost_balanced_shards``; ``gather_instances`` puts the energies and gradients
back in instance order on rank 0).
"""
from __future__ import annotations

import numpy as np
import torch
import torch.distributed as dist


def shard_range(count: int, rank: int, world: int) -> range:
    """Contiguous, balanced shard of `count` items for `rank` of `world`."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank / world size")
    base, extra = divmod(count, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def cost_balanced_shards(costs, world: int) -> list[list[int]]:
    """Greedy longest-first assignment of items to ranks by cost (deterministic)."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    loads = [0.0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        out[r].append(i)
        loads[r] += costs[i]
    return [sorted(s) for s in out]


def instance_cost(inst) -> float:
    """Estimated device work of one VQE instance: amplitudes x (gates for the
    forward and reverse sweeps + Pauli terms of H psi)."""
    return float(1 << int(inst.n)) * (3 * len(inst.structure()) + int(inst.H.n_terms))


def shard_instances(instances, rank: int, world: int) -> list[int]:
    """Indices of the instances rank `rank` evaluates in a strong-scaling split."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank / world size")
    return cost_balanced_shards([instance_cost(i) for i in instances], world)[rank]


def gather_instances(ids, energies, grads: list, count: int, device=None):
    """Energies and per-instance gradients of every rank's shard, reassembled in
    instance order on rank 0: (energies[count], [gradient per instance]); None
    on other ranks.  ids: this rank's instance indices; grads: one array each."""
    ids = np.asarray(ids, dtype=np.float64)
    lens = np.array([len(g) for g in grads], dtype=np.float64)
    flat = np.concatenate([np.asarray(g, dtype=np.float64) for g in grads]) if len(grads) else np.zeros(0)
    head = np.concatenate([ids, lens, np.asarray(energies, dtype=np.float64)])
    heads = _gather_parts(head, device)
    flats = _gather_parts(flat, device)
    if heads is None:
        return None
    E = np.full(count, np.nan)
    G: list = [None] * count
    for h, f in zip(heads, flats):
        k = len(h) // 3  # [ids, lens, energies] of k instances
        o = 0
        for i, ln, e in zip(h[:k], h[k:2 * k], h[2 * k:]):
            E[int(i)] = e
            G[int(i)] = f[o:o + int(ln)]
            o += int(ln)
    return E, G


def _gather_parts(local: np.ndarray, device=None) -> list | None:
    """Every rank's 1-D float64 array on rank 0, as a list in rank order (None elsewhere)."""
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return [np.asarray(local, dtype=np.float64)]
    world = dist.get_world_size()
    n = torch.tensor([len(local)], dtype=torch.int64, device=device)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n)
    m = max(1, int(max(int(x.item()) for x in sizes)))
    buf = torch.zeros(m, dtype=torch.float64, device=device)
    buf[: len(local)] = torch.as_tensor(np.asarray(local, dtype=np.float64), device=device)
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    if dist.get_rank() != 0:
        return None
    return [x[: int(c.item())].cpu().numpy() for x, c in zip(parts, sizes)]


def max_over_ranks(value: float, device=None) -> float:
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_results(local: np.ndarray, device=None) -> np.ndarray | None:
    """Concatenate every rank's 1-D result on rank 0 (None on other ranks)."""
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return np.asarray(local)
    world = dist.get_world_size()
    n = torch.tensor([len(local)], dtype=torch.int64, device=device)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n)
    m = int(max(int(s.item()) for s in sizes))
    buf = torch.zeros(m, dtype=torch.float64, device=device)
    buf[: len(local)] = torch.as_tensor(np.asarray(local, dtype=np.float64), device=device)
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    if dist.get_rank() != 0:
        return None
    return np.concatenate([p[: int(s.item())].cpu().numpy() for p, s in zip(parts, sizes)])
