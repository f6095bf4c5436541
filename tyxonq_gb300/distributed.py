"""Instance sharding across ranks (one process per GPU).

VQE instances are independent, so N GPUs evaluate disjoint shards with no
data-path collective: each rank builds and runs its own BatchedVQE; the only
communication is a barrier, the MAX of the step time, and (optionally) a
gather of energies / gradients to rank 0 on the host.  A single statevector
is not sharded (replicas only).  Works with NCCL on GPUs and gloo on CPU.
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
