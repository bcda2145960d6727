"""Multi-GPU placement of independent traps (one process per GPU).

Traps never exchange data, so a multi-GPU run needs no data-path collective:
* weak scaling (the default of bench.py): every rank steps its own batch, seeded
  by rank, so per-GPU work is fixed as the GPU count grows;
* strong scaling: one workload is split into per-rank shards of whole traps,
  balanced by node count (largest-first greedy onto the least-loaded rank).
The only collectives are the host-side barrier and the max-over-ranks reduction
of the timed region, through whatever torch.distributed backend is initialised
(NCCL on GPUs, gloo in the CPU tests).
"""
from __future__ import annotations

from typing import List, Sequence


def balanced_shards(weights: Sequence[int], world: int) -> List[List[int]]:
    """Deterministic partition of item indices into `world` shards of similar weight."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(weights)), key=lambda i: (-int(weights[i]), i))
    load = [0] * world
    shards: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        shards[r].append(i)
        load[r] += int(weights[i])
    return [sorted(s) for s in shards]


def rank_seed(base_seed: int, rank: int) -> int:
    """Workload seed of a rank in weak-scaling runs."""
    return base_seed + rank


def max_over_ranks(value: float) -> float:
    """Max of a float over the ranks of the default process group (or itself)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
