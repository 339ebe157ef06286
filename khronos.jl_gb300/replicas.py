"""Replicas across GPUs: independent simulations per rank, no domain decomposition.

The step loop runs on one GPU with no halo exchange (the reference shards one
grid into chunks and exchanges halos over NCCL, src/Distributed.jl:448-506;
that decomposition is not rebuilt).  Several GPUs serve independent work:
each rank (one process per GPU, launched by torchrun) steps its own
simulations, and the only collective is on the host side of a measurement —
a barrier around the timed region and the maximum of the ranks' times.

* ``shard``          deterministic assignment of independent requests to ranks,
                     balancing their cell-updates (longest first, to the least
                     loaded rank); every rank computes the same plan locally
* ``max_over_ranks`` the slowest rank's value (all_reduce MAX; gloo or NCCL)
* ``aggregate_rate`` whole-job units per second over the slowest rank's time
"""
from __future__ import annotations

import heapq
from typing import List, Optional, Sequence


def shard(work: Sequence[float], world: int, rank: int) -> List[int]:
    """Indices of the items `rank` owns: items in decreasing work (ties by
    index) go to the rank with the least work so far (ties by rank)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    order = sorted(range(len(work)), key=lambda i: (-float(work[i]), i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    owned: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        owned[r].append(i)
        heapq.heappush(heap, (load + float(work[i]), r))
    return sorted(owned[rank])


def max_over_ranks(value: float, dist=None, device: Optional[str] = None) -> float:
    """max of `value` over the ranks of the default process group (the value
    itself without one).  `device` is where the reduction tensor lives: "cpu"
    for gloo, "cuda" for NCCL."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput when every rank processes `units_per_rank` and the
    slowest takes `seconds_max` (weak scaling: per-rank work fixed)."""
    if seconds_max <= 0:
        raise ValueError("the timed region must be positive")
    return world * float(units_per_rank) / float(seconds_max)
