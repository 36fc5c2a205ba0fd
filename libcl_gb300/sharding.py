"""Multi-GPU layout of the workloads: the plain step does not shard (one scene is one
coupled particle system), so N GPUs run N independent replicas; a batch of independent
scenes is split into contiguous per-rank ranges balanced by particle count, with no
collective on the data path. The only collective is the timing reduction (max over ranks).
"""
from __future__ import annotations


def scene_shards(counts, world: int) -> list[tuple[int, int]]:
    """Contiguous [first, last) scene ranges, one per rank, that split the total particle
    count as evenly as a contiguous split allows (greedy on the running prefix: rank r ends
    at the first scene whose prefix reaches (r + 1) / world of the total). Every scene is in
    exactly one range; a range may be empty when there are fewer scenes than ranks."""
    if world < 1:
        raise ValueError("world must be >= 1")
    counts = [int(c) for c in counts]
    total = sum(counts)
    bounds, prefix, s = [0], 0, 0
    for r in range(1, world):
        target = total * r / world
        while s < len(counts) and prefix + counts[s] / 2 <= target:
            prefix += counts[s]
            s += 1
        bounds.append(max(s, bounds[-1]))
    bounds.append(len(counts))
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over the ranks of the default process group (the value itself
    without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
