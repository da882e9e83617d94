"""Replica sharding for more than one GPU (one process per GPU).

Frames are independent, so N GPUs run N replicas with no collective on the
data path: the batched scenes are dealt to ranks by a greedy
longest-processing-time partition of an estimated cost (triangles, map
texels of every light, camera pixels per light), and only timings are
reduced (max over ranks).
"""
from __future__ import annotations


def frame_cost(triangles: int, map_sides, camera_pixels: int) -> float:
    """Estimated work of one batched frame: T + sum of S^2 + L * P."""
    return float(triangles) + float(sum(s * s for s in map_sides)) + len(map_sides) * float(camera_pixels)


def partition_by_cost(costs, world: int) -> list[list[int]]:
    """Greedy LPT: items in decreasing cost, each to the currently lightest
    rank (ties to the lowest rank).  Deterministic; every rank computes the
    same partition.  Load of the heaviest rank <= 4/3 of optimal."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    loads = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += costs[i]
    for p in parts:
        p.sort()
    return parts


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Max of a per-rank float over the process group (identity without one)."""
    if dist is None or not dist.is_initialized():
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
