"""Partitioning an ensemble of independent systems across ranks (one GPU per rank).

Systems do not interact, so the only multi-GPU structure is a partition of the systems: no
collective touches the data path.  `shard` assigns systems to ranks greedily by estimated cost
(largest first onto the least-loaded rank), deterministically, so every rank computes the same
partition without communicating.  `gather` collects per-system results on every rank (used
only after the timed region, for checks and reporting).
"""
from __future__ import annotations

import math


def system_cost(n_particles: int, mesh_cells: int) -> float:
    """Per-step cost model: particle work plus an FFT term for the mesh."""
    return float(n_particles) + 2.0 * mesh_cells * max(1.0, math.log2(max(mesh_cells, 2)) / 10.0)


def shard(costs, world: int):
    """List of system indices per rank (deterministic greedy longest-processing-time)."""
    if world < 1:
        raise ValueError("world size must be positive")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def gather(local: dict, world: int):
    """All ranks' {system index: result} merged (torch.distributed object all-gather)."""
    if world == 1:
        return dict(local)
    import torch.distributed as dist
    buf = [None] * world
    dist.all_gather_object(buf, local)
    merged = {}
    for part in buf:
        merged.update(part)
    return merged
