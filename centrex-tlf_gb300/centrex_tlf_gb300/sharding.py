"""Trajectory sharding across GPUs (one process per GPU, no collective on the data path).

Trajectories are independent (rust/src/lindblad/ode_batch.rs:270-296 solves them in any order),
so N ranks take disjoint contiguous ranges of a batch and the host gathers the slices; the only
collectives are the timing's barrier and the maximum of the ranks' times.  Weak scaling gives
every rank the same number of trajectories; a mixed batch (plans of different sizes, different
end times) is split by an estimated cost instead (work ∝ packed state length × end time).
"""

from __future__ import annotations

from typing import Sequence

import numpy as np


def shard_bounds(per_rank: int, rank: int) -> tuple[int, int]:
    """[lo, hi) of rank `rank` when every rank solves `per_rank` trajectories (weak scaling)."""
    if per_rank < 0 or rank < 0:
        raise ValueError("per_rank and rank must be non-negative")
    return rank * per_rank, (rank + 1) * per_rank


def cost_balanced_bounds(costs: Sequence[float], world: int) -> list[tuple[int, int]]:
    """Contiguous [lo, hi) ranges, one per rank, whose summed costs are as even as a split at the
    prefix sums' world-quantiles makes them; every index in exactly one range."""
    if world <= 0:
        raise ValueError("world must be positive")
    c = np.asarray(costs, dtype=np.float64).reshape(-1)
    if np.any(c < 0):
        raise ValueError("costs must be non-negative")
    prefix = np.concatenate([[0.0], np.cumsum(c)])
    total = prefix[-1]
    cuts = [0]
    for r in range(1, world):
        cuts.append(int(np.searchsorted(prefix, total * r / world, side="left")) if total > 0 else (c.size * r) // world)
    cuts.append(c.size)
    cuts = np.maximum.accumulate(np.clip(cuts, 0, c.size))
    return [(int(cuts[r]), int(cuts[r + 1])) for r in range(world)]


def trajectory_cost(packed_len: int, t_end: float) -> float:
    """Estimated work of one trajectory: RHS work per step ∝ packed state length, steps ∝ end time."""
    return float(packed_len) * float(t_end)


def max_over_ranks(values: Sequence[float], device=None) -> list[float]:
    """Element-wise maximum of `values` over the ranks of the default process group (identity
    without one): the job's time is its slowest rank's."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]
