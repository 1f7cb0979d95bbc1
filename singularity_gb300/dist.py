"""Multi-GPU host logic: one process per GPU, work sharded with no data-path
collective.

Every (pixel, sample) ray is independent, so the units shard by view (a frame
per rank, or the views of a batch split by cost across ranks); the only
collective is the max over ranks of the timed region, and, when a caller wants
one image, a gather at the end.  Used by ``bench.py`` under torchrun; the
functions take plain values so they are testable with the gloo backend on CPU.
"""

from __future__ import annotations

import math
import os
from typing import List, Sequence


def env_rank() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment (1 process: 0, 1, 0)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def view_azimuth(rank: int, world: int) -> float:
    """Camera azimuth of rank's frame in the weak-scaling bench: the orbit split evenly."""
    return 2.0 * math.pi * rank / max(1, world)


def view_cost(width: int, height: int, spp: int) -> float:
    """Estimated cost of a view: its rays (steps per ray vary far less across the
    batch's views than their ray counts do)."""
    return float(width) * float(height) * float(max(1, min(1024, spp)))


def split_by_cost(costs: Sequence[float], world: int) -> List[List[int]]:
    """Longest-processing-time split of items across `world` ranks: items in
    decreasing cost, each to the currently lightest rank (ties to the lower
    rank).  Deterministic; every item appears exactly once; within a rank the
    items keep their original order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def imbalance(costs: Sequence[float], parts: Sequence[Sequence[int]]) -> float:
    """max rank load / mean rank load (1.0 = perfect balance)."""
    loads = [sum(costs[i] for i in p) for p in parts]
    mean = sum(loads) / max(1, len(loads))
    return max(loads) / mean if mean > 0 else 1.0


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over the process group (the timed region's
    duration: the job ends with its slowest rank).  Without an initialised
    group, the value itself."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    """The sum of `value` over the process group (e.g. rays traced by all ranks)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds_per_rank: float, device=None) -> float:
    """Whole-job throughput: units all ranks processed / the slowest rank's time."""
    total = sum_over_ranks(units_per_rank, device)
    slowest = max_over_ranks(seconds_per_rank, device)
    return total / slowest if slowest > 0 else 0.0


__all__ = ["env_rank", "view_azimuth", "view_cost", "split_by_cost", "imbalance", "max_over_ranks",
           "sum_over_ranks", "whole_job_rate"]
