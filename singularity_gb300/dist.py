"""Multi-GPU host logic: one process per GPU, work sharded with no data-path
collective.

Every (pixel, sample) ray is independent, so the units shard three ways:
  * one frame split across ranks (the reference parallelises one frame over
    pixels, render/cuda/cuda_backend.cu:145-147): the rows are dealt in bands
    of ``band`` rows round-robin, band b to rank b % N, so every rank gets
    rows from the whole height (the disc and the shadow are not spread evenly
    over the frame); each rank traces its slice through ``sgx_render_device``
    with ``opts.slice_*`` and a gather to rank 0 puts the rows back; every
    pixel is computed exactly as in a one-GPU render, in the reference's
    per-pixel sample order, so the assembled frame equals it bit for bit;
  * a frame per rank (replicas, weak scaling);
  * the views of a batch split by cost across ranks.
The only collectives are the gather of a split frame and the max over ranks of
the timed region.  Used by ``bench.py`` under torchrun; the functions take
plain values so they are testable with the gloo backend on CPU.
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


SLICE_BAND_DEFAULT = 8  # rows per band (the C ABI's SGX_SLICE_BAND_DEFAULT)


def slice_rows(height: int, band: int, count: int, index: int) -> int:
    """Rows of slice `index` of `count` in a frame of `height` rows (bands of
    `band` rows, band b to slice b % count); the C ABI's sgx_slice_rows."""
    band = band or SLICE_BAND_DEFAULT
    if count <= 1:
        return height if index == 0 else 0
    if index >= count:
        return 0
    bands = -(-height // band)
    mine = range(index, bands, count)
    return sum(min(band, height - b * band) for b in mine)


def slice_row_indices(height: int, band: int, count: int, index: int):
    """The frame rows of slice `index`, top to bottom (numpy int64 array)."""
    import numpy as np
    band = band or SLICE_BAND_DEFAULT
    if count <= 1:
        return np.arange(height if index == 0 else 0, dtype=np.int64)
    if index >= count:
        return np.zeros(0, dtype=np.int64)
    bands = -(-height // band)
    rows = [np.arange(b * band, min(height, (b + 1) * band), dtype=np.int64) for b in range(index, bands, count)]
    return np.concatenate(rows) if rows else np.zeros(0, dtype=np.int64)


def assemble_slices(slices, height: int, band: int):
    """The whole frame from all `count = len(slices)` slices (each
    [rows, width, ...], numpy or torch), rows put back in frame order."""
    count = len(slices)
    first = slices[0]
    shape = (height,) + tuple(first.shape[1:])
    if hasattr(first, "new_empty"):  # torch
        import torch
        out = first.new_empty(shape)
        for i, sl in enumerate(slices):
            idx = torch.as_tensor(slice_row_indices(height, band, count, i), device=sl.device)
            out[idx] = sl
        return out
    import numpy as np
    out = np.empty(shape, dtype=first.dtype)
    for i, sl in enumerate(slices):
        out[slice_row_indices(height, band, count, i)] = sl
    return out


def gather_frame(local_slice, height: int, band: int):
    """Gathers every rank's slice of one frame to rank 0 and assembles it.

    local_slice: this rank's [rows, width, ...] tensor (a CUDA tensor under
    NCCL, a CPU tensor under gloo).  The collective is ordered after the
    work queued on torch's current stream: a slice rendered on another stream
    must be waited for first (`torch.cuda.current_stream().wait_stream(s)`).
    Slices differ in rows by at most one
    band, so each is padded to the largest for the collective.  Returns the
    [height, width, ...] frame on rank 0 and None on the other ranks; with
    no initialised group (one process), the slice itself."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local_slice
    world, rank = dist.get_world_size(), dist.get_rank()
    rows = [slice_rows(height, band, world, i) for i in range(world)]
    pad = max(rows)
    buf = local_slice.new_zeros((pad,) + tuple(local_slice.shape[1:]))
    buf[: local_slice.shape[0]] = local_slice
    bufs = [torch.empty_like(buf) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, bufs, dst=0)
    if rank != 0:
        return None
    return assemble_slices([b[:r] for b, r in zip(bufs, rows)], height, band)


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


__all__ = ["env_rank", "view_azimuth", "view_cost", "split_by_cost", "imbalance", "SLICE_BAND_DEFAULT",
           "slice_rows", "slice_row_indices", "assemble_slices", "gather_frame", "max_over_ranks",
           "sum_over_ranks", "whole_job_rate"]
