"""Multi-GPU placement of independent solves.

The DTS and HFBS solves of different images (and of the two HFBS chroma
channels) share nothing, so several GPUs split a batch by instance with no
data-path collective: one process per GPU takes its share, solves it, and
only the host gathers results.  This module holds the placement rule and
the two host-side reductions the benchmark uses; the tests run them on CPU
with the gloo backend.
"""
from __future__ import annotations

import heapq


def partition_lpt(sizes, world: int) -> list[list[int]]:
    """Split instances (w, h) over `world` ranks by pixel count: longest
    processing time first, each instance to the least loaded rank.  Returns
    the instance indices of each rank, in ascending order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i][0] * sizes[i][1], i))
    heap = [(0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + sizes[i][0] * sizes[i][1], r))
    return [sorted(p) for p in parts]


def max_over_ranks(value: float, device=None) -> float:
    """The slowest rank's value (all ranks get it); the time of a parallel
    step is its slowest rank's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
