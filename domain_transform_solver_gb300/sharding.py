"""Multi-GPU placement of independent solves.

The DTS and HFBS solves of different images (and of the two HFBS chroma
channels) share nothing, so several GPUs split a batch by instance with no
data-path collective: one process per GPU takes its share, solves it, and
only the host gathers results.  This module holds the placement rule, the
partition-solve-gather flow (solve_sharded, with batch_solver as the
per-rank GPU solve) and the two host-side reductions the benchmark uses;
the tests run them on CPU with the gloo backend.
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


def solve_sharded(instances, solve, rank: int | None = None, world: int | None = None,
                  dst: int = 0):
    """Solve a batch split over the ranks of the default process group.

    instances: every rank's identical list of instances (anything with
    .width and .height).  Each rank passes its share (partition_lpt) to
    solve(list) -> list of results, one per instance, in order.  The
    results travel to rank dst only (gather_object: a host-side exchange
    after the solves, none inside them), which returns them in instance
    order; the other ranks return None.  Without an initialised process
    group (or world 1) the whole batch is solved here."""
    import torch.distributed as dist
    grouped = dist.is_available() and dist.is_initialized()
    if world is None:
        world = dist.get_world_size() if grouped else 1
    if rank is None:
        rank = dist.get_rank() if grouped else 0
    sizes = [(i.width, i.height) for i in instances]
    mine = partition_lpt(sizes, world)[rank]
    results = list(solve([instances[i] for i in mine])) if mine else []
    if len(results) != len(mine):
        raise ValueError("solve returned a different number of results")
    if world == 1:
        return results
    gathered = [None] * world if rank == dst else None
    dist.gather_object(list(zip(mine, results)), gathered, dst=dst)
    if rank != dst:
        return None
    out = [None] * len(instances)
    for part in gathered:
        for i, r in part:
            out[i] = r
    return out


def batch_solver(filter_params=None, optimize_params=None, grid_params=None,
                 color_space=None, flags: int = 0):
    """A solve(list) for solve_sharded on this rank's GPU: one Batch of the
    share, DTS and/or HFBS, results downloaded as (dts, hfbs) pairs (None
    for a solver not run)."""
    def solve(insts):
        from . import solvers as S
        cs = S.COLOR_SPACE.YCbCr if color_space is None else color_space
        b = S.Batch([(i.width, i.height) for i in insts], flags=flags)
        try:
            b.upload(cs, [i.rgba for i in insts], [i.target for i in insts],
                     [i.confidence for i in insts])
            d = h = [None] * len(insts)
            if optimize_params is not None:
                b.solve_dts(filter_params, optimize_params)
                d = b.download(0)
            if grid_params is not None:
                b.solve_hfbs(grid_params)
                h = b.download(1)
            return list(zip(d, h))
        finally:
            b.close()
    return solve


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
