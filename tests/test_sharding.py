"""Host-side multi-GPU logic on CPU: instance placement and the cross-rank
reductions, run as two gloo ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from domain_transform_solver_gb300 import sharding
from domain_transform_solver_gb300 import workloads as W


def test_partition_covers_every_instance_once_and_balances():
    sizes = W.batched_sizes()
    for world in (1, 2, 3, 4, 8):
        parts = sharding.partition_lpt(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i][0] * sizes[i][1] for i in p) for p in parts]
        biggest = max(w * h for w, h in sizes)
        assert max(loads) - min(loads) <= biggest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = W.batched_sizes()
        mine = sharding.partition_lpt(sizes, world)[rank]
        pixels = sum(sizes[i][0] * sizes[i][1] for i in mine)
        # a rank's "step time" proportional to its pixels
        t = sharding.max_over_ranks(pixels * 1e-6, device="cpu")
        total = sharding.sum_over_ranks(pixels, device="cpu")
        q.put((rank, sorted(mine), t, total))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_two_gloo_ranks_agree_on_placement_and_reductions(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sizes = W.batched_sizes()
    parts = sharding.partition_lpt(sizes, world)
    res.sort()
    allpix = sum(w * h for w, h in sizes)
    for rank, mine, t, total in res:
        assert mine == parts[rank]
        assert total == allpix
        assert t == max(sum(sizes[i][0] * sizes[i][1] for i in p) for p in parts) * 1e-6


def _gather_worker(rank, world, port, q):
    """Each rank solves its share of a small ragged batch with the FP32
    oracle port (standing in for the per-rank GPU solve) and rank 0 gathers
    the results."""
    import sys
    from pathlib import Path
    import torch.distributed as dist
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        insts = W.batched_instances(n=7, scale=0.06)
        seen = []

        def solve(share):
            seen.extend((i.width, i.height) for i in share)
            return [O.dts_solve(i.rgba, i.target, i.confidence, 1, W.CFG0_FILTER,
                                dict(W.CFG0_OPT, num_iterations=3), real="f32")[0]
                    for i in share]

        out = sharding.solve_sharded(insts, solve)
        q.put((rank, seen, None if out is None else [o.tobytes() for o in out]))
    finally:
        dist.destroy_process_group()


def test_partition_solve_gather_on_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gather_worker, args=(r, world, port, q))
             for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import oracle as O
    insts = W.batched_instances(n=7, scale=0.06)
    sizes = [(i.width, i.height) for i in insts]
    parts = sharding.partition_lpt(sizes, world)
    (r0, seen0, out0), (r1, seen1, out1) = res
    assert out1 is None and out0 is not None
    assert seen0 == [sizes[i] for i in parts[0]] and seen1 == [sizes[i] for i in parts[1]]
    for inst, got in zip(insts, out0):
        ref = O.dts_solve(inst.rgba, inst.target, inst.confidence, 1, W.CFG0_FILTER,
                          dict(W.CFG0_OPT, num_iterations=3), real="f32")[0]
        assert got == ref.tobytes()


def test_solve_sharded_without_a_process_group_solves_everything():
    insts = W.batched_instances(n=3, scale=0.05)
    out = sharding.solve_sharded(insts, lambda share: [i.width * i.height for i in share])
    assert out == [i.width * i.height for i in insts]
