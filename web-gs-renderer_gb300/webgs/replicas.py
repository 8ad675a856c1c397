"""Replica parallelism: views (and scenes) are independent units of the splat pipeline, so several
GPUs each render their own share with no exchange on the data path. One process per GPU; the only
collectives are for bookkeeping (gathering results, the slowest rank's time), on any torch.distributed
backend (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

import heapq
from typing import Callable, Sequence


def view_cost(width: int, height: int, count: int) -> float:
    """Relative cost of one view: pixels (raster) plus Gaussians (preprocess, binning)."""
    return float(width) * float(height) + 2.0 * float(count)


def shard(costs: Sequence[float], world: int) -> list[list[int]]:
    """Longest-processing-time assignment of views to ranks: deterministic, every view exactly once,
    each rank's list in ascending view order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    heap = [(0.0, r) for r in range(world)]
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(s) for s in out]


def max_over_ranks(value: float) -> float:
    """The largest value over all ranks (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return value
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def render_sharded(render: Callable[[int], object], costs: Sequence[float], rank: int, world: int) -> dict:
    """Renders this rank's share (render(i) for each assigned view i) and gathers every rank's results
    into {view index: result} on all ranks."""
    mine = {i: render(i) for i in shard(costs, world)[rank]}
    if world == 1:
        return mine
    import torch.distributed as dist

    parts: list = [None] * world
    dist.all_gather_object(parts, mine)
    merged: dict = {}
    for p in parts:
        merged.update(p)
    return merged
