"""Sharding a request across ranks (one process per GPU).

Events are independent and each event's random stream is keyed by (seed, event index), so a
request of n events splits into contiguous event ranges with no communication: rank r produces
events [first_r, first_r + n_r) exactly as a single process would.  Generate needs no exchange;
AverageOn needs one: every rank contributes its 24-byte StatsPHSP (mean, M2, W) and all ranks
merge them in rank order with AddStatsPHSP (hydra/detail/functors/StatsPHSP.h:67-84), so every
rank holds the same result.
"""
from __future__ import annotations

from typing import Callable, Sequence


def event_range(rank: int, world: int, n: int, first: int = 0) -> tuple[int, int]:
    """(first event, count) of rank `rank` out of `world` for events [first, first + n)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    lo = n * rank // world
    hi = n * (rank + 1) // world
    return first + lo, hi - lo


def stats_merge(x: Sequence[float], y: Sequence[float]) -> tuple[float, float, float]:
    """AddStatsPHSP on (mean, M2, W) triples; two empty partials merge to the left one."""
    w = x[2] + y[2]
    if w == 0.0:
        return (x[0], x[1], x[2])
    delta = y[0] - x[0]
    mean = (x[0] * x[2] + y[0] * y[2]) / w
    m2 = x[1] + y[1]
    m2 += delta * delta * x[2] * y[2] / w
    return (mean, m2, w)


def merge_in_order(parts: Sequence[Sequence[float]]) -> tuple[float, float, float]:
    acc = (0.0, 0.0, 0.0)
    for p in parts:
        acc = stats_merge(acc, p)
    return acc


def average_on_sharded(n: int, first: int, compute: Callable[[int, int], Sequence[float]], group=None):
    """AverageOn of events [first, first + n) over the ranks of `group` (torch.distributed).

    `compute(first_r, n_r)` returns this rank's (mean, M2, W) -- on a GPU rank that is
    hps_average_on on its own device.  Returns the merged (mean, M2, W), identical on every rank.
    """
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    f, m = event_range(rank, world, n, first)
    mine = torch.tensor(list(compute(f, m)), dtype=torch.float64)
    backend = dist.get_backend(group)
    if backend == "nccl":
        mine = mine.cuda()
    gathered = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(gathered, mine, group=group)
    return merge_in_order([tuple(t.cpu().tolist()) for t in gathered])
