"""Site-pattern sharding across GPUs (one process per GPU).

The scoring path shards by site pattern: patterns are independent, and the
only exchange is a sum of per-tree scalars -- the u64 Fitch total and the
FP64 log-likelihood.  These helpers split the patterns into contiguous
blocks, one per rank, and combine the per-rank results with one small
collective; the log-likelihood sum is done in rank order with Neumaier's
compensation, so every rank gets the same, deterministic value.
"""
from __future__ import annotations


def pattern_shards(n_pat: int, world: int) -> list[tuple[int, int]]:
    """Contiguous [start, stop) blocks, sizes differing by at most one."""
    if world < 1:
        raise ValueError("world must be >= 1")
    base, extra = divmod(n_pat, world)
    out, start = [], 0
    for r in range(world):
        stop = start + base + (1 if r < extra else 0)
        out.append((start, stop))
        start = stop
    return out


def neumaier(values) -> float:
    s = c = 0.0
    for v in values:
        t = s + v
        c += (s - t) + v if abs(s) >= abs(v) else (v - t) + s
        s = t
    return s + c


def allreduce_lnl(local: float, group=None) -> float:
    """Sum of every rank's log-likelihood, in rank order, compensated."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    t = torch.tensor([local], dtype=torch.float64)
    parts = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    return neumaier(float(p.item()) for p in parts)


def allreduce_count(local: int, group=None) -> int:
    """Sum of every rank's integer count (Fitch totals)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([int(local)], dtype=torch.int64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return int(t.item())


def max_over_ranks(x: float, device=None, group=None) -> float:
    """The largest value over the ranks (the job's time is the slowest rank's)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
