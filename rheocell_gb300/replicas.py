"""Host-side logic of multi-GPU runs.

A single monolayer is not sharded (one GPU per monolayer, as the path is
defined); N GPUs run N independent replicas or, for an ensemble of monolayers,
disjoint contiguous blocks of it.  There is no data-path collective: ranks
only meet at a barrier around the timed region and in one reduction of the
timing and of the units processed.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple


def shard(items: Sequence, rank: int, world: int) -> List:
    """Contiguous block of `items` owned by `rank` (sizes differ by at most one)."""
    n = len(items)
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return list(items[lo:hi])


def reduce_timing(ms: float, units: float) -> Tuple[float, float]:
    """(max over ranks of ms, sum over ranks of units) with torch.distributed;
    identity when no process group is initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return ms, units
    t = torch.tensor([ms], dtype=torch.float64)
    u = torch.tensor([units], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
