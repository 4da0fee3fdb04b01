"""Multi-GPU bookkeeping for independent replicas / ensemble shards.

A single cavity case does not shard (per-sweep halos, global max-norm tests
and domain-long chain recurrences), so N GPUs run N independent replicas;
an ensemble of independent instances is partitioned across ranks with no
data-path exchange.  The only collectives are the timing barrier and the
max-over-ranks reduction of the elapsed time.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple


def partition(n_items: int, world: int, rank: int) -> List[int]:
    """Contiguous block of item indices owned by `rank` (sizes differ by at
    most one)."""
    base, extra = divmod(n_items, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return list(range(lo, hi))


def partition_work(weights: Sequence[float], world: int, rank: int) -> List[int]:
    """Item indices owned by `rank` when items of uneven work (an ensemble's
    cases, weighted by cells) are spread over `world` ranks: largest first to
    the least-loaded rank (ties to the lower rank), returned in item order.
    Every rank computes the same assignment."""
    load = [0.0] * world
    owner = [0] * len(weights)
    for i in sorted(range(len(weights)), key=lambda i: (-weights[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += weights[i]
    return [i for i in range(len(weights)) if owner[i] == rank]


def max_over_ranks(values: Tuple[float, ...], device=None) -> Tuple[float, ...]:
    """Element-wise max of per-rank values (identity when not distributed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return tuple(values)
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return tuple(float(x) for x in t.cpu())


def whole_job_rate(units_per_rank: float, world: int, t_max: float) -> float:
    """Throughput of the whole job: all ranks' units over the slowest rank's
    time."""
    return units_per_rank * world / t_max
