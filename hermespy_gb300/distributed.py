"""Drop sharding across ranks (one process per GPU).

Drops are independent (the reference already runs them per actor,
core/pymonte/actors.py:367-452) and every random draw is a Philox stream of
(campaign seed, drop index, stream id), so a rank simulates exactly the drops of its
index range and the union over ranks equals a single-process run. The only exchange
is at the end: integer counters (bit errors, bits, drops per noise level) summed over
ranks, and the slowest rank's time for throughput. There is no data-path collective.
"""

from __future__ import annotations

import numpy as np
import torch


def shard(total: int, rank: int, world: int) -> tuple[int, int]:
    """(first drop, drop count) of `rank`: [rank n / G, (rank + 1) n / G)."""

    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("shard: need 0 <= rank < world and total >= 0")
    lo = (total * rank) // world
    hi = (total * (rank + 1)) // world
    return lo, hi - lo


def rank_base(rank: int, bits: int = 44) -> int:
    """Disjoint drop-index space of a rank for open-ended runs (rank << bits)."""

    return int(rank) << bits


def sum_counters(counters, group=None) -> np.ndarray:
    """Sum int64 counters (per noise level: errors, bits, drops) over all ranks."""

    import torch.distributed as dist

    t = torch.as_tensor(np.asarray(counters, dtype=np.int64))
    if dist.is_available() and dist.is_initialized():
        dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
        t = t.to(dev)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def max_over_ranks(value: float, group=None) -> float:
    """The largest value over ranks (the slowest rank's time)."""

    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
