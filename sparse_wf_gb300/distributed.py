"""Walker sharding across ranks (one process per GPU).

Walkers are independent, so the hot path shards them with no data-path collective (the reference
pmaps over walkers, ``update.py:111, 221-222``).  The only exchange is the batch statistic of E_loc
(``update.py:130-134``): an all-reduce of (sum E, sum E^2, N) in FP64.
"""
from __future__ import annotations

import math


def shard(n_total: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of this rank's walkers; the first n_total % world ranks get one extra."""
    base, extra = divmod(n_total, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def energy_stats(e_local, group=None):
    """(mean, std) of E_loc over all ranks' walkers, reduced in FP64 (population std, update.py:130-134)."""
    import torch
    import torch.distributed as dist

    e = e_local.to(torch.float64)
    v = torch.stack([e.sum(), (e * e).sum(), torch.tensor(float(e.numel()), dtype=torch.float64, device=e.device)])
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(v, group=group)
    s, s2, n = (float(x) for x in v.cpu())
    mean = s / n
    return mean, math.sqrt(max(s2 / n - mean * mean, 0.0))
