"""Sharding a ray batch over ranks (one process per GPU).

Rays are independent, so a batch splits into contiguous ranges with no
exchange on the data path.  The split is the reference's thread split
(src/AOpticsManager.cxx:533-541): rank i takes [q*i, q*(i+1)) with
q = n // world, and the last rank also takes the remainder.  Each shard is
traced with ray_id_offset = its start, so every random draw (keyed by
seed and global ray id) and therefore every result is the same as in an
unsharded trace of the whole batch.

The one exchange a user needs afterwards is a sum of per-group
accumulators (focused count, sum x, sum y, sum x^2, sum y^2, sum t; or the
bins of a focal-plane histogram), done with one all_reduce on whatever
process group is active (NCCL on GPUs, gloo on host tensors).
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np


def shard_range(n: int, rank: int, world: int) -> Tuple[int, int]:
    """[start, stop) of rank `rank` among `world` ranks over n rays."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError(f"bad shard request n={n} rank={rank} world={world}")
    q = n // world
    start = q * rank
    stop = n if rank == world - 1 else q * (rank + 1)
    return start, stop


def shard_batch(batch: Dict[str, np.ndarray], rank: int, world: int):
    """The rank's slice of a batch of per-ray arrays and its first ray id."""
    n = len(next(iter(batch.values())))
    start, stop = shard_range(n, rank, world)
    return {k: v[start:stop] for k, v in batch.items()}, start


def allreduce_sum(t):
    """Sum a tensor over the ranks of the default process group in place
    (no-op when torch.distributed is not initialised or has one rank)."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t


def spot_from_moments(sums) -> np.ndarray:
    """Per-group (count, mean x, mean y, RMS radius, mean t) from summed
    moments rows (count, sum x, sum y, sum x^2, sum y^2, sum t), the spot
    size and plate position of tutorials/SchwarzschildCouder.C:133-161."""
    s = np.asarray(sums, dtype=np.float64).reshape(-1, 6)
    out = np.full((s.shape[0], 5), np.nan)
    for g, (c, sx, sy, sxx, syy, st) in enumerate(s):
        if c <= 0:
            out[g, 0] = 0
            continue
        mx, my = sx / c, sy / c
        var = max(sxx / c - mx * mx, 0.0) + max(syy / c - my * my, 0.0)
        out[g] = (c, mx, my, np.sqrt(var), st / c)
    return out
