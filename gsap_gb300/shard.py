"""Scene sharding across ranks (one process per GPU).

Batched scenes are independent, so N ranks split the scene list into N
contiguous ranges of about equal object count and run the batched pipeline
on their own range with no collective on the data path; only the final
counts/timings are reduced.  A single scene does not shard (the reference's
and this broadphase's unit of work is one whole scene): N GPUs then run N
independent replicas.
"""
from __future__ import annotations

import numpy as np


def shard_scenes(offsets, world: int, rank: int):
    """Contiguous scene range [s0, s1) of `rank` balancing object counts.

    offsets: S+1 scene starts (offsets[0] = 0, offsets[S] = n).  Every scene
    goes to exactly one rank; ranks may get no scene when S < world.
    """
    off = np.asarray(offsets, dtype=np.int64)
    S = len(off) - 1
    if world <= 1:
        return 0, S
    n = int(off[-1])
    # rank r takes the scenes whose start lies in [r n / world, (r+1) n / world)
    bounds = [int(np.searchsorted(off[:-1], (r * n) // world, side="left")) for r in range(world)] + [S]
    bounds[0] = 0
    for r in range(1, world + 1):
        bounds[r] = max(bounds[r], bounds[r - 1])
    return bounds[rank], bounds[rank + 1]


def local_offsets(offsets, s0: int, s1: int):
    """Offsets of the scenes [s0, s1) rebased to start at 0, and the global
    id of the first object (add it to local pair ids)."""
    off = np.asarray(offsets, dtype=np.int64)
    base = int(off[s0])
    return (off[s0:s1 + 1] - base).astype(np.int64), base
