"""Batch sharding across GPUs (one rank per GPU, no collective on the data path).

Paths are independent, so N GPUs split a batch into N contiguous groups of
paths and each rank runs the signature kernels on its own group; outputs are
per path, so nothing is exchanged.  For ragged batches the split balances the
number of increments (the work) rather than the number of paths.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(offsets, world: int, rank: int) -> tuple[int, int]:
    """Paths [b0, b1) of `rank` among `world` ranks.  `offsets` (host, int64,
    batch + 1 entries) are the ragged-batch offsets; the cut before rank r is
    the first path whose starting increment reaches r/world of the total.
    Contiguous groups keep each rank's increments contiguous in memory."""
    offsets = np.asarray(offsets, dtype=np.int64)
    batch = len(offsets) - 1
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    total = int(offsets[-1])

    def cut(r: int) -> int:
        if r <= 0:
            return 0
        if r >= world:
            return batch
        target = (total * r + world - 1) // world
        return int(np.searchsorted(offsets[:-1], target, side="left"))

    return cut(rank), cut(rank + 1)


def shard_offsets(offsets, world: int, rank: int):
    """(b0, b1, local_offsets): the rank's paths and their offsets rebased to
    the start of its increments."""
    b0, b1 = shard_bounds(offsets, world, rank)
    offsets = np.asarray(offsets, dtype=np.int64)
    return b0, b1, offsets[b0:b1 + 1] - offsets[b0]
