"""Splitting a filtered base stream over GPUs (one process per GPU).

A window is scored only if it lies inside one run (the reference's
run-length check, pwmscan.cpp:122-126), so cutting the stream at run starts
gives shards that need no halo and no exchange: each rank scans its own
shard, hit positions are shifted by the shard offset, and the union of the
ranks' hits is the hit set of the whole stream.  The reference does the
same with one host thread per device pulling blocks from a shared queue
(pwmscan.cpp:439-453); with one process per GPU the split is static.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, run_start: np.ndarray, world: int) -> list[tuple[int, int]]:
    """world contiguous [lo, hi) ranges cut at run starts, balanced by bases."""
    runs = np.asarray(run_start, dtype=np.int64)
    cuts = [0]
    for r in range(1, world):
        target = n * r / world
        i = int(np.argmin(np.abs(runs - target))) if len(runs) else 0
        c = int(runs[i]) if len(runs) else 0
        cuts.append(max(c, cuts[-1]))
    cuts.append(n)
    return [(cuts[i], cuts[i + 1]) for i in range(world)]


def shard(bases: np.ndarray, run_start: np.ndarray, rank: int, world: int):
    """(bases, run_start, offset) of one rank's shard (run starts rebased)."""
    lo, hi = shard_bounds(len(bases), run_start, world)[rank]
    runs = np.asarray(run_start, dtype=np.int64)
    sel = runs[(runs >= lo) & (runs < hi)] - lo
    if hi > lo and (len(sel) == 0 or sel[0] != 0):
        sel = np.concatenate([[0], sel])
    return bases[lo:hi], sel.astype(np.int64), lo
