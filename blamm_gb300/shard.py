"""Splitting one filtered base stream over GPUs (one process per GPU).

Each rank takes a contiguous, equally long range [lo, hi) of window starts and scans
bases[lo : hi + halo] with halo = longest motif - 1, so every window that starts in its
range lies inside what it scans; hits starting at or after hi belong to the next rank and
are dropped.  A window is scored only inside one run (the reference's run-length check,
src/pwmscan.cpp:122-126), so the shard's run table is the run that holds lo, rebased to 0,
and the runs that start after it.  No exchange is needed: the union of the ranks' hits,
shifted by their offsets, is the hit set of the whole stream.  The reference does the same
with overlapping blocks pulled from a shared queue by one host thread per device
(src/sequence.cpp:274-293, src/pwmscan.cpp:439-453); with one process per GPU the split is
static, and a stream that is one long run splits as evenly as any other.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, world: int) -> list[tuple[int, int]]:
    """world contiguous [lo, hi) ranges of window starts covering [0, n), lengths within 1."""
    cuts = [n * r // world for r in range(world + 1)]
    return [(cuts[i], cuts[i + 1]) for i in range(world)]


def shard(bases: np.ndarray, run_start: np.ndarray, rank: int, world: int, halo: int):
    """(bases, run_start, offset, keep) of one rank's shard.

    The rank scans the returned bases with the returned run table, keeps the hits at
    positions < keep and adds offset to their positions."""
    if halo < 0:
        raise ValueError("halo must be >= 0 (the longest motif - 1)")
    n = len(bases)
    lo, hi = shard_bounds(n, world)[rank]
    end = min(n, hi + halo) if hi > lo else lo
    runs = np.asarray(run_start, dtype=np.int64)
    inner = runs[(runs > lo) & (runs < end)] - lo
    sel = np.concatenate([[0], inner]) if end > lo else inner
    return bases[lo:end], sel.astype(np.int64), lo, hi - lo
