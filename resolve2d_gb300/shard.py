"""Independent worlds dealt out to GPUs: one process per GPU, nothing exchanged.

A world never touches another, so a batch splits into per-rank batches that
step with no data-path communication.  A frame ends when the slowest rank
ends, and a rank's step time grows with its body count.  The ranks therefore
get equal body totals by Graham's longest-processing-time rule: worlds, largest
first, each go to the rank with the fewest bodies so far.  A rank then ends at
most one world's bodies above the mean.
"""

from __future__ import annotations

import heapq

import numpy as np


def balanced_shards(counts, nshards: int) -> list[np.ndarray]:
    """World indices of each of `nshards` ranks, ascending within a rank.

    `counts` are the worlds' body counts.  Ties go to the lower world index and
    the lower rank, so every rank computes the same deal.
    """
    counts = np.asarray(counts, np.int64)
    if nshards < 1:
        raise ValueError("nshards must be >= 1")
    heap = [(0, r) for r in range(nshards)]  # (bodies so far, rank)
    members: list[list[int]] = [[] for _ in range(nshards)]
    for w in np.argsort(-counts, kind="stable"):
        total, r = heapq.heappop(heap)
        members[r].append(int(w))
        heapq.heappush(heap, (total + int(counts[w]), r))
    return [np.array(sorted(m), np.int64) for m in members]
