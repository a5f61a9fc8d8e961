"""Multi-GPU partitioning of digest work.

Digests of different inputs are independent (sdhash hashes files on separate
threads, sdhash-src/sdhash_threads.cc:152-186), so N GPUs split the inputs
with no data-path exchange: each rank digests its own files and the host
concatenates results in input order.  Comparison shards the same way by whole
digests.
"""
from __future__ import annotations

import heapq


def shard_sizes(sizes, world: int) -> list[list[int]]:
    """Size-balanced assignment of input indices to `world` ranks (largest
    first onto the least-loaded rank).  Each rank's list is in input order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    heap = [(0, r) for r in range(world)]
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(x) for x in out]


def merge_in_order(parts: list[list[tuple[int, object]]], n: int) -> list[object]:
    """Reassemble per-rank (index, result) lists into input order."""
    res: list[object] = [None] * n
    seen = [False] * n
    for part in parts:
        for i, v in part:
            if seen[i]:
                raise ValueError(f"input {i} produced by two ranks")
            seen[i] = True
            res[i] = v
    if not all(seen):
        raise ValueError("some inputs were not produced")
    return res
