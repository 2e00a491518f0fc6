"""Sharding of independent meshes (batched builds) or requests (serving) across ranks.

Meshes are independent units, so there is no data-path collective: each rank builds its own
share and keeps its own trees.  The assignment is greedy longest-processing-time by triangle
count (largest mesh first to the least-loaded rank), deterministic for a given count list so
every rank computes the same partition without communicating.
"""
from __future__ import annotations

import heapq
from typing import List, Sequence

import numpy as np


def assign(counts: Sequence[int], world_size: int) -> List[np.ndarray]:
    """Mesh indices per rank (each sorted ascending)."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    counts = np.asarray(counts, np.int64)
    order = sorted(range(len(counts)), key=lambda i: (-int(counts[i]), i))
    heap = [(0, r) for r in range(world_size)]
    heapq.heapify(heap)
    parts: List[list] = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + int(counts[i]), r))
    return [np.array(sorted(p), np.int64) for p in parts]


def shard_offsets(counts: Sequence[int], meshes: np.ndarray) -> np.ndarray:
    """offsets[count+1] of the concatenation of the selected meshes, in the given order."""
    c = np.asarray(counts, np.int64)[meshes]
    off = np.zeros(len(c) + 1, np.int64)
    np.cumsum(c, out=off[1:])
    return off.astype(np.uint32)


def stream_share(sizes: Sequence[int], world_size: int, rank: int) -> np.ndarray:
    """The requests of one serving stream that `rank` serves (indices in arrival order): the
    same balanced partition by request size as assign(), so every rank derives its share alone."""
    return assign(sizes, world_size)[rank]
