"""Assignment of ensemble systems to GPUs (one process per GPU).

Systems are independent, so a multi-GPU ensemble shards by system with no
data exchange: each rank steps its own batch (bh_ensemble_create) and only
the timing and the diagnostics are gathered on the host.  The assignment is
longest-processing-time first on body counts, which keeps the per-rank body
totals within max(size) of each other.
"""
from __future__ import annotations

import heapq


def shard_systems(sizes, world_size: int):
    """Return, for each rank, the sorted indices of the systems it owns."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    heap = [(0, r) for r in range(world_size)]
    heapq.heapify(heap)
    owned = [[] for _ in range(world_size)]
    for i in sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k)):
        load, r = heapq.heappop(heap)
        owned[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(o) for o in owned]


def shard_of(sizes, world_size: int, rank: int):
    return shard_systems(sizes, world_size)[rank]
