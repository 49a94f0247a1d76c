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


def gather_by_system(n_systems: int, mine, rows, all_gather_object=None):
    """Per-system diagnostic rows from every rank, in system order.

    mine: the system indices this rank owns; rows: one row per owned system,
    in the order of `mine` (may be empty).  all_gather_object:
    torch.distributed.all_gather_object when several ranks run, None for one
    rank.  Every system must be owned by exactly one rank."""
    import numpy as np

    r = np.asarray(rows, dtype=np.float64)
    part = (list(map(int, mine)), r.reshape(len(mine), -1) if len(mine) else np.zeros((0, 0)))
    parts = [part]
    if all_gather_object is not None:
        import torch.distributed as dist

        parts = [None] * dist.get_world_size()
        all_gather_object(parts, part)
    width = max(r.shape[1] for _, r in parts)
    out = np.full((n_systems, width), np.nan)
    seen = np.zeros(n_systems, np.int64)
    for idx, r in parts:
        for k, i in enumerate(idx):
            out[i] = r[k]
            seen[i] += 1
    if not np.all(seen == 1):
        raise RuntimeError("systems not owned by exactly one rank")
    return out


def run_sharded(sizes, world_size: int, rank: int, load, step, diagnostics, steps: int,
                all_gather_object=None):
    """Step this rank's shard of an ensemble and gather per-system diagnostics.

    The per-rank step of a sharded ensemble: the systems shard_of() gives this
    rank are loaded (load(indices) -> handle), advanced `steps` steps
    (step(handle, steps)), and their diagnostics taken once at the end
    (diagnostics(handle) -> one row per owned system); the rows of all ranks
    are gathered on every rank in system order.  No data moves between ranks
    while stepping: systems are independent (the reference's step,
    BarnesHutParticleSystem.cpp:301-347, on each of them)."""
    mine = shard_of(sizes, world_size, rank)
    rows = []
    if mine:
        h = load(mine)
        step(h, steps)
        rows = diagnostics(h)
    return gather_by_system(len(sizes), mine, rows, all_gather_object)
