"""Multi-GPU placement of independent bunches.

A single bunch's kick has no data-parallel exchange worth a collective at
the mesh sizes of this library (a rho all-reduce plus a replicated solve is
the only split), so multiple GPUs run independent work: a batch of bunches
is sharded by bunch, one shard per rank, with no collective on the data path.
"""
from __future__ import annotations

import heapq
from typing import Sequence


def shard_bunches(counts: Sequence[int], world_size: int, rank: int) -> list[int]:
    """Bunch indices for `rank`: longest-processing-time-first assignment
    by particle count (deterministic; every rank computes the same
    partition without communicating)."""
    if world_size < 1 or not (0 <= rank < world_size):
        raise ValueError("need 0 <= rank < world_size")
    order = sorted(range(len(counts)), key=lambda i: (-int(counts[i]), i))
    heap = [(0, r) for r in range(world_size)]
    owner = [0] * len(counts)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + int(counts[i]), r))
    return [i for i in range(len(counts)) if owner[i] == rank]
