"""Multi-GPU placement.

* A batch of independent bunches is sharded by bunch, one shard per rank,
  with no collective on the data path (shard_bunches).
* One bunch whose particles are spread over ranks (each rank holds its own
  particles) has one real exchange: the charge.  kick_sharded deposits the
  local particles, sums rho over the ranks (one all-reduce of N mesh
  elements), solves on every rank and gathers the local particles' field;
  global_bounds gives every rank the particle constructor's bounds of the
  whole bunch (MIN/MAX all-reduce of the local extrema).
"""
from __future__ import annotations

import ctypes as C
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


def global_bounds(grid_size, x, y, z, group=None):
    """Bounds of the particle constructor (mesh.jl:125-150) for a bunch whose
    particles are split over the ranks of `group`: this rank's extrema (its
    share may be empty), MIN/MAX all-reduced, then sc_bounds_from_extrema.
    Returns (min_bounds, max_bounds) as tuples."""
    import torch
    import torch.distributed as dist

    from . import _lib as L

    ext = []
    for a in (x, y, z):
        t = torch.as_tensor(a).reshape(-1)
        if t.numel() == 0:
            ext.append((float("inf"), float("-inf")))
        else:
            ext.append((float(t.min()), float(t.max())))
    # NCCL reduces device tensors only, whatever container the particles came in
    dev = "cpu"
    if dist.is_initialized() and dist.get_backend(group) == "nccl":
        dev = torch.device("cuda", torch.cuda.current_device())
    red = torch.tensor([e[0] for e in ext] + [-e[1] for e in ext], dtype=torch.float64, device=dev)
    if dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(red, op=dist.ReduceOp.MIN, group=group)
    red = red.cpu().tolist()
    mins = (C.c_double * 3)(*red[:3])
    maxs = (C.c_double * 3)(*[-v for v in red[3:]])
    lo, hi, dl = (C.c_double * 3)(), (C.c_double * 3)(), (C.c_double * 3)()
    L.call("sc_bounds_from_extrema", (C.c_int32 * 3)(*grid_size), mins, maxs, lo, hi, dl)
    return tuple(lo), tuple(hi)


def kick_sharded(mesh, x, y, z, q, at_cathode: bool = False, group=None):
    """Kick of one bunch whose particles are split over the ranks of `group`
    (this rank passes its own particles, device arrays): local deposit, SUM
    all-reduce of rho, the solve on every rank, the local particles' field.
    Every rank must hold a mesh with the same geometry (global_bounds)."""
    import torch.distributed as dist

    from .mesh import deposit, interpolate_field, solve

    deposit(mesh, x, y, z, q)
    if dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(mesh.rho.permute(2, 1, 0), op=dist.ReduceOp.SUM, group=group)
    solve(mesh, at_cathode=at_cathode)
    return interpolate_field(mesh, x, y, z)
