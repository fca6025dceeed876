"""Sharding the voxelization across ranks (one process per GPU).

The path has no exchange during compute: occupancy columns, SDF cells and the
meshes of a batch are independent. A forward is split by whole meshes (a batch) or
by z-slabs of one grid, each rank holding the full triangle list; its outputs stay
sharded or are gathered once. The adjoint of a sharded forward needs one reduction
of the per-vertex gradient partials (3 x V values); it is done in a fixed rank
order, so every rank gets the same, bitwise reproducible sum (no collective
reduction whose order the library chooses).

All functions take a ``torch.distributed`` process group (the default group when
None) and work with any backend (NCCL for device tensors, gloo on the host).
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import torch
import torch.distributed as dist


def z_slab(nz: int, world: int, rank: int) -> Tuple[int, int]:
    """Cell layers [z0, z1) of rank `rank` when nz layers are split into `world`
    contiguous slabs whose sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank outside the world")
    base, extra = divmod(int(nz), world)
    z0 = rank * base + min(rank, extra)
    return z0, z0 + base + (1 if rank < extra else 0)


def slab_mask(dims: Sequence[int], world: int, rank: int, device=None) -> torch.Tensor:
    """Boolean mask over the flat cells (idx = (k*ny + j)*nx + i) of rank's slab."""
    nx, ny, nz = (int(d) for d in dims)
    z0, z1 = z_slab(nz, world, rank)
    m = torch.zeros(nz, dtype=torch.bool, device=device)
    m[z0:z1] = True
    return m.repeat_interleave(nx * ny)


def assign_meshes(cells: Sequence[int], world: int) -> List[List[int]]:
    """Whole meshes to ranks, largest first onto the least loaded rank (ties to the
    lower rank): a deterministic longest-processing-time split by cell count.
    Each rank's list is in ascending mesh order."""
    load = [0] * world
    out: List[List[int]] = [[] for _ in range(world)]
    order = sorted(range(len(cells)), key=lambda i: (-int(cells[i]), i))
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += int(cells[i])
    return [sorted(x) for x in out]


def fixed_order_sum(partial: torch.Tensor, group: Optional[dist.ProcessGroup] = None) -> torch.Tensor:
    """Sum of every rank's `partial` (same shape and dtype on all ranks), added in
    rank order 0, 1, ..., world-1 on every rank: identical and reproducible."""
    world = dist.get_world_size(group)
    parts = [torch.empty_like(partial) for _ in range(world)]
    dist.all_gather(parts, partial.contiguous(), group=group)
    total = parts[0].clone()
    for p in parts[1:]:
        total += p
    return total


def gather_to_rank0(obj, group: Optional[dist.ProcessGroup] = None):
    """Rank 0 receives every rank's `obj` (any picklable value) in rank order;
    other ranks receive None."""
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    out = [None] * world if rank == 0 else None
    dist.gather_object(obj, out, dst=0, group=group)
    return out


# ---------------------------------------------------------------- the library, sharded
SLAB_ARRAYS = ("occupancy", "sdf32", "sdf64", "nearest_triangle", "nearest_region")


def voxelize_slab(plc, world: int, rank: int, resolution: int = 64, pad: int = 1, grid=None, **kw):
    """Rank `rank`'s share of ``voxelize_ex(plc, ...)``: the cell layers
    ``z_slab(nz, world, rank)`` of the grid (from resolution/pad, or ``grid`` =
    (corner, spacing, dims)), evaluated by the library on this rank's GPU with the
    whole grid's geometry, so the slab equals those layers of the whole grid bit for
    bit. Returns (VoxelResult or None for an empty share, (z0, z1))."""
    import cybermeshgenerator_gb300 as cm
    dims = grid[2] if grid is not None else cm.plc_grid(plc, resolution, pad)[2]
    z0, z1 = z_slab(int(dims[2]), world, rank)
    if z0 == z1:
        return None, (z0, z1)
    if grid is not None:
        kw["grid"] = grid
    else:
        kw["resolution"], kw["pad"] = resolution, pad
    return cm.voxelize_ex(plc, layers=(z0, z1), **kw), (z0, z1)


def gather_slabs(result, group: Optional[dist.ProcessGroup] = None):
    """Rank 0 receives the whole grid's arrays: every rank's slab arrays (those
    present of SLAB_ARRAYS) concatenated in rank order, which for the z-major cell
    layout is the whole grid. Other ranks receive None."""
    import numpy as np
    mine = {} if result is None else {n: np.asarray(getattr(result, n)) for n in SLAB_ARRAYS
                                       if getattr(result, n) is not None}
    parts = gather_to_rank0(mine, group)
    if parts is None:
        return None
    names = [n for n in SLAB_ARRAYS if any(n in p for p in parts)]
    return {n: np.concatenate([p[n] for p in parts if n in p]) for n in names}


def batch_shard(plcs, resolutions, pads, world: int, rank: int, **kw):
    """Rank `rank`'s whole meshes of a batch (assign_meshes by cell count, from each
    mesh's grid) as one library Batch on this rank's GPU: (Batch or None, the meshes'
    indices in the batch)."""
    import cybermeshgenerator_gb300 as cm
    cells = []
    for p, r, q in zip(plcs, resolutions, pads):
        d = cm.plc_grid(p, int(r), int(q))[2]
        cells.append(d[0] * d[1] * d[2])
    mine = assign_meshes(cells, world)[rank]
    if not mine:
        return None, mine
    b = cm.Batch([plcs[i] for i in mine], [int(resolutions[i]) for i in mine],
                 [int(pads[i]) for i in mine], **kw)
    return b, mine
