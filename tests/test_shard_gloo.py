"""The multi-rank path on the host: z-slab and whole-mesh partitions, the
fixed-rank-order gradient reduction and the rank-0 gather, run as two gloo ranks
(CPU). The per-rank work is the oracle's (the same sums the GPU adjoint makes),
so no GPU is needed."""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from cybermeshgenerator_gb300 import shard


def test_z_slabs_cover_the_grid():
    for nz in (1, 7, 64, 255):
        for world in (1, 2, 3, 8):
            spans = [shard.z_slab(nz, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == nz
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    m = shard.slab_mask((3, 2, 5), 2, 1)
    assert m.sum().item() == 2 * 6 and not m[:18].any() and m[18:].all()


def test_mesh_assignment_is_balanced_and_deterministic():
    rng = np.random.default_rng(3)
    cells = rng.integers(32 ** 3, 192 ** 3, size=512).tolist()
    a = shard.assign_meshes(cells, 4)
    assert a == shard.assign_meshes(cells, 4)
    assert sorted(i for r in a for i in r) == list(range(512))
    loads = [sum(cells[i] for i in r) for r in a]
    assert max(loads) - min(loads) <= max(cells)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle as O
    from cybermeshgenerator_gb300 import workloads as W
    orc = O.Oracle()
    # adjoint of one mesh, cells split into z-slabs
    pts, tris = W.jittered_icosphere(2, 0.02, seed=7)
    g = orc.make_grid(pts, 20, 1)
    occ, _ = orc.occupancy(pts, tris, g, O.COMPAT, threads=1)
    _, tri, _ = orc.sdf_brute(pts, tris, g, threads=1)
    rng = np.random.default_rng(11)
    w = rng.uniform(0.0, 1.0, g.ncell)
    t = rng.normal(0.0, 0.1, g.ncell)
    mask = shard.slab_mask((g.nx, g.ny, g.nz), world, rank).numpy()
    part = orc.sdf_grad(pts, tris, g, occ, tri, np.where(mask, w, 0.0), t)
    total = shard.fixed_order_sum(torch.from_numpy(part))
    again = shard.fixed_order_sum(torch.from_numpy(part))
    # whole meshes split across ranks, gathered on rank 0 in rank order
    items = W.mesh_batch(6, seed=9, resolutions=(12, 16), max_subdiv=2, max_seg=24)
    grids = [orc.make_grid(b.points, b.resolution, b.pad) for b in items]
    mine = shard.assign_meshes([gr.ncell for gr in grids], world)[rank]
    res = {i: orc.occupancy(items[i].points, items[i].triangles, grids[i], O.COMPAT,
                            threads=1)[0] for i in mine}
    got = shard.gather_to_rank0(res)
    if rank == 0:
        merged = {}
        for d in got:
            merged.update(d)
        np.savez(os.path.join(out_dir, "out.npz"), total=total.numpy(), again=again.numpy(),
                 **{f"occ{i}": merged[i] for i in range(len(items))})
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_gather(orc):
    import oracle as O
    from cybermeshgenerator_gb300 import workloads as W
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(2, _free_port(), d), nprocs=2, join=True,
                           start_method="spawn")
        z = np.load(os.path.join(d, "out.npz"))
        total, again = z["total"], z["again"]
        pts, tris = W.jittered_icosphere(2, 0.02, seed=7)
        g = orc.make_grid(pts, 20, 1)
        occ, _ = orc.occupancy(pts, tris, g, O.COMPAT)
        _, tri, _ = orc.sdf_brute(pts, tris, g)
        rng = np.random.default_rng(11)
        w = rng.uniform(0.0, 1.0, g.ncell)
        t = rng.normal(0.0, 0.1, g.ncell)
        full = orc.sdf_grad(pts, tris, g, occ, tri, w, t)
        assert np.array_equal(total, again)
        assert np.abs(total - full).max() <= 1e-12 * np.abs(full).max()
        items = W.mesh_batch(6, seed=9, resolutions=(12, 16), max_subdiv=2, max_seg=24)
        for i, b in enumerate(items):
            gi = orc.make_grid(b.points, b.resolution, b.pad)
            want, _ = orc.occupancy(b.points, b.triangles, gi, O.COMPAT)
            assert np.array_equal(z[f"occ{i}"], want)
