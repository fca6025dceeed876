"""Sharding through the library on the GPU.

* z-slabs: voxelize_ex with cell layers [z0, z1) evaluates those layers with the whole
  grid's geometry; the slabs of a split, concatenated in order, equal the whole grid
  bit for bit (occupancy, float and FP64 distance, nearest triangle and region), in
  FP64 and in mixed precision, for slab edges inside 16^3 bricks and sub-bricks, on
  the fixtures and on the full-size headline grid;
* two gloo ranks (processes) on this GPU, each calling the library for its own share
  (shard.voxelize_slab, shard.batch_shard), gathered on rank 0: equal to the whole
  grid and to the whole batch. The ranks' kernels never wait on one another; only
  the host collectives join them.
"""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

ARRAYS = ("occupancy", "sdf32", "sdf64", "nearest_triangle", "nearest_region")
OUTS = 1 | 2 | 4 | 8  # occupancy, float and FP64 distance, nearest triangle + region


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint8) if a.dtype.itemsize == 1 else a.view(f"u{a.dtype.itemsize}")


def _whole_and_slabs(cm, plc, world, **kw):
    from cybermeshgenerator_gb300 import shard
    whole = cm.voxelize_ex(plc, outputs=OUTS, **kw)
    nz = whole.dims[2]
    parts = []
    for r in range(world):
        res, (z0, z1) = shard.voxelize_slab(plc, world, r, outputs=OUTS, **kw)
        assert res.layers == (z0, z1, nz) and res.dims == (whole.dims[0], whole.dims[1], z1 - z0)
        assert np.array_equal(res.corner, whole.corner) and res.spacing == whole.spacing
        parts.append(res)
    return whole, parts


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name,world", [("shsphere64_r30p1", 3), ("icosphere_s3_r58p3", 5),
                                        ("boxtorus64_facegrid", 2)])
def test_slabs_equal_whole_grid(cm, golden, name, world, precision):
    g = golden(name)
    plc = cm.PLC.from_arrays(g["points"], g["triangles"])
    kw = dict(precision=precision)
    if "resolution" in g:
        kw.update(resolution=int(g["resolution"]), pad=int(g["pad"]))
    else:
        kw.update(grid=(g["corner"], g["spacing"], g["dims"]))
    whole, parts = _whole_and_slabs(cm, plc, world, **kw)
    for n in ARRAYS:
        cat = np.concatenate([getattr(p, n) for p in parts])
        assert np.array_equal(_bits(cat), _bits(getattr(whole, n))), n


def test_slabs_equal_whole_headline_grid(cm, golden):
    """The full-size headline grid (231 x 247 x 256) in mixed precision, three slabs."""
    z = golden("shsphere256")
    plc = cm.PLC.from_arrays(z["points"], z["triangles"])
    whole, parts = _whole_and_slabs(cm, plc, 3, resolution=254, pad=1, precision=1)
    for n in ARRAYS:
        cat = np.concatenate([getattr(p, n) for p in parts])
        assert np.array_equal(_bits(cat), _bits(getattr(whole, n))), n


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    torch.cuda.set_device(0)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import shard
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.sh_sphere(nlon=64, nlat=32, seed=3)
    plc = cm.PLC.from_arrays(pts, tris)
    res, _ = shard.voxelize_slab(plc, world, rank, resolution=40, pad=1, outputs=OUTS,
                                 precision=cm.PREC_MIXED)
    whole = shard.gather_slabs(res)
    items = W.mesh_batch(6, seed=9, resolutions=(12, 16), max_subdiv=2, max_seg=24)
    plcs = [cm.PLC.from_arrays(b.points, b.triangles) for b in items]
    resl, pads = [b.resolution for b in items], [b.pad for b in items]
    bt, mine = shard.batch_shard(plcs, resl, pads, world, rank, outputs=1 | 2,
                                 precision=cm.PREC_MIXED)
    got = {}
    if bt is not None:
        bt.run().sync()
        for k, i in enumerate(mine):
            r = bt.result(k)
            got[i] = (np.array(r.occupancy), np.array(r.sdf32))
    allgot = shard.gather_to_rank0(got)
    if rank == 0:
        ref = cm.voxelize_ex(plc, resolution=40, pad=1, outputs=OUTS, precision=cm.PREC_MIXED)
        ok = all(np.array_equal(_bits(whole[n]), _bits(getattr(ref, n))) for n in ARRAYS)
        merged = {}
        for d in allgot:
            merged.update(d)
        full = cm.Batch(plcs, resl, pads, outputs=1 | 2, precision=cm.PREC_MIXED).run().sync()
        okb = sorted(merged) == list(range(len(items)))
        for i in range(len(items)):
            r = full.result(i)
            okb = okb and np.array_equal(merged[i][0], r.occupancy) and \
                np.array_equal(_bits(merged[i][1]), _bits(r.sdf32))
        with open(os.path.join(out_dir, "result.txt"), "w") as f:
            f.write(f"{int(ok)} {int(okb)}")
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_share_the_work(cm):
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(2, _free_port(), d), nprocs=2, join=True,
                           start_method="spawn")
        ok, okb = open(os.path.join(d, "result.txt")).read().split()
        assert ok == "1", "gathered slabs differ from the whole grid"
        assert okb == "1", "gathered meshes differ from the whole batch"
