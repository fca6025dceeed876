"""Many meshes in one pipeline (the batch workload): 512 closed meshes (icospheres of
subdivision 1-5 and tori of 16-256 segments per ring, random scale 0.5-2 and
rotation, per-mesh resolution in {32, 48, 64, 96, 128, 192}, pad 1), one persistent
evaluation launch, replayed as a CUDA graph, brick edge and queue grab chosen by
the autotuner. Checks per mesh against the oracle: occupancy bit for bit, the
mixed-precision distance within 1e-6 of the mesh's bounding-box diagonal, and the
plain FP64 distance bit for bit."""
import numpy as np
import pytest

from conftest import ROOT  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c4(cm):
    from cybermeshgenerator_gb300 import workloads as W
    items = W.mesh_batch(512)
    plcs = [cm.PLC.from_arrays(b.points, b.triangles) for b in items]
    return dict(items=items, plcs=plcs, res=[b.resolution for b in items],
                pads=[b.pad for b in items])


def _centres(g, vox):
    k, rem = np.divmod(vox, g.nx * g.ny)
    j, i = np.divmod(rem, g.nx)
    h = g.spacing
    return np.stack([g.corner[0] + (i + 0.5) * h, g.corner[1] + (j + 0.5) * h,
                     g.corner[2] + (k + 0.5) * h], 1)


@pytest.fixture(scope="module")
def mixed_batch(cm, c4):
    b = cm.Batch(c4["plcs"], c4["res"], c4["pads"], outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F32,
                 precision=cm.PREC_MIXED, autotune=True)
    b.run().sync()
    return b


def test_batch_occupancy_and_mixed_sdf_per_mesh(cm, orc, c4, mixed_batch):
    import oracle as O
    items = c4["items"]
    st = mixed_batch.stats()
    assert (st["brick"], st["grab"]) in {(16, 1), (16, 2), (8, 0)}
    rng = np.random.default_rng(41)
    for i in range(0, len(items), 8):
        it = items[i]
        r = mixed_batch.result(i)
        g = orc.make_grid(it.points, it.resolution, it.pad)
        assert r.dims == (g.nx, g.ny, g.nz)
        assert np.array_equal(r.corner, np.array(list(g.corner)))
        occ, _ = orc.occupancy(it.points, it.triangles, g, O.COMPAT)
        assert np.array_equal(r.occupancy, occ), f"mesh {i} ({it.kind})"
        vox = rng.choice(g.ncell, size=min(256, g.ncell), replace=False)
        d2, _ = orc.dist2_points(it.points, it.triangles, _centres(g, vox))
        want = np.where(occ[vox] != 0, -1.0, 1.0) * np.sqrt(d2)
        diag = float(np.linalg.norm(it.points.max(0) - it.points.min(0)))
        err = np.abs(r.sdf32[vox].astype(np.float64) - want).max()
        assert err <= 1e-6 * diag, f"mesh {i} ({it.kind}): {err}"


def test_batch_graph_replay_equals_eager(cm, c4, mixed_batch):
    eager = [mixed_batch.result(i) for i in (0, 101, 257, 511)]
    mixed_batch.run(graph=True).sync()  # capture + replay
    mixed_batch.run(graph=True).sync()  # replay
    for r0, i in zip(eager, (0, 101, 257, 511)):
        r1 = mixed_batch.result(i)
        assert np.array_equal(r0.occupancy, r1.occupancy)
        assert np.array_equal(r0.sdf32, r1.sdf32)


def test_fp64_batch_bit_exact_and_equals_single_calls(cm, orc, c4):
    """A plain FP64 batch of every 16th mesh: FP64 distances equal the oracle's
    brute-force minimum bit for bit on sampled cells, and each mesh's outputs equal
    a single-mesh call."""
    idx = list(range(3, 512, 16))
    items = [c4["items"][i] for i in idx]
    outs = cm.OUT_OCCUPANCY | cm.OUT_SDF_F32 | cm.OUT_SDF_F64
    b = cm.Batch([c4["plcs"][i] for i in idx], [c4["res"][i] for i in idx],
                 [c4["pads"][i] for i in idx], outputs=outs, precision=cm.PREC_FP64)
    b.run(graph=True).sync()
    b.run(graph=True).sync()
    rng = np.random.default_rng(42)
    for k, it in enumerate(items):
        r = b.result(k)
        g = orc.make_grid(it.points, it.resolution, it.pad)
        vox = rng.choice(g.ncell, size=min(256, g.ncell), replace=False)
        d2, _ = orc.dist2_points(it.points, it.triangles, _centres(g, vox))
        assert np.array_equal(np.abs(r.sdf64[vox]), np.sqrt(d2)), f"mesh {idx[k]} ({it.kind})"
        if k % 8 == 0:
            one = cm.voxelize_ex(c4["plcs"][idx[k]], resolution=it.resolution, pad=it.pad,
                                 outputs=outs, precision=cm.PREC_FP64)
            assert np.array_equal(one.occupancy, r.occupancy)
            assert np.array_equal(one.sdf64, r.sdf64)
            assert np.array_equal(one.sdf32, r.sdf32)
