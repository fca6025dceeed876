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


def test_batch_overlapped_phases_equal_the_sizing_pass(cm, c4, mixed_batch):
    """The SDF preparation runs on a second stream beside the occupancy passes, in the
    sizing pass (arenas re-planned between the two streams' halves) and in later runs:
    eager runs after the sizing pass give the same outputs, the timed phases are all
    recorded and the evaluation starts after both phases end."""
    ref = cm.Batch(c4["plcs"][:64], c4["res"][:64], c4["pads"][:64],
                   outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F32, precision=cm.PREC_MIXED)
    ref.run().sync()
    sized = [ref.result(i) for i in range(0, 64, 9)]
    ref.set_timing(True)
    for _ in range(3):
        ref.run()
    ref.sync()
    t = ref.timing()
    for i, r0 in zip(range(0, 64, 9), sized):
        r1 = ref.result(i)
        assert np.array_equal(r0.occupancy, r1.occupancy)
        assert np.array_equal(r0.sdf32, r1.sdf32)
    assert all(t[k] > 0 for k in ("occupancy_ms", "sdf_prep_ms", "eval_ms", "total_ms")), t
    assert t["eval_ms"] < t["total_ms"]
    assert max(t["occupancy_ms"], t["sdf_prep_ms"]) + t["eval_ms"] <= t["total_ms"] * 1.01, t


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
