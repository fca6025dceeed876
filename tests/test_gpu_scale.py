"""The scale workload: 2000 non-overlapping ellipsoids (semi-axes U(0.01, 0.04),
subdivision-3 icospheres, 2.56M triangles) in the unit cube at 512^3 (resolution
510, pad 1): occupancy bit for bit against the oracle, the mixed-precision
distance within 1e-6 of the bounding-box diagonal and the plain FP64 distance
bit for bit on sampled cells (uniform and near the surfaces), and the adjoint
against the oracle's FP64 analytic gradient over the whole grid. Predicate
streams: 1e7 orient3d and insphere queries (10 % exactly degenerate, 10 % within a
few ulps) against the oracle's signs in both modes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c5(cm, orc):
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.ellipsoid_field()
    g = orc.make_grid(pts, 510, 1)
    return dict(pts=pts, tris=tris, g=g, plc=cm.PLC.from_arrays(pts, tris),
                diag=float(np.linalg.norm(pts.max(0) - pts.min(0))))


def _centres(g, vox):
    k, rem = np.divmod(vox, g.nx * g.ny)
    j, i = np.divmod(rem, g.nx)
    h = g.spacing
    return np.stack([g.corner[0] + (i + 0.5) * h, g.corner[1] + (j + 0.5) * h,
                     g.corner[2] + (k + 0.5) * h], 1)


def _samples(g, sdf, rng, n=200):
    uni = rng.choice(g.ncell, size=n, replace=False)
    near = np.nonzero(np.abs(sdf) < 1.5 * g.spacing)[0]
    return np.concatenate([uni, rng.choice(near, size=n, replace=False)])


def test_scale_occupancy_and_mixed_sdf(cm, orc, c5):
    import oracle as O
    g = c5["g"]
    r = cm.voxelize_ex(c5["plc"], resolution=510, pad=1,
                       outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F32, precision=cm.PREC_MIXED)
    assert r.dims == (g.nx, g.ny, g.nz) == (512, 511, 512)
    occ, _ = orc.occupancy(c5["pts"], c5["tris"], g, O.COMPAT)
    assert np.array_equal(r.occupancy, occ)
    rng = np.random.default_rng(51)
    vox = _samples(g, r.sdf32, rng)
    d2, _ = orc.dist2_points(c5["pts"], c5["tris"], _centres(g, vox))
    want = np.where(occ[vox] != 0, -1.0, 1.0) * np.sqrt(d2)
    err = np.abs(r.sdf32[vox].astype(np.float64) - want)
    assert err.max() <= 1e-6 * c5["diag"], err.max()


def test_scale_fp64_sampled_bit_exact(cm, orc, c5):
    g = c5["g"]
    r = cm.voxelize_ex(c5["plc"], resolution=510, pad=1, outputs=cm.OUT_SDF_F64,
                       precision=cm.PREC_FP64)
    rng = np.random.default_rng(52)
    vox = _samples(g, r.sdf64, rng)
    d2, _ = orc.dist2_points(c5["pts"], c5["tris"], _centres(g, vox))
    assert np.array_equal(np.abs(r.sdf64[vox]), np.sqrt(d2))


def test_two_warps_per_brick_walk(cm, orc, c5):
    """The same surface at 320^3: 8000 candidate bricks, between 32 and 64 per SM, so the
    brick walk runs with two warps per brick (the headline grid takes four, the 512^3
    grid one). Plain FP64 distances bit for bit and mixed ones within 1e-6 of the
    diagonal on sampled cells, occupancy bit for bit."""
    torch = pytest.importorskip("torch")
    import oracle as O
    g = orc.make_grid(c5["pts"], 318, 1)
    nb = -(-g.nx // 16) * -(-g.ny // 16) * -(-g.nz // 16)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert 32 * sms < nb <= 64 * sms, (nb, sms)
    occ, _ = orc.occupancy(c5["pts"], c5["tris"], g, O.COMPAT)
    rng = np.random.default_rng(53)
    plain = cm.voxelize_ex(c5["plc"], resolution=318, pad=1,
                           outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F64, precision=cm.PREC_FP64)
    mixed = cm.voxelize_ex(c5["plc"], resolution=318, pad=1,
                           outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F32, precision=cm.PREC_MIXED)
    assert np.array_equal(plain.occupancy, occ) and np.array_equal(mixed.occupancy, occ)
    vox = _samples(g, plain.sdf64, rng)
    d2, _ = orc.dist2_points(c5["pts"], c5["tris"], _centres(g, vox))
    assert np.array_equal(np.abs(plain.sdf64[vox]), np.sqrt(d2))
    want = np.where(occ[vox] != 0, -1.0, 1.0) * np.sqrt(d2)
    assert np.abs(mixed.sdf32[vox].astype(np.float64) - want).max() <= 1e-6 * c5["diag"]


def test_scale_adjoint_matches_host_gradient(cm, orc, c5):
    torch = pytest.importorskip("torch")
    from cybermeshgenerator_gb300 import torch_sdf as TS
    g = c5["g"]
    grid = TS.grid_of(list(g.corner), g.spacing, (g.nx, g.ny, g.nz))
    plan = TS.SDFPlan(c5["pts"], c5["tris"], grid)
    rng = np.random.default_rng(53)
    w = rng.uniform(0.0, 1.0, g.ncell)
    t = rng.normal(0.0, 0.01, g.ncell)
    v = torch.tensor(c5["pts"], device="cuda")
    sdf, occ, tri, reg = plan.forward(v)
    gs = 2.0 * torch.tensor(w, device="cuda") * (sdf - torch.tensor(t, device="cuda"))
    grad = plan.backward(v, occ, tri, reg, gs)
    again = plan.backward(v, occ, tri, reg, gs)
    assert torch.equal(grad, again)
    want = orc.sdf_grad(c5["pts"], c5["tris"], g, occ.cpu().numpy(), tri.cpu().numpy(), w, t)
    got = grad.cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-11 * np.linalg.norm(want)
    plan.close()


@pytest.mark.parametrize("kind", ["orient3d", "insphere"])
def test_predicate_stream_1e7(cm, orc, kind):
    import oracle as O
    from cybermeshgenerator_gb300 import workloads as W
    S = W.predicate_stream(10_000_000, kind, degenerate=0.1, near=0.1, seed=61)
    fn = cm.orient3d_stream if kind == "orient3d" else cm.insphere_stream
    for mode, om in ((cm.PRED_COMPAT, O.COMPAT), (cm.PRED_EXACT, O.EXACT)):
        got, st = fn(S, mode)
        assert np.array_equal(got, orc.stream(kind, S, om))
        assert st["queries"] == S.shape[1]
        assert st["exact_queries"] >= int(0.1 * S.shape[1])
