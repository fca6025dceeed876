"""The SDF adjoint (dL/d vertex positions) on the GPU.

The workload is the differentiable-SDF configuration: the spherical-harmonics
sphere (256 x 128 bands, 65,024 triangles) on a 128^3 grid (resolution 126,
pad 1), loss L = sum w (sdf - t)^2 with w ~ U(0, 1) and t ~ N(0, 0.1^2) per cell.
Checks: the FP64 host analytic gradient of the oracle (same checkpoint), FP64
central differences (h = 1e-6) of the plain FP64 distance on 64 random
vertices x 3 coordinates at 1e-5 relative, bitwise reproducibility, and the
torch.autograd path in float32 and float64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def c3(cm, orc):
    from cybermeshgenerator_gb300 import workloads as W
    from cybermeshgenerator_gb300 import torch_sdf as TS
    pts, tris = W.sh_sphere()
    g = orc.make_grid(pts, 126, 1)
    grid = TS.grid_of(list(g.corner), g.spacing, (g.nx, g.ny, g.nz))
    plan = TS.SDFPlan(pts, tris, grid)
    rng = np.random.default_rng(21)
    w = rng.uniform(0.0, 1.0, g.ncell)
    t = rng.normal(0.0, 0.1, g.ncell)
    return dict(pts=pts, tris=tris, g=g, grid=grid, plan=plan, w=w, t=t)


def _forward(plan, pts):
    v = torch.tensor(pts, dtype=torch.float64, device="cuda")
    return [x for x in plan.forward(v)]


def _grad(plan, pts, w, t):
    v = torch.tensor(pts, dtype=torch.float64, device="cuda")
    sdf, occ, tri, reg = plan.forward(v)
    W_ = torch.tensor(w, device="cuda")
    T_ = torch.tensor(t, device="cuda")
    gs = 2.0 * W_ * (sdf - T_)
    return plan.backward(v, occ, tri, reg, gs), (sdf, occ, tri, reg)


def test_adjoint_matches_host_analytic_gradient(c3, orc):
    grad, (sdf, occ, tri, reg) = _grad(c3["plan"], c3["pts"], c3["w"], c3["t"])
    grad = grad.cpu().numpy()
    occ_h, tri_h = occ.cpu().numpy(), tri.cpu().numpy()
    assert tri_h.min() >= 0
    want = orc.sdf_grad(c3["pts"], c3["tris"], c3["g"], occ_h, tri_h, c3["w"], c3["t"])
    # same checkpoint, different summation order: agreement to rounding
    assert np.linalg.norm(grad - want) <= 1e-11 * np.linalg.norm(want)
    assert np.abs(grad - want).max() <= 1e-10 * np.abs(want).max()


def _central_differences(plan, pts, verts, w, t, h):
    """FP64 central differences of L = sum w (sdf - t)^2 in difference form (only
    the cells that change carry rounding), per (vertex, axis): the full sum, the
    sum over the cells whose nearest triangle is the same at +h and -h, and the
    mask of the others."""
    full, kept, masks = np.zeros((len(verts), 3)), np.zeros((len(verts), 3)), []
    for i, v in enumerate(verts):
        row = []
        for a in range(3):
            s, tri = [], []
            for step in (h, -h):
                p = pts.copy()
                p[v, a] += step
                sd, _, tr, _ = _forward(plan, p)
                s.append(sd.cpu().numpy())
                tri.append(tr.cpu().numpy())
            c = w * (s[0] - s[1]) * (s[0] + s[1] - 2 * t) / (2 * h)
            switched = tri[0] != tri[1]
            full[i, a] = c.sum()
            kept[i, a] = c[~switched].sum()
            row.append(switched)
        masks.append(row)
    return full, kept, masks


def test_adjoint_vs_central_differences(c3, c3_mixed):
    """FP64 central differences (h = 1e-6) of the plain FP64 distance (bit-identical
    to the reference's) on 64 random vertices x 3 coordinates, relative 1e-5.

    The distance is the minimum over triangles, so it has kinks where the nearest
    triangle changes between non-adjacent features. Near this mesh's poles the
    bands are 6e-4 wide; tilting one by 1e-6 moves such switches across cells, and
    the difference quotient there is not the derivative (the oracle's own central
    differences on the CPU show the same discrepancy). At h = 1e-6 the comparison
    is therefore made over the cells whose nearest triangle is the same at +h and
    -h, on both sides (the adjoint with dL/dsdf zeroed on the others); at h = 1e-8,
    where no switch is left in range, over every cell."""
    plan, pts, w, t = c3["plan"], c3["pts"], c3["w"], c3["t"]
    v = torch.tensor(pts, dtype=torch.float64, device="cuda")
    sdf, occ, tri, reg = plan.forward(v)
    gs = 2.0 * torch.tensor(w, device="cuda") * (sdf - torch.tensor(t, device="cuda"))
    grad = plan.backward(v, occ, tri, reg, gs).cpu().numpy()
    rng = np.random.default_rng(22)
    verts = rng.choice(len(pts), size=64, replace=False)

    full, kept, masks = _central_differences(plan, pts, verts, w, t, 1e-6)
    an_kept = np.zeros_like(kept)
    an_kept32 = np.zeros_like(kept)  # the FP32 adjoint, same checkpoint
    for i, vv in enumerate(verts):
        for a in range(3):
            g = gs.clone()
            g[torch.from_numpy(masks[i][a]).to("cuda")] = 0.0
            an_kept[i, a] = plan.backward(v, occ, tri, reg, g)[vv, a].item()
            an_kept32[i, a] = c3_mixed.backward(v, occ, tri, reg, g)[vv, a].item()
    rel_kept = np.linalg.norm(kept - an_kept) / np.linalg.norm(an_kept)
    rel_kept32 = np.linalg.norm(kept - an_kept32) / np.linalg.norm(an_kept32)
    print(f"h=1e-6, FP32 adjoint: relative error {rel_kept32:.2e}")
    assert rel_kept32 <= 1e-5, rel_kept32
    rel_full = np.linalg.norm(full - grad[verts]) / np.linalg.norm(grad[verts])
    print(f"h=1e-6: relative error {rel_kept:.2e} without the "
          f"{sum(int(m.sum()) for r in masks for m in r)} switching cells, "
          f"{rel_full:.2e} with them")
    assert rel_kept <= 1e-5, rel_kept

    full8, _, _ = _central_differences(plan, pts, verts, w, t, 1e-8)
    rel8 = np.linalg.norm(full8 - grad[verts]) / np.linalg.norm(grad[verts])
    print(f"h=1e-8: relative error {rel8:.2e}")
    assert rel8 <= 1e-5, rel8
    _forward(plan, pts)


def test_adjoint_is_bitwise_reproducible(c3):
    g1, _ = _grad(c3["plan"], c3["pts"], c3["w"], c3["t"])
    g2, _ = _grad(c3["plan"], c3["pts"], c3["w"], c3["t"])
    assert torch.equal(g1, g2)


def test_autograd_function(c3):
    from cybermeshgenerator_gb300 import torch_sdf as TS
    plan, pts, w, t = c3["plan"], c3["pts"], c3["w"], c3["t"]
    nx, ny, nz = plan.dims
    W_ = torch.tensor(w, device="cuda").view(nz, ny, nx).permute(2, 1, 0)
    T_ = torch.tensor(t, device="cuda").view(nz, ny, nx).permute(2, 1, 0)
    want, _ = _grad(plan, pts, w, t)
    v64 = torch.tensor(pts, dtype=torch.float64, device="cuda", requires_grad=True)
    s = TS.sdf(v64, plan)
    assert s.shape == (nx, ny, nz)
    (W_ * (s - T_) ** 2).sum().backward()
    assert torch.equal(v64.grad, want)
    # float32 vertices: float32 distances and gradient (computed in FP64). Rounding
    # the vertices to float32 moves them by ~6e-8, itself a perturbation that crosses
    # nearest-triangle switches, so the reference is the FP64 adjoint at the rounded
    # positions; what is left is the float32 arithmetic of the loss.
    p32 = pts.astype(np.float32)
    want32, _ = _grad(plan, p32.astype(np.float64), w, t)
    v32 = torch.tensor(p32, device="cuda", requires_grad=True)
    s32 = TS.sdf(v32, plan)
    assert s32.dtype == torch.float32
    (W_.float() * (s32 - T_.float()) ** 2).sum().backward()
    assert v32.grad.dtype == torch.float32
    ref = want32.cpu().numpy()
    assert np.linalg.norm(v32.grad.cpu().numpy() - ref) <= 1e-4 * np.linalg.norm(ref)
    _forward(plan, pts)


@pytest.fixture(scope="module")
def c3_mixed(c3, cm):
    from cybermeshgenerator_gb300 import torch_sdf as TS
    pm = TS.SDFPlan(c3["pts"], c3["tris"], c3["grid"], precision=cm.PREC_MIXED)
    yield pm
    pm.close()


def test_mixed_precision_forward_gradient(c3, c3_mixed):
    """A mixed-precision plan: its forward within 1e-6 of the bbox diagonal, its
    FP32 adjoint within 1e-5 of the FP64 adjoint on the same checkpoint, and its own
    checkpoint giving nearly the same gradient."""
    pm = c3_mixed
    gm, (sm, _, _, _) = _grad(pm, c3["pts"], c3["w"], c3["t"])
    g64, (s64, occ, tri, reg) = _grad(c3["plan"], c3["pts"], c3["w"], c3["t"])
    diag = float(np.linalg.norm(c3["pts"].max(0) - c3["pts"].min(0)))
    assert (sm - s64).abs().max().item() <= 1e-6 * diag
    v = torch.tensor(c3["pts"], device="cuda")
    gs = 2.0 * torch.tensor(c3["w"], device="cuda") * (s64 - torch.tensor(c3["t"], device="cuda"))
    g32 = pm.backward(v, occ, tri, reg, gs).cpu().numpy()
    b = g64.cpu().numpy()
    rel = np.linalg.norm(g32 - b) / np.linalg.norm(b)
    print(f"FP32 adjoint vs FP64 adjoint, same checkpoint: {rel:.2e}")
    assert rel <= 1e-5
    assert torch.equal(pm.backward(v, occ, tri, reg, gs), pm.backward(v, occ, tri, reg, gs))
    a = gm.cpu().numpy()
    assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b)


def test_plan_moves_points_and_resizes(c3, cm, orc):
    """Forwards at new positions (a scaled, shifted copy) re-size the workspace and
    equal a fresh voxelization at those positions."""
    from cybermeshgenerator_gb300 import torch_sdf as TS
    plan = TS.SDFPlan(c3["pts"], c3["tris"], c3["grid"])
    moved = c3["pts"] * 0.8 + 0.05
    sd, oc, _, _ = _forward(plan, moved)
    r = cm.voxelize_ex(cm.PLC.from_arrays(moved, c3["tris"]),
                       outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F64, grid=c3["grid"])
    assert np.array_equal(oc.cpu().numpy(), r.occupancy)
    assert np.array_equal(sd.cpu().numpy(), r.sdf64)
    plan.close()
