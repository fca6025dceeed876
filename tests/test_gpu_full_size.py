"""GPU path at the full sizes of the measured configurations, against the
reference's own outputs (tests/golden/shsphere256.npz, boxtorus512.npz, made by
tests/golden/make_golden.py) and the oracle.

* the headline SH surface (65,024 triangles) at resolution 126 pad 1 (128^3) and at
  resolution 254 pad 1 (231 x 247 x 256, the grid the bench number is quoted on);
* the 262,156-triangle box + torus on the exact-face 256^3 grid (h = 2^-7, cell
  centres on the box's faces and edges: grazes, nudges, exact signs) and through the
  API at resolution 254 pad 1.

The meshes are read from their serialised float64 bits, so this host and the one that
made the fixtures see the same input. Occupancy is compared bit for bit (SHA-256 of the
reference's grid and the grid itself), in both predicate modes; nudge and exhaustion
counts against the oracle; FP64 distances at 2048 sampled cells bit for bit against the
reference's point_tri_dist2 minimum; the float field at those cells against the
reference's cast of the signed distance; the mixed-precision field within 1e-6 of the
bounding-box diagonal and within its stated per-cell bound of the FP64 field."""
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [("shsphere256", "r126p1"), ("shsphere256", "r254p1"), ("boxtorus512", "facegrid"),
         ("boxtorus512", "r254p1")]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _case(golden, name, gname):
    z = golden(name)
    g = {k[len(gname) + 1:]: v for k, v in z.items() if k.startswith(gname + "_")}
    return z, g


def _run(cm, z, g, **kw):
    plc = cm.PLC.from_arrays(z["points"], z["triangles"])
    if "resolution" in g:
        kw["resolution"], kw["pad"] = int(g["resolution"]), int(g["pad"])
    else:
        kw["grid"] = (g["corner"], g["spacing"], g["dims"])
    return cm.voxelize_ex(plc, **kw)


def _ref_occ(g):
    return np.unpackbits(g["occ_bits"])[:int(np.prod(g["dims"]))]


@pytest.mark.parametrize("name,gname", CASES)
def test_full_size_occupancy_bit_exact(cm, golden, name, gname):
    z, g = _case(golden, name, gname)
    r = _run(cm, z, g, outputs=cm.OUT_OCCUPANCY)
    assert r.dims == tuple(int(d) for d in g["dims"])
    assert np.array_equal(r.corner, g["corner"]) and r.spacing == float(g["spacing"])
    assert _sha(r.occupancy) == str(g["occ_sha"])
    assert np.array_equal(r.occupancy, _ref_occ(g))


@pytest.mark.parametrize("name,gname", CASES)
def test_full_size_exact_predicates_and_nudges(cm, golden, orc, name, gname):
    import oracle as O
    z, g = _case(golden, name, gname)
    grid = orc.grid(g["corner"], g["spacing"], g["dims"])
    for mode in (cm.PRED_COMPAT, cm.PRED_EXACT):
        r = _run(cm, z, g, outputs=cm.OUT_OCCUPANCY, predicates=mode)
        occ, st = orc.occupancy(z["points"], z["triangles"], grid, O.EXACT if mode else O.COMPAT)
        assert np.array_equal(r.occupancy, occ)
        assert r.stats["nudged_columns"] == st["nudged_columns"]
        assert r.stats["exhausted_columns"] == st["exhausted_columns"]
        if name == "boxtorus512":  # the face-aligned and symmetric grids force grazes
            assert st["nudged_columns"] > 0


@pytest.mark.parametrize("name,gname", CASES)
def test_full_size_distances(cm, golden, name, gname):
    z, g = _case(golden, name, gname)
    r = _run(cm, z, g, outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F64 | cm.OUT_SDF_F32)
    vox = g["sample_vox"]
    want = np.sqrt(g["sample_d2"])
    assert np.array_equal(np.abs(r.sdf64[vox]).view(np.uint64), want.view(np.uint64))
    # the reference's float output: float(occupied ? -d : d), sign from occupancy
    inside = _ref_occ(g)[vox].astype(bool)
    ref32 = np.where(inside, -want, want).astype(np.float32)
    assert np.array_equal(r.sdf32[vox].view(np.uint32), ref32.view(np.uint32))
    occ = r.occupancy.astype(bool)
    assert np.all(np.signbit(r.sdf64[occ])) and not np.any(np.signbit(r.sdf64[~occ]))


@pytest.mark.parametrize("name,gname", [("shsphere256", "r254p1"), ("boxtorus512", "facegrid")])
def test_full_size_mixed_precision(cm, golden, name, gname):
    z, g = _case(golden, name, gname)
    plain = _run(cm, z, g, outputs=cm.OUT_SDF_F64 | cm.OUT_OCCUPANCY)
    mixed = _run(cm, z, g, outputs=cm.OUT_SDF_F64 | cm.OUT_OCCUPANCY | cm.OUT_ERROR_BOUND,
                 precision=cm.PREC_MIXED)
    assert np.array_equal(mixed.occupancy, plain.occupancy)
    assert np.array_equal(mixed.occupancy, _ref_occ(g))
    diag = float(np.linalg.norm(z["points"].max(0) - z["points"].min(0)))
    tol = 1e-6 * diag  # stated tolerance: 1e-6 of the bbox diagonal
    err = np.abs(mixed.sdf64 - plain.sdf64)
    assert err.max() <= tol, (err.max(), tol)
    assert np.all(err <= mixed.error_bound.astype(np.float64) + 1e-300)
    band = mixed.error_bound == 0
    assert np.array_equal(mixed.sdf64[band].view(np.uint64), plain.sdf64[band].view(np.uint64))
    vox = g["sample_vox"]
    near = band[vox]
    assert np.array_equal(np.abs(mixed.sdf64[vox][near]), np.sqrt(g["sample_d2"])[near])
