"""GPU path against the reference's own outputs (tests/golden) and the oracle.

Occupancy and the FP64 signed distance are compared bit for bit; the mixed
precision field against the FP64 one with the stated tolerance (1e-6 of the
bounding-box diagonal) and the stated per-cell bound."""
import hashlib

import numpy as np
import pytest

from conftest import unpack_occ

pytestmark = pytest.mark.gpu

API_CASES = ["icosphere_s3_r58p3", "cube4_r16p1", "cube4deg_r16p1", "uvsphere16_r20p1",
             "brick312_r20p1", "shsphere64_r30p1", "boxtorus64_r62p1"]
GRID_CASES = ["boxtorus64_facegrid", "cube3_facegrid"]
ALL = API_CASES + GRID_CASES


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _plc(cm, g):
    return cm.PLC.from_arrays(g["points"], g["triangles"])


def _run(cm, g, name, **kw):
    if name in GRID_CASES:
        kw["grid"] = (g["corner"], g["spacing"], g["dims"])
    else:
        kw["resolution"], kw["pad"] = int(g["resolution"]), int(g["pad"])
    return cm.voxelize_ex(_plc(cm, g), **kw)


def _diag(points):
    return float(np.linalg.norm(points.max(0) - points.min(0)))


@pytest.mark.parametrize("name", ALL)
def test_occupancy_bit_exact(cm, golden, name):
    g = golden(name)
    r = _run(cm, g, name, outputs=cm.OUT_OCCUPANCY)
    assert r.dims == tuple(int(d) for d in g["dims"])
    assert np.array_equal(np.array(r.corner), g["corner"])
    assert np.array_equal(r.occupancy, unpack_occ(g))


@pytest.mark.parametrize("name", GRID_CASES + ["icosphere_s3_r58p3"])
def test_occupancy_exact_predicates(cm, golden, orc, name):
    import oracle as O
    g = golden(name)
    r = _run(cm, g, name, outputs=cm.OUT_OCCUPANCY, predicates=cm.PRED_EXACT)
    grid = orc.grid(r.corner, r.spacing, r.dims)
    occ, _ = orc.occupancy(g["points"], g["triangles"], grid, O.EXACT)
    assert np.array_equal(r.occupancy, occ)


def test_nudge_statistics_match_oracle(cm, golden, orc):
    g = golden("boxtorus64_facegrid")
    r = _run(cm, g, "boxtorus64_facegrid", outputs=cm.OUT_OCCUPANCY)
    grid = orc.grid(g["corner"], g["spacing"], g["dims"])
    _, st = orc.occupancy(g["points"], g["triangles"], grid)
    assert r.stats["nudged_columns"] == st["nudged_columns"] > 0
    assert r.stats["exhausted_columns"] == st["exhausted_columns"]


@pytest.mark.parametrize("mode", [0, 1])
def test_exhausted_nudges_keep_last_partial(cm, golden, orc, mode):
    """A zero-area facet halfway through the triangle list: 81 columns graze on all six
    nudges and keep the crossings of the triangles before it (voxelize.cpp:158-165)."""
    g = golden("cube4deg_r16p1")
    r = _run(cm, g, "cube4deg_r16p1", outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F32, predicates=mode)
    grid = orc.grid(r.corner, r.spacing, r.dims)
    occ, st = orc.occupancy(g["points"], g["triangles"], grid, mode)
    assert r.stats["exhausted_columns"] == st["exhausted_columns"] == 81
    assert r.stats["nudged_columns"] == st["nudged_columns"]
    assert np.array_equal(r.occupancy, occ)
    assert np.array_equal(r.occupancy, unpack_occ(g))
    assert _sha(r.sdf32) == str(g["sdf32_sha"])


@pytest.mark.parametrize("name", [c for c in API_CASES if c != "boxtorus64_r62p1"])
@pytest.mark.parametrize("brick", [4, 8, 16])
def test_sdf_float_bit_exact(cm, golden, name, brick):
    g = golden(name)
    r = _run(cm, g, name, outputs=cm.OUT_SDF_F32, brick=brick)
    assert _sha(r.sdf32) == str(g["sdf32_sha"])


@pytest.mark.parametrize("name", ALL)
def test_sdf64_matches_reference_distance(cm, golden, name):
    g = golden(name)
    r = _run(cm, g, name, outputs=cm.OUT_SDF_F64 | cm.OUT_OCCUPANCY)
    got = np.abs(r.sdf64[g["sample_vox"]])
    want = np.sqrt(g["sample_d2"])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    # sign from occupancy, never approximated
    occ = r.occupancy.astype(bool)
    assert np.all(np.signbit(r.sdf64[occ])) and not np.any(np.signbit(r.sdf64[~occ]))


@pytest.mark.parametrize("name", ["icosphere_s3_r58p3", "shsphere64_r30p1", "boxtorus64_facegrid",
                                  "cube4deg_r16p1", "uvsphere16_r20p1"])
@pytest.mark.parametrize("brick", [4, 8, 16])
def test_mixed_precision_error(cm, golden, name, brick):
    # cube4deg_r16p1 holds a zero-area facet of exactly collinear dyadic points,
    # uvsphere16_r20p1 slivers at its poles
    g = golden(name)
    plain = _run(cm, g, name, outputs=cm.OUT_SDF_F64, brick=brick)
    mixed = _run(cm, g, name, outputs=cm.OUT_SDF_F64 | cm.OUT_ERROR_BOUND,
                 precision=cm.PREC_MIXED, brick=brick, band=1.0)
    tol = 1e-6 * _diag(g["points"])  # stated tolerance: 1e-6 of the bbox diagonal
    err = np.abs(mixed.sdf64 - plain.sdf64)
    assert err.max() <= tol, (err.max(), tol)
    assert np.all(err <= mixed.error_bound.astype(np.float64) + 1e-300)
    # band cells are refined in FP64: bit-identical to the plain path
    band = mixed.error_bound == 0
    assert band.sum() == mixed.stats["band_cells"] > 0
    assert np.array_equal(mixed.sdf64[band].view(np.uint64), plain.sdf64[band].view(np.uint64))
    assert np.array_equal(np.signbit(mixed.sdf64), np.signbit(plain.sdf64))


def test_nearest_triangle_checkpoint(cm, golden, orc):
    g = golden("uvsphere16_r20p1")
    r = _run(cm, g, "uvsphere16_r20p1", outputs=cm.OUT_SDF_F64 | cm.OUT_NEAREST)
    grid = orc.grid(r.corner, r.spacing, r.dims)
    d2, tri, reg = orc.sdf_brute(g["points"], g["triangles"], grid)
    assert np.array_equal(np.abs(r.sdf64), np.sqrt(d2))
    # the checkpointed triangle attains the minimum (ties may pick another id)
    pts, T = g["points"], g["triangles"]
    for v in np.random.default_rng(0).choice(grid.ncell, 300, replace=False):
        p = np.array([grid.corner[a] + (idx + 0.5) * grid.spacing for a, idx in
                      enumerate(np.unravel_index(v, r.dims[::-1])[::-1])])
        t = r.nearest_triangle[v]
        d, rg = orc.point_tri_dist2(p, *pts[T[t]])
        assert d == d2[v] and rg == r.nearest_region[v]


@pytest.mark.parametrize("name", ["icosphere_s3_r58p3", "shsphere64_r30p1", "boxtorus64_facegrid"])
def test_mixed_record_access_modes_identical(cm, golden, name):
    """Reading records from L1/L2 or staging them in shared memory evaluates the
    same candidates in the same order: identical outputs."""
    g = golden(name)
    outs = cm.OUT_SDF_F64 | cm.OUT_NEAREST
    r = [_run(cm, g, name, outputs=outs, precision=cm.PREC_MIXED, stage=m) for m in (0, 1)]
    for x in r[1:]:
        assert np.array_equal(x.sdf64.view(np.uint64), r[0].sdf64.view(np.uint64))
        assert np.array_equal(x.nearest_triangle, r[0].nearest_triangle)
        assert np.array_equal(x.nearest_region, r[0].nearest_region)
