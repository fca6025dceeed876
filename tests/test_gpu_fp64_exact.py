"""The FP64 path on 16^3 bricks (CMG_PREC_FP64: the FP32 pass with its bounds widened to
every near-tie of each cell's FP32 minimum, then the FP64 distance in the reference's
order over those) against the plain FP64 path (CMG_PREC_FP64_PLAIN: every candidate in
FP64). Every output equals bit for bit: occupancy, float and FP64 distance, nearest
triangle and Ericson region. Covered: the golden fixtures (the UV sphere's poles have
more near-ties than a cell keeps, so the band pass takes those cells), the full-size
headline grid and the full-size box + torus on its exact-face 256^3 grid. The FP64
evaluations drop by well over an order of magnitude."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OUTS = 1 | 2 | 4 | 8  # occupancy, float and FP64 distance, nearest triangle + region
ARRAYS = ("occupancy", "sdf32", "sdf64", "nearest_triangle", "nearest_region")


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint8) if a.dtype.itemsize == 1 else a.view(f"u{a.dtype.itemsize}")


def _both(cm, plc, **kw):
    exact = cm.voxelize_ex(plc, outputs=OUTS, precision=cm.PREC_FP64, **kw)
    plain = cm.voxelize_ex(plc, outputs=OUTS, precision=cm.PREC_FP64_PLAIN, **kw)
    for n in ARRAYS:
        assert np.array_equal(_bits(getattr(exact, n)), _bits(getattr(plain, n))), n
    return exact, plain


def _grid_kw(g):
    if "resolution" in g:
        return dict(resolution=int(g["resolution"]), pad=int(g["pad"]))
    return dict(grid=(g["corner"], g["spacing"], g["dims"]))


@pytest.mark.parametrize("name", ["cube4_r16p1", "uvsphere16_r20p1", "icosphere_s3_r58p3",
                                  "shsphere64_r30p1", "boxtorus64_facegrid", "boxtorus64_r62p1",
                                  "cube4deg_r16p1", "brick312_r20p1"])
def test_exact_equals_plain_on_fixtures(cm, golden, name):
    g = golden(name)
    exact, plain = _both(cm, cm.PLC.from_arrays(g["points"], g["triangles"]), **_grid_kw(g))
    assert exact.stats["fp64_evaluations"] < plain.stats["evaluations"]


def test_exact_equals_plain_on_the_headline_grid(cm, golden):
    z = golden("shsphere256")
    exact, plain = _both(cm, cm.PLC.from_arrays(z["points"], z["triangles"]), resolution=254, pad=1)
    # the FP32 pass carries the search; FP64 only for the near-ties
    assert exact.stats["fp64_evaluations"] * 20 < plain.stats["evaluations"]
    # the poles of the 256 x 128 bands have more near-ties than a cell keeps
    assert 0 < exact.stats["band_cells"] < exact.stats["cells"] // 10


def test_exact_equals_plain_on_the_ellipsoid_field(cm):
    """2000 small ellipsoids (2.56M triangles) at resolution 254 pad 1: cells mostly far
    from every surface, whose near-ties come from neighbouring bodies."""
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.ellipsoid_field()
    exact, plain = _both(cm, cm.PLC.from_arrays(pts, tris), resolution=254, pad=1)
    assert exact.stats["fp64_evaluations"] * 20 < plain.stats["evaluations"]


def test_exact_equals_plain_on_the_box_torus_face_grid(cm, golden):
    z = golden("boxtorus512")
    grid = (z["facegrid_corner"], float(z["facegrid_spacing"]), z["facegrid_dims"])
    _both(cm, cm.PLC.from_arrays(z["points"], z["triangles"]), grid=grid)
