"""Grid vertex clustering on the GPU against the reference's simplify (fixtures made by
it) and the oracle restatement: representative points bit for bit, the kept triangles
in the reference's order, the reference's errors; polygon facets; the reference
tests' own properties; the full-size surface."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _simplify(cm, pts, tris, grid):
    out = cm.simplify(cm.PLC.from_arrays(pts, tris), grid)
    return out.points, out.triangles


def _same(got, want_p, want_t):
    p, t = got
    return np.array_equal(p.view(np.uint64), np.asarray(want_p).view(np.uint64)) and np.array_equal(t, want_t)


def test_fixtures_match_reference(cm, golden):
    g = golden("simplify")
    for name in g["names"]:
        name = str(name)
        pts, tris, grid = g[name + "_points"], g[name + "_triangles"], int(g[name + "_grid"])
        want_err = str(g[name + "_error"])
        if want_err:
            with pytest.raises(RuntimeError) as e:
                _simplify(cm, pts, tris, grid)
            assert str(e.value) == want_err, name
            continue
        assert _same(_simplify(cm, pts, tris, grid), g[name + "_out_points"],
                     g[name + "_out_triangles"]), name


@pytest.mark.parametrize("grid", [1, 8, 34, 256, 4096])
def test_ellipsoid_field_matches_oracle(cm, orc, grid):
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.ellipsoid_field(n=300, seed=14)      # 384,000 triangles
    want_p, want_t, err = orc.simplify(pts, tris, grid)
    assert err == ""
    assert _same(_simplify(cm, pts, tris, grid), want_p, want_t)


def test_polygon_facets_fan_like_the_reference(cm, orc):
    # facets of 3 to 7 corners: the reference fans each polygon (simplify.cpp:35-44)
    from cybermeshgenerator_gb300 import workloads as W
    pts, _ = W.jittered_icosphere(3, 0.02, seed=2)
    rng = np.random.default_rng(4)
    plc = cm.PLC().add_points(pts)
    fan = []
    for _ in range(700):
        k = int(rng.integers(3, 8))
        f = rng.choice(len(pts), size=k, replace=False)
        plc.add_facet(f)
        fan += [[f[0], f[i - 1], f[i]] for i in range(2, k)]
    out = cm.simplify(plc, 9)
    want_p, want_t, err = orc.simplify(pts, np.array(fan), 9)
    assert err == ""
    assert _same((out.points, out.triangles), want_p, want_t)


def test_errors_where_reference_is_undefined(cm):
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.jittered_icosphere(2, 0.02, seed=2)
    bad = pts.copy()
    bad[5, 1] = np.nan
    with pytest.raises(RuntimeError, match="non-finite point coordinate"):
        _simplify(cm, bad, tris, 8)
    bad[5, 1] = np.inf
    with pytest.raises(RuntimeError, match="non-finite point coordinate"):
        _simplify(cm, bad, tris, 8)
    t2 = tris.copy()
    t2[3, 2] = len(pts)
    with pytest.raises(RuntimeError, match="facet vertex index out of range"):
        _simplify(cm, pts, t2, 8)
    # the library stays usable after an error
    assert len(_simplify(cm, pts, tris, 8)[1]) > 0


def test_reference_test_properties(cm):
    """tests/test_simplify.cpp:138-167 on the GPU: fewer triangles, enclosed volume
    within 15 %, deterministic, coarser grid keeps no more triangles."""
    from cybermeshgenerator_gb300 import workloads as W

    def volume(p, t):
        a, b, c = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
        return abs(np.einsum("ij,ij->i", a, np.cross(b, c)).sum()) / 6.0

    p, t = W.uv_sphere(1.0, 24, 24)
    q, u = _simplify(cm, p, t, 8)
    assert 0 < len(u) < len(t)
    assert abs(volume(q, u) - volume(p, t)) / volume(p, t) < 0.15
    p, t = W.uv_sphere(1.0, 20, 20)
    a, b = _simplify(cm, p, t, 10), _simplify(cm, p, t, 10)
    assert _same(a, b[0], b[1])
    p, t = W.uv_sphere(1.0, 28, 28)
    assert len(_simplify(cm, p, t, 8)[1]) <= len(_simplify(cm, p, t, 24)[1])


def test_full_size_surface(cm, orc):
    """The 2,560,000-triangle ellipsoid field at the reference's default grid (34) and
    at 512: identical to the oracle; kept triangles have distinct corners and distinct
    sorted triples; representatives number the occupied cells."""
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.ellipsoid_field(n=2000, seed=5)
    plc = cm.PLC.from_arrays(pts, tris)
    for grid in (34, 512):
        out = cm.simplify(plc, grid)
        p, t = out.points, out.triangles
        want_p, want_t, err = orc.simplify(pts, tris, grid)
        assert err == ""
        assert _same((p, t), want_p, want_t), grid
        assert np.all((t[:, 0] != t[:, 1]) & (t[:, 1] != t[:, 2]) & (t[:, 0] != t[:, 2]))
        assert len(np.unique(np.sort(t, axis=1), axis=0)) == len(t)
        lo = pts.min(0)
        inv = grid / (pts.max(0) - lo).max()
        cells = np.clip(((pts - lo) * inv).astype(np.int64), 0, grid - 1)
        assert len(np.unique(cells, axis=0)) == len(p)
