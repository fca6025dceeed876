"""Self-intersections on the GPU (grid broad phase + Guigue-Devillers on the reference's
orient3d signs) against the reference's self_intersections (fixtures made by it) and
the oracle's all-pairs restatement."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _hits(cm, pts, tris):
    return cm.self_intersections(cm.PLC.from_arrays(pts, tris))


def test_fixtures_match_reference(cm, golden):
    g = golden("detect")
    for name in g["names"]:
        name = str(name)
        got = _hits(cm, g[name + "_points"], g[name + "_triangles"])
        assert np.array_equal(got, g[name + "_hits"]), name


def test_overlapping_icospheres_match_oracle(cm, orc):
    from cybermeshgenerator_gb300 import workloads as W
    p, t = W.jittered_icosphere(4, 0.01, seed=9)
    pts = np.vstack([p, p * 0.93 + np.array([0.41, 0.2, -0.17])])
    tris = np.vstack([t, t + len(p)])
    got = _hits(cm, pts, tris)
    want = orc.self_intersections(pts, tris)
    assert len(want) > 100
    assert np.array_equal(got[:, :2].astype(np.int64), want)
    assert np.array_equal(got[:, 2:5], tris[want[:, 0]]) and np.array_equal(got[:, 5:8], tris[want[:, 1]])


def test_ellipsoid_field_clean_then_one_overlap(cm, orc):
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.ellipsoid_field(n=300, seed=12)      # 384,000 triangles, disjoint
    assert len(_hits(cm, pts, tris)) == 0
    # re-centre ellipsoid 7 on ellipsoid 8, scaled to reach 0.005 beyond 8's bounding
    # radius: it crosses 8, and stays clear of every other ellipsoid, whose bounding
    # spheres (radius >= 0.01) keep at least r_8 + 0.01 from 8's centre
    per_p, per_t = len(pts) // 300, len(tris) // 300
    a, b = slice(7 * per_p, 8 * per_p), slice(8 * per_p, 9 * per_p)
    moved = pts.copy()
    ca, cb = pts[a].mean(0), pts[b].mean(0)
    ra = np.linalg.norm(pts[a] - ca, axis=1).max()
    rb = np.linalg.norm(pts[b] - cb, axis=1).max()
    moved[a] = cb + (pts[a] - ca) * ((rb + 0.005) / ra)
    got = _hits(cm, moved, tris)
    sub_t = np.vstack([tris[7 * per_t:8 * per_t], tris[8 * per_t:9 * per_t]]) - 7 * per_p
    want = orc.self_intersections(np.vstack([moved[a], moved[b]]), sub_t) + 7 * per_t
    assert len(want) > 0
    assert np.array_equal(got[:, :2].astype(np.int64), want)
