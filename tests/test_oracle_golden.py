"""The oracle restatement against outputs of the reference itself (tests/golden,
made by tests/golden/make_golden.py from the reference's sources). Bit for bit."""
import hashlib

import numpy as np
import pytest

from conftest import unpack_occ

API_CASES = ["icosphere_s3_r58p3", "cube4_r16p1", "cube4deg_r16p1", "uvsphere16_r20p1",
             "brick312_r20p1", "shsphere64_r30p1", "boxtorus64_r62p1"]
# full-size configurations: (fixture, grid) pairs
FULL_CASES = [("shsphere256", "r126p1"), ("shsphere256", "r254p1"), ("boxtorus512", "facegrid"),
              ("boxtorus512", "r254p1")]
GRID_CASES = ["boxtorus64_facegrid", "cube3_facegrid"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", API_CASES)
def test_grid_setup(orc, golden, name):
    g = golden(name)
    grid = orc.make_grid(g["points"], int(g["resolution"]), int(g["pad"]))
    assert grid.dims == tuple(int(d) for d in g["dims"])
    assert grid.spacing == float(g["spacing"])
    assert np.array_equal(np.array(grid.corner), g["corner"])


@pytest.mark.parametrize("name", API_CASES)
def test_occupancy_compat(orc, golden, name):
    g = golden(name)
    grid = orc.make_grid(g["points"], int(g["resolution"]), int(g["pad"]))
    occ, _ = orc.occupancy(g["points"], g["triangles"], grid)
    assert np.array_equal(occ, unpack_occ(g))


@pytest.mark.parametrize("name", GRID_CASES)
def test_occupancy_explicit_grid(orc, golden, name):
    g = golden(name)
    grid = orc.grid(g["corner"], g["spacing"], g["dims"])
    occ, st = orc.occupancy(g["points"], g["triangles"], grid)
    assert np.array_equal(occ, unpack_occ(g))
    assert _sha(occ) == str(g["occ_sha"])


def test_face_grid_forces_nudges(orc, golden):
    g = golden("boxtorus64_facegrid")
    grid = orc.grid(g["corner"], g["spacing"], g["dims"])
    _, st = orc.occupancy(g["points"], g["triangles"], grid)
    assert st["nudged_columns"] > 0
    assert st["exact_calls"] > 0


def test_known_answer_cube_block(golden):
    # tests/test_voxelize.cpp:140-163: R=16, pad=1 -> exactly the 16^3 interior block
    g = golden("cube4_r16p1")
    nx, ny, nz = (int(d) for d in g["dims"])
    occ = unpack_occ(g).reshape(nz, ny, nx)
    block = np.zeros_like(occ)
    block[1:17, 1:17, 1:17] = 1
    assert np.array_equal(occ, block)


@pytest.mark.parametrize("name", ["icosphere_s3_r58p3", "cube4_r16p1", "cube4deg_r16p1",
                                  "uvsphere16_r20p1", "brick312_r20p1", "shsphere64_r30p1"])
def test_sdf_float_bits(orc, golden, name):
    g = golden(name)
    grid = orc.make_grid(g["points"], int(g["resolution"]), int(g["pad"]))
    occ = unpack_occ(g)
    _, s32 = orc.sdf_ring(g["points"], g["triangles"], grid, occ)
    assert _sha(s32) == str(g["sdf32_sha"])
    if "sdf32" in g:
        assert np.array_equal(s32.view(np.uint32), g["sdf32"].view(np.uint32))


@pytest.mark.parametrize("name", API_CASES + GRID_CASES)
def test_sdf64_samples_bruteforce(orc, golden, name):
    g = golden(name)
    grid = orc.grid(g["corner"], g["spacing"], g["dims"])
    d2, _, _ = orc.sdf_brute(g["points"], g["triangles"], grid, g["sample_vox"])
    assert np.array_equal(d2.view(np.uint64), g["sample_d2"].view(np.uint64))


def test_ring_equals_bruteforce(orc, golden):
    g = golden("uvsphere16_r20p1")
    grid = orc.grid(g["corner"], g["spacing"], g["dims"])
    vox = np.arange(grid.ncell)
    d_ring = orc.sdf_ring_sample(g["points"], g["triangles"], grid, vox)
    d_brute, _, _ = orc.sdf_brute(g["points"], g["triangles"], grid, vox)
    assert np.array_equal(d_ring, d_brute)


@pytest.mark.parametrize("kind", ["orient3d", "insphere"])
@pytest.mark.parametrize("mode", ["compat", "exact"])
def test_predicate_signs(orc, golden, kind, mode):
    import oracle as O
    g = golden("predicates")
    got = orc.stream(kind, g[kind + "_soa"], O.COMPAT if mode == "compat" else O.EXACT)
    assert np.array_equal(got, g[kind + "_" + mode])


def test_compat_differs_from_exact(golden):
    # the reference's as-initialised signs are not the exact ones on near cases
    g = golden("predicates")
    assert (g["orient3d_compat"] != g["orient3d_exact"]).sum() > 0


def _fd_grad(orc, pts, tris, grid, occ, w, t, verts, h=1e-6):
    """Central differences of L = sum w (sdf - t)^2 of the oracle's FP64 distance,
    in difference form: L(+h) - L(-h) = sum w (s+ - s-)(s+ + s- - 2t), so that
    only the cells that change carry rounding."""
    sgn = np.where(occ != 0, -1.0, 1.0)
    out = np.zeros((len(verts), 3))
    for i, v in enumerate(verts):
        for a in range(3):
            s = []
            for step in (h, -h):
                p = pts.copy()
                p[v, a] += step
                d2, _, _ = orc.sdf_brute(p, tris, grid)
                s.append(sgn * np.sqrt(d2))
            out[i, a] = np.sum(w * (s[0] - s[1]) * (s[0] + s[1] - 2 * t)) / (2 * h)
    return out


def test_oracle_gradient_matches_central_differences(orc):
    """The FP64 host analytic gradient (the adjoint's second check) against FP64
    central differences, h = 1e-6, relative 1e-5."""
    from cybermeshgenerator_gb300 import workloads as W
    import oracle as O
    pts, tris = W.jittered_icosphere(2, 0.02, seed=7)
    g = orc.make_grid(pts, 14, 1)
    occ, _ = orc.occupancy(pts, tris, g, O.COMPAT)
    d2, tri, _ = orc.sdf_brute(pts, tris, g)
    rng = np.random.default_rng(11)
    w = rng.uniform(0.0, 1.0, g.ncell)
    t = rng.normal(0.0, 0.1, g.ncell)
    grad = orc.sdf_grad(pts, tris, g, occ, tri, w, t)
    verts = rng.choice(len(pts), size=8, replace=False)
    fd = _fd_grad(orc, pts, tris, g, occ, w, t, verts)
    an = grad[verts]
    assert np.linalg.norm(fd - an) <= 1e-5 * np.linalg.norm(an)
    # vertices no cell's nearest triangle touches have zero gradient
    used = np.unique(tris[tri[tri >= 0]].ravel())
    assert np.all(grad[np.setdiff1d(np.arange(len(pts)), used)] == 0.0)


def test_stl_reader_matches_reference(orc, golden):
    """The STL restatement against the reference's read_stl on every fixture: points
    bit for bit (first occurrence kept, signed zeros merged), triangles, errors."""
    g = golden("stl")
    for name in g["names"]:
        name = str(name)
        pts, tri, err = orc.stl_read(g[name + "_bytes"].tobytes())
        assert err == str(g[name + "_error"]), name
        if err:
            continue
        assert np.array_equal(pts.view(np.uint64), g[name + "_points"].view(np.uint64)), name
        assert np.array_equal(tri, g[name + "_triangles"]), name


def test_self_intersections_match_reference(orc, golden):
    """The self-intersection restatement against the reference's self_intersections on
    every fixture: the same (i, j) pairs in the same order."""
    g = golden("detect")
    for name in g["names"]:
        name = str(name)
        got = orc.self_intersections(g[name + "_points"], g[name + "_triangles"])
        want = g[name + "_hits"]
        assert np.array_equal(got, want[:, :2].astype(np.int64)), name


def test_simplify_matches_reference(orc, golden):
    """The simplify restatement against the reference's simplify on every fixture:
    representative points bit for bit, kept triangles in order, errors."""
    g = golden("simplify")
    for name in g["names"]:
        name = str(name)
        pts, tri, err = orc.simplify(g[name + "_points"], g[name + "_triangles"], int(g[name + "_grid"]))
        assert err == str(g[name + "_error"]), name
        if err:
            continue
        assert np.array_equal(pts.view(np.uint64), g[name + "_out_points"].view(np.uint64)), name
        assert np.array_equal(tri, g[name + "_out_triangles"]), name


def test_simplify_reference_properties(golden):
    """The reference tests' own checks on its fixtures (tests/test_simplify.cpp:138-174):
    a coarser surface enclosing nearly the same volume, fewer triangles at a coarser
    grid."""
    g = golden("simplify")

    def volume(p, t):
        a, b, c = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
        return abs(np.einsum("ij,ij->i", a, np.cross(b, c)).sum()) / 6.0

    p, t = g["uvsphere24_g8_points"], g["uvsphere24_g8_triangles"]
    q, u = g["uvsphere24_g8_out_points"], g["uvsphere24_g8_out_triangles"]
    assert 0 < len(u) < len(t)
    assert abs(volume(q, u) - volume(p, t)) / volume(p, t) < 0.15
    assert len(g["uvsphere28_g8_out_triangles"]) <= len(g["uvsphere28_g24_out_triangles"])
    # every kept triangle has three distinct corners and no sorted triple repeats
    for name in g["names"]:
        name = str(name)
        u = g[name + "_out_triangles"]
        if len(u):
            assert np.all((u[:, 0] != u[:, 1]) & (u[:, 1] != u[:, 2]) & (u[:, 0] != u[:, 2]))
            assert len(np.unique(np.sort(u, axis=1), axis=0)) == len(u)


def test_orient3d_values_match_reference(orc, golden):
    """robust::orient3d VALUES (not just signs) restated: 3000 inputs whose rounded
    determinant is zero (every adaptive stage, the exact expansion's top component
    included) and 500 random ones, bit for bit against the reference."""
    g = golden("sizing")
    P = g["o3_points"]
    soa = np.stack([P[:, i, j] for i in range(4) for j in range(3)])
    got = orc.orient3d_values(soa)
    assert np.array_equal(got.view(np.uint64), g["o3_values"].view(np.uint64))
    assert np.count_nonzero(g["o3_values"][:3000]) > 0


def test_sizing_matches_reference(orc, golden):
    """The sizing-field restatement against the reference's from_background closure on
    every fixture, bit for bit (NaN where the reference gives NaN)."""
    g = golden("sizing")
    for name in g["names"]:
        name = str(name)
        got, which = orc.sizing(g[name + "_points"], g[name + "_tets"], g[name + "_sizes"],
                                float(g[name + "_scale"]), g[name + "_queries"])
        assert np.array_equal(got.view(np.uint64), g[name + "_values"].view(np.uint64)), name


def test_sizing_reference_properties(orc):
    """tests/test_sizing.cpp:85-108 on the restatement: exact at a node, about 0.45 at
    the centre of the six-tetrahedron cube, scale 0.5 halves a constant field."""
    from cybermeshgenerator_gb300 import workloads as W
    P, T = W.kuhn_tet_mesh(1)
    S = 0.2 + 0.5 * P[:, 0]
    v, _ = orc.sizing(P, T, S, 1.0, np.vstack([P[1], [0.5, 0.5, 0.5]]))
    assert abs(v[0] - (0.2 + 0.5 * P[1, 0])) < 1e-6
    assert 0.2 < v[1] < 0.7 and abs(v[1] - 0.45) < 0.05
    full, _ = orc.sizing(P, T, np.full(len(P), 0.4), 1.0, [[0.5, 0.5, 0.5]])
    half, _ = orc.sizing(P, T, np.full(len(P), 0.4), 0.5, [[0.5, 0.5, 0.5]])
    assert abs(half[0] - 0.5 * full[0]) < 1e-9 and abs(full[0] - 0.4) < 1e-6


def test_exhausted_nudges_keep_partial_heights(orc, golden):
    """A zero-area facet makes every nudge of 81 columns graze; the reference keeps the
    crossings of the triangles before it in bucket order (voxelize.cpp:158-165), which
    differs from the plain cube's occupancy."""
    g = golden("cube4deg_r16p1")
    grid = orc.make_grid(g["points"], int(g["resolution"]), int(g["pad"]))
    for mode in (0, 1):
        occ, st = orc.occupancy(g["points"], g["triangles"], grid, mode)
        assert st["exhausted_columns"] == 81 and st["nudged_columns"] == 131
        assert np.array_equal(occ, unpack_occ(g))
    plain = golden("cube4_r16p1")
    assert int((unpack_occ(plain) != unpack_occ(g)).sum()) == 720


def _full(golden, name, gname):
    z = golden(name)
    return z, {k[len(gname) + 1:]: v for k, v in z.items() if k.startswith(gname + "_")}


@pytest.mark.parametrize("name,gname", FULL_CASES)
def test_full_size_occupancy(orc, golden, name, gname):
    z, g = _full(golden, name, gname)
    if "resolution" in g:
        grid = orc.make_grid(z["points"], int(g["resolution"]), int(g["pad"]))
        assert grid.dims == tuple(int(d) for d in g["dims"])
        assert np.array_equal(np.array(grid.corner), g["corner"])
    else:
        grid = orc.grid(g["corner"], g["spacing"], g["dims"])
    occ, st = orc.occupancy(z["points"], z["triangles"], grid)
    assert _sha(occ) == str(g["occ_sha"])
    assert np.array_equal(occ, np.unpackbits(g["occ_bits"])[:grid.ncell])
    if name == "boxtorus512":
        assert st["nudged_columns"] > 0 and st["exact_calls"] > 0
    d2, _, _ = orc.sdf_brute(z["points"], z["triangles"], grid, g["sample_vox"])
    assert np.array_equal(d2.view(np.uint64), g["sample_d2"].view(np.uint64))


def test_full_size_meshes_match_generators(golden):
    """The serialised meshes are the generators' (triangle indices exactly; point
    coordinates to the last bits, which transcendental functions may round
    differently on another host)."""
    from cybermeshgenerator_gb300 import workloads as W
    for name, (p, t) in (("shsphere256", W.sh_sphere(256, 128, seed=3)),
                         ("boxtorus512", W.box_and_torus(512, 256))):
        z = golden(name)
        assert np.array_equal(z["triangles"], t)
        assert np.allclose(z["points"], p, rtol=0, atol=1e-13)
