"""Generate the golden fixtures from the reference's own code.

Run where the reference sources are available (it builds oracle/_ref from them;
CMG_REFERENCE_ROOT names the reference source tree):

    CMG_REFERENCE_ROOT=<tree> python tests/golden/make_golden.py [case ...]

Every fixture stores its input mesh as raw float64/int32 bits (so hosts whose
libm differs still see identical inputs) and the reference's outputs:
  - occupancy through the public cmg::voxelize::voxelize (or classify_occupancy
    on an explicit grid), bit-packed;
  - float SDF through the public entry point (full, or its SHA-256 for big grids);
  - FP64 squared distances at sampled cells from the reference's point_tri_dist2
    (brute force, i.e. before the float cast);
  - orient3d / insphere signs as the reference initialises them (robust::*) and
    exact (predicates::*exact).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from cybermeshgenerator_gb300 import workloads as W  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)


def api_case(ref, name, pts, tris, resolution, pad, full_sdf=True, nsample=512, seed=0):
    facets = [list(t) for t in tris]
    st, origin, sp, dims, occ = ref.voxelize(pts, facets, resolution, pad, 0)
    assert st == 0, (name, st)
    st2, _, _, _, sdf = ref.voxelize(pts, facets, resolution, pad, 1)
    assert st2 == 0
    rc, corner, sp2, dims2 = ref.make_grid(pts, resolution, pad)
    assert dims2 == dims and sp2 == sp
    n = int(np.prod(dims))
    rng = np.random.default_rng(seed)
    vox = np.sort(rng.choice(n, size=min(nsample, n), replace=False)).astype(np.int64)
    d2 = ref.dist2_brute(pts, tris, corner, sp, dims, vox)
    out = dict(points=pts, triangles=tris.astype(np.int32), resolution=np.int32(resolution),
               pad=np.int32(pad), dims=np.array(dims, np.int32), corner=corner,
               spacing=np.float64(sp), origin=origin, occ_bits=np.packbits(occ),
               sdf32_sha=np.array(sha(sdf)), sample_vox=vox, sample_d2=d2)
    if full_sdf:
        out["sdf32"] = sdf
    save(name, **out)
    return occ, sdf


def grid_case(ref, name, pts, tris, corner, spacing, dims, nsample=512, seed=0):
    occ = ref.occupancy_grid(pts, tris, corner, spacing, dims)
    n = int(np.prod(dims))
    rng = np.random.default_rng(seed)
    vox = np.sort(rng.choice(n, size=min(nsample, n), replace=False)).astype(np.int64)
    d2 = ref.dist2_brute(pts, tris, corner, spacing, dims, vox)
    save(name, points=pts, triangles=tris.astype(np.int32), dims=np.array(dims, np.int32),
         corner=np.asarray(corner, np.float64), spacing=np.float64(spacing),
         occ_bits=np.packbits(occ), occ_sha=np.array(sha(occ)), sample_vox=vox, sample_d2=d2)
    return occ


def full_case(ref, name, pts, tris, grids, nsample=2048, seed=0):
    """A full-size configuration: the mesh as raw bits and, per grid, the reference's
    occupancy (public voxelize for ("api", resolution, pad), classify_occupancy for
    ("grid", corner, spacing, dims)) as a SHA-256 and bit-packed, plus FP64 squared
    distances (brute-force point_tri_dist2) at sampled cells."""
    out = dict(points=pts, triangles=tris.astype(np.int32), grids=np.array([g[0] for g in grids]))
    facets = [list(t) for t in tris]
    for gname, g in grids:
        if g[0] == "api":
            _, resolution, pad = g
            st, origin, sp, dims, occ = ref.voxelize(pts, facets, resolution, pad, 0)
            assert st == 0, (name, gname, st)
            rc, corner, sp2, dims2 = ref.make_grid(pts, resolution, pad)
            assert dims2 == dims and sp2 == sp
            out[gname + "_resolution"] = np.int32(resolution)
            out[gname + "_pad"] = np.int32(pad)
        else:
            _, corner, sp, dims = g
            occ = ref.occupancy_grid(pts, tris, corner, sp, dims)
        n = int(np.prod(dims))
        rng = np.random.default_rng(seed)
        vox = np.sort(rng.choice(n, size=min(nsample, n), replace=False)).astype(np.int64)
        out[gname + "_dims"] = np.array(dims, np.int32)
        out[gname + "_corner"] = np.asarray(corner, np.float64)
        out[gname + "_spacing"] = np.float64(sp)
        out[gname + "_occ_sha"] = np.array(sha(occ))
        out[gname + "_occ_bits"] = np.packbits(occ)
        out[gname + "_sample_vox"] = vox
        out[gname + "_sample_d2"] = ref.dist2_brute(pts, tris, corner, sp, dims, vox)
    out["grid_names"] = np.array([g for g, _ in grids])
    del out["grids"]
    save(name, **out)


def pred_case(ref, name, n, seed):
    out = {}
    for kind, npt in (("orient3d", 4), ("insphere", 5)):
        S = W.predicate_stream(n, kind, degenerate=0.25, near=0.25, seed=seed)
        comp = np.zeros(n, np.int8)
        ex = np.zeros(n, np.int8)
        for i in range(n):
            p = [S[3 * k:3 * k + 3, i] for k in range(npt)]
            comp[i] = np.sign(ref.pred(kind, *p))
            ex[i] = np.sign(ref.pred(kind + "exact", *p))
        out[kind + "_soa"] = S
        out[kind + "_compat"] = comp
        out[kind + "_exact"] = ex
    save(name, **out)


def stl_cases():
    """(name, image bytes) of the STL fixtures: binary and ASCII variants and errors."""
    cases = []
    p, t = W.jittered_icosphere(2, 0.02, seed=4)
    cases.append(("bin_icosphere", W.stl_binary(p * 3.7 - 1.25, t)))
    # +0 and -0 (equal as coordinates), a repeated and a degenerate triangle
    q = np.array([[0.0, 0.0, 0.0], [-0.0, 1.0, 0.0], [1.0, -0.0, 0.0], [0.0, 0.0, 1.0],
                  [0.0, -0.0, -0.0], [2.5, 2.5, 2.5]])
    tt = np.array([[0, 1, 2], [4, 2, 3], [1, 2, 3], [0, 1, 3], [1, 2, 3], [5, 5, 5]])
    cases.append(("bin_signed_zero", W.stl_binary(q, tt)))
    one = np.array([[0, 0, 0], [2, 0, 0], [0, 3, 0]], float)
    cases.append(("bin_one", W.stl_binary(one, [[0, 1, 2]])))
    tet = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    ttet = [[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]]
    cases.append(("ascii_tetra", W.stl_ascii(tet, ttet)))
    cases.append(("ascii_variants", W.stl_ascii(p * 0.3, t, fmt="{:.17g}", crlf=True,
                                                comments=True, commas=True, upper=True)))
    odd = (b"solid odd\n facet normal 0 0 1\n  outer loop\n"
           b"   vertex 1e0 +2.5 -0\n   vertex 0x1p-2 .5 3E-1\n   vertex 7 8 9 extra tokens\n"
           b"  endloop\n endfacet\nendsolid\n")
    cases.append(("ascii_number_forms", odd))
    cases.append(("ascii_short_vertex", b"solid bad\n  facet normal 0 0 1\n    outer loop\n"
                                        b"      vertex 0 0\n    endloop\n  endfacet\nendsolid bad\n"))
    cases.append(("ascii_non_numeric", b"solid bad\nvertex 0 0 0\nvertex 1 0 0\nvertex 0 1x 0\n"))
    cases.append(("ascii_out_of_range", b"solid bad\nvertex 0 0 0\nvertex 1e400 0 0\nvertex 0 1 0\n"))
    cases.append(("ascii_four_vertices", b"vertex 0 0 0\nvertex 1 0 0\nvertex 0 1 0\nvertex 0 0 1\n"))
    cases.append(("empty", b""))
    return cases


def detect_cases():
    """(name, points, triangles) of the self-intersection fixtures."""
    cases = []
    cases.append(("crossing", np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0], [0, -1, -1], [0, 1, -1],
                                        [0, 0, 1]], float), np.array([[0, 1, 2], [3, 4, 5]])))
    cp, ct = W.unit_box()
    cases.append(("cube", cp, ct))
    tet = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    cases.append(("tetra", tet, np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]])))
    p, t = W.jittered_icosphere(2, 0.02, seed=3)
    cases.append(("two_icospheres", np.vstack([p, p * 0.9 + 0.5]), np.vstack([t, t + len(p)])))
    rng = np.random.default_rng(17)
    soup = rng.random((450, 3))
    cases.append(("random_soup", soup, np.arange(450).reshape(150, 3)))
    # integer grid points: coplanar overlaps, vertex and edge contacts, repeated indices,
    # an out-of-range index (skipped)
    g = np.array([[x, y, z] for z in range(3) for y in range(3) for x in range(3)], float)
    idx = lambda x, y, z: x + 3 * y + 9 * z
    tri = [[idx(0, 0, 0), idx(2, 0, 0), idx(0, 2, 0)],      # z = 0
           [idx(1, 1, 0), idx(2, 2, 0), idx(0, 2, 0)],      # z = 0, overlapping (coplanar)
           [idx(1, 0, 1), idx(1, 0, 0), idx(1, 1, 2)],      # touches the first at a vertex/edge
           [idx(0, 1, 0), idx(2, 1, 2), idx(0, 1, 2)],      # through the z = 0 triangles
           [idx(1, 1, 1), idx(1, 1, 1), idx(2, 2, 2)],      # repeated index
           [idx(0, 0, 2), idx(2, 0, 2), idx(1, 2, 0)],
           [idx(2, 0, 1), idx(0, 2, 1), idx(0, 0, 1)],      # z = 1
           [idx(1, 1, 0), idx(1, 1, 2), idx(2, 0, 1)],      # contains an edge point of the last
           [idx(0, 0, 0), 99, idx(1, 1, 1)]]                # out of range
    cases.append(("grid_degenerate", g, np.array(tri)))
    return cases


def detect_case(ref, manifest):
    out = {}
    names = []
    for name, pts, tris in detect_cases():
        out[name + "_points"] = np.asarray(pts, float)
        out[name + "_triangles"] = np.asarray(tris, np.int32)
        out[name + "_hits"] = ref.self_intersections(pts, tris)
        names.append(name)
    out["names"] = np.array(names)
    save("detect", **out)
    manifest["detect"] = ("self-intersection configurations (the reference tests' crossing, cube and "
                          "tetrahedron, overlapping icospheres, a random soup, degenerate grid "
                          "contacts) with the reference's self_intersections rows")


def simplify_cases():
    """(name, points, triangles, grid) of the simplify fixtures."""
    cases = []
    # the reference tests' UV spheres at their grids (tests/test_simplify.cpp:138-174)
    for (n, g) in ((24, 8), (20, 10), (28, 8), (28, 24), (8, 0)):
        p, t = W.uv_sphere(1.0, n, n)
        cases.append((f"uvsphere{n}_g{g}", p, t, g))
    p, t = W.jittered_icosphere(3, 0.02, seed=5)
    for g in (1, 3, 34):
        cases.append((f"icosphere_g{g}", p, t, g))
    p, t = W.sh_sphere(nlon=64, nlat=32, seed=4)
    cases.append(("shsphere64_g34", p, t, 34))
    # vertices on cell boundaries, signed zeros, collapsed triangles
    q = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [-0.0, 0.5, 0.25],
                  [0.5, -0.0, 0.75], [0.25, 0.25, 0.25]], float)
    tq = np.array([[0, 1, 2], [0, 2, 3], [0, 3, 1], [1, 2, 3], [4, 5, 6], [0, 4, 5]])
    for g in (2, 4):
        cases.append((f"boundaries_g{g}", q, tq, g))
    # repeated triangles, also reversed: the first occurrence's orientation is kept
    p, t = W.jittered_icosphere(2, 0.01, seed=6)
    cases.append(("repeats_g6", p, np.vstack([t, t[::-1, ::-1], t[:17]]), 6))
    # 64-bit key wrap: with grid 2^22 the cells ix and ix + 2^20 share a key
    w = np.array([[0, 0, 0], [0.25, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    cases.append(("wrap_g4194304", w, np.array([[0, 1, 2], [1, 2, 3], [0, 2, 3]]), 1 << 22))
    cases.append(("icosphere_gmax", *W.jittered_icosphere(2, 0.01, seed=7), 2 ** 31 - 1))
    rng = np.random.default_rng(23)
    soup = np.round(rng.normal(size=(300, 3)) * 8) / 8
    cases.append(("quantized_soup_g7", soup, rng.integers(0, 300, size=(500, 3)), 7))
    cases.append(("points_only_g5", rng.random((40, 3)), np.zeros((0, 3), np.int32), 5))
    cases.append(("no_points", np.zeros((0, 3)), np.zeros((0, 3), np.int32), 8))
    cases.append(("grid_negative", q, tq, -3))
    cases.append(("flat", np.ones((5, 3)), np.array([[0, 1, 2]]), 4))
    return cases


def simplify_case(ref, manifest):
    out = {}
    names = []
    for name, pts, tris, g in simplify_cases():
        rp, rt, err = ref.simplify(pts, tris, g)
        out[name + "_points"] = np.asarray(pts, float).reshape(-1, 3)
        out[name + "_triangles"] = np.asarray(tris, np.int32).reshape(-1, 3)
        out[name + "_grid"] = np.array(g, np.int64)
        out[name + "_error"] = np.array(err)
        out[name + "_out_points"] = rp if rp is not None else np.zeros((0, 3))
        out[name + "_out_triangles"] = rt if rt is not None else np.zeros((0, 3), np.int32)
        names.append(name)
    out["names"] = np.array(names)
    save("simplify", **out)
    manifest["simplify"] = ("grid vertex clustering (the reference tests' UV spheres at their grids, "
                            "icospheres at grids 1/3/34/2^31-1, cell boundaries and signed zeros, "
                            "repeated and reversed triangles, 64-bit key wrap, errors) with the "
                            "reference's simplify output")


def sizing_cases():
    """(name, points, tets, node sizes, scale, queries) of the sizing-field fixtures."""
    rng = np.random.default_rng(31)
    specials = np.array([[np.nan, 0.5, 0.5], [np.inf, 0.5, 0.5], [-np.inf, 0, 0],
                         [0.5, np.inf, -np.inf], [1e3, -2e3, 5e2], [40.0, 0.5, 0.5]])
    cases = []
    # the reference test's background: a cube of six tetrahedra, size 0.2 + 0.5 x
    # (tests/test_sizing.cpp:85-108)
    P, T = W.kuhn_tet_mesh(1)
    S = 0.2 + 0.5 * P[:, 0]
    Q = np.vstack([P, [[0.5, 0.5, 0.5]], W.sizing_queries(P, T, 300, seed=1), specials])
    cases.append(("cube6", P, T, S, 1.0, Q))
    cases.append(("cube6_half", P, T, np.full(len(P), 0.4), 0.5, Q[:40]))
    P, T = W.kuhn_tet_mesh(3, 0.3, seed=4)
    S = rng.uniform(0.05, 0.5, len(P))
    cases.append(("kuhn3_jitter", P, T, S, 0.5, np.vstack([W.sizing_queries(P, T, 1500, seed=2), specials])))
    # two overlapping meshes (non-conforming): in the overlap the first index answers
    P1, T1 = W.kuhn_tet_mesh(2, 0.2, seed=5)
    P2, T2 = W.kuhn_tet_mesh(2, 0.2, seed=6, lo=(0.3, 0.2, 0.1))
    P = np.vstack([P1, P2])
    T = np.vstack([T2 + len(P1), T1])
    S = rng.uniform(0.1, 1.0, len(P))
    cases.append(("overlap", P, T, S, 1.0, W.sizing_queries(P, T, 1200, seed=3)))
    # slivers (four nearly coplanar nodes), a tiny tetrahedron and flat ones (D == 0)
    P, T = W.kuhn_tet_mesh(2, 0.0, seed=1)
    extra = np.array([[0.2, 0.2, 0.5], [0.8, 0.2, 0.5], [0.5, 0.8, 0.5], [0.5, 0.4, 0.5 + 1e-13],
                      [0.31, 0.47, 0.53], [0.31 + 1e-7, 0.47, 0.53], [0.31, 0.47 + 1e-7, 0.53],
                      [0.31, 0.47, 0.53 + 1e-7], [0.1, 0.1, 0.1], [0.9, 0.1, 0.1], [0.5, 0.9, 0.1]])
    b = len(P)
    P = np.vstack([P, extra])
    T = np.vstack([[[b, b + 1, b + 2, b + 3]], [[b + 4, b + 5, b + 6, b + 7]],
                   [[b + 8, b + 9, b + 10, b + 8]], [[b, b + 1, b + 2, b]], T])
    S = rng.uniform(0.1, 1.0, len(P))
    Q = np.vstack([W.sizing_queries(P, T, 800, seed=4), extra, (extra[:4].mean(0))[None],
                   extra[4:8].mean(0)[None] + 1e-9])
    cases.append(("slivers_flat", P, T, S, 1.0, Q))
    # short and long size arrays
    P, T = W.kuhn_tet_mesh(2, 0.1, seed=7)
    Q = W.sizing_queries(P, T, 400, seed=5)
    cases.append(("short_sizes", P, T, rng.uniform(0.1, 1.0, 10), 1.0, Q))
    cases.append(("long_sizes", P, T, rng.uniform(0.1, 1.0, len(P) + 7), 1.0, Q))
    # nearest-node ties: queries outside the mesh on its symmetry planes
    P, T = W.kuhn_tet_mesh(2)
    Q = np.array([[0.5, 0.5, 2.0], [0.25, 0.5, -1.0], [1.75, 0.5, 0.5], [0.5, -0.75, 0.25],
                  [-1.0, -1.0, -1.0], [0.75, 1.5, 0.75]])
    cases.append(("nearest_ties", P, T, np.arange(len(P), dtype=np.float64), 1.0, Q))
    cases.append(("empty", np.zeros((0, 3)), np.zeros((0, 4), np.int32), np.zeros(0), 1.0,
                  np.array([[0.2, 0.2, 0.0], [np.nan, 0, 0]])))
    return cases


def _o3_fast(a, b, c, d):
    adx, ady, adz = a - d
    bdx, bdy, bdz = b - d
    cdx, cdy, cdz = c - d
    return adz * (bdx * cdy - cdx * bdy) + bdz * (cdx * ady - adx * cdy) + cdz * (adx * bdy - bdx * ady)


def o3_value_queries():
    """(n, 4, 3) orient3d inputs whose rounded determinant is zero, reaching every stage
    of the adaptive routine (points exactly on the plane z = x after large offsets, some
    nudged by one ulp; nearly coplanar and collinear points), plus random ones."""
    rng = np.random.default_rng(77)
    out = []
    while len(out) < 3000:
        B = rng.normal(size=(4, 3))
        k = len(out) % 3
        if k == 0:
            B[:, 2] = B[:, 0]
            off = rng.choice([1e3, 1e6, 12345.678, 3e8, 1e12]) * rng.random()
            B[:, 0] += off
            B[:, 2] += off
            B[:, 1] += rng.choice([0.0, off])
            if rng.random() < 0.5:
                i, j = rng.integers(0, 4), rng.integers(0, 3)
                B[i, j] = np.nextafter(B[i, j], np.inf if rng.random() < 0.5 else -np.inf)
        elif k == 1:
            a_, b_ = rng.normal(size=2)
            B[:, 2] = a_ * B[:, 0] + b_ * B[:, 1]
            B += rng.choice([0.0, 1.0, 1e3, 0.1])
        else:
            B[3] = B[0] + rng.random() * (B[1] - B[0])
            B += rng.choice([0.0, 1.0, 1e6])
        if _o3_fast(*B) == 0.0:
            out.append(B)
    out += list(rng.normal(size=(500, 4, 3)))
    return np.ascontiguousarray(np.array(out))


def sizing_case(ref, manifest):
    out = {}
    names = []
    for name, P, T, S, scale, Q in sizing_cases():
        out[name + "_points"] = np.asarray(P, float).reshape(-1, 3)
        out[name + "_tets"] = np.asarray(T, np.int32).reshape(-1, 4)
        out[name + "_sizes"] = np.asarray(S, float)
        out[name + "_scale"] = np.array(scale)
        out[name + "_queries"] = np.asarray(Q, float).reshape(-1, 3)
        out[name + "_values"] = ref.sizing(P, T, S, scale, Q)
        names.append(name)
    out["names"] = np.array(names)
    Pq = o3_value_queries()
    out["o3_points"] = Pq
    out["o3_values"] = np.array([ref.pred("orient3d", *p) for p in Pq])
    save("sizing", **out)
    manifest["sizing"] = ("background sizing fields (the reference test's six-tetrahedron cube, a "
                          "jittered mesh, overlapping meshes, slivers, a tiny and flat tetrahedra, "
                          "short and long size arrays, nearest-node ties, far / NaN / infinite "
                          "queries, an empty mesh) with the reference's closure values")


def stl_case(ref, manifest):
    out = {}
    tmp = os.path.join(ROOT, "oracle", "_ref", "stl_fixture.stl")
    names = []
    for name, data in stl_cases():
        with open(tmp, "wb") as f:
            f.write(data)
        pts, tri, err = ref.stl_read(tmp)
        out[name + "_bytes"] = np.frombuffer(data, dtype=np.uint8)
        out[name + "_error"] = np.array(err)
        out[name + "_points"] = pts if pts is not None else np.zeros((0, 3))
        out[name + "_triangles"] = tri if tri is not None else np.zeros((0, 3), np.int32)
        names.append(name)
    os.remove(tmp)
    out["names"] = np.array(names)
    save("stl", **out)
    manifest["stl"] = ("STL images (binary and ASCII variants, signed zeros, repeated and degenerate "
                       "triangles, number forms, errors) read by the reference's read_stl")


def main():
    O.build(ref=True)
    ref = O.Reference()
    only = set(sys.argv[1:])
    path = os.path.join(HERE, "MANIFEST.json")
    manifest = json.load(open(path)) if only and os.path.exists(path) else {}

    def want(name):
        return not only or name in only

    pts, tris = W.jittered_icosphere(3, 0.02, seed=1)
    if want("icosphere_s3_r58p3"):
        api_case(ref, "icosphere_s3_r58p3", pts, tris, 58, 3, nsample=2048)
    manifest["icosphere_s3_r58p3"] = "icosphere subdivision 3, radial jitter 2% (seed 1); resolution 58, pad 3 (64^3)"

    pts, tris = W.subdivided_cube(4)
    if want("cube4_r16p1"):
        api_case(ref, "cube4_r16p1", pts, tris, 16, 1)
    manifest["cube4_r16p1"] = "reference test fixture subdivided_cube(4); resolution 16, pad 1 (exact 16^3 block)"

    # the same cube with a zero-area facet (three collinear dyadic points at z = 0.5)
    # inserted halfway through its triangle list: every column whose bucket holds it
    # grazes on all six nudges, and the reference keeps the last attempt's crossings
    # of the triangles before it (voxelize.cpp:158-165), which changes 720 cells
    k = len(pts)
    pts_d = np.vstack([pts, [[0.25, 0.25, 0.5], [0.5, 0.5, 0.5], [0.75, 0.75, 0.5]]])
    tris_d = np.insert(tris, len(tris) // 2, [k, k + 1, k + 2], axis=0)
    if want("cube4deg_r16p1"):
        api_case(ref, "cube4deg_r16p1", pts_d, tris_d, 16, 1)
    manifest["cube4deg_r16p1"] = ("subdivided_cube(4) with a zero-area facet (0.25,0.25,0.5)-(0.5,0.5,0.5)-"
                                  "(0.75,0.75,0.5) inserted at triangle 96; resolution 16, pad 1 "
                                  "(81 columns exhaust every nudge)")

    pts, tris = W.uv_sphere(1.0, 16, 16)
    if want("uvsphere16_r20p1"):
        api_case(ref, "uvsphere16_r20p1", pts, tris, 20, 1)
    manifest["uvsphere16_r20p1"] = "reference test fixture sphere_plc(1,16,16); resolution 20, pad 1"

    pts, tris = W.brick(3.0, 1.0, 2.0)
    if want("brick312_r20p1"):
        api_case(ref, "brick312_r20p1", pts, tris, 20, 1)
    manifest["brick312_r20p1"] = "box [0,3]x[0,1]x[0,2]; resolution 20, pad 1 (axis order)"

    pts, tris = W.sh_sphere(nlon=64, nlat=32, seed=3)
    if want("shsphere64_r30p1"):
        api_case(ref, "shsphere64_r30p1", pts, tris, 30, 1)
    manifest["shsphere64_r30p1"] = "SH star surface on a 64x32-band UV sphere (seed 3); resolution 30, pad 1"

    pts, tris = W.box_and_torus(64, 32)
    h = 2.0 ** -5
    if want("boxtorus64_facegrid"):
        grid_case(ref, "boxtorus64_facegrid", pts, tris, [-16.5 * h, -16.5 * h, -10.5 * h], h, (64, 64, 64))
    manifest["boxtorus64_facegrid"] = ("unit box + torus(R .35, r .12, 64x32) on an explicit 64^3 grid, h=2^-5, "
                                       "cell centres exactly on the box faces (forces grazes)")
    if want("boxtorus64_r62p1"):
        api_case(ref, "boxtorus64_r62p1", pts, tris, 62, 1, full_sdf=False)
    manifest["boxtorus64_r62p1"] = "same mesh through the API, resolution 62, pad 1"

    pts, tris = W.subdivided_cube(3)
    if want("cube3_facegrid"):
        grid_case(ref, "cube3_facegrid", pts, tris, [-4.5 / 12, -4.5 / 12, -4.5 / 12], 1.0 / 12, (20, 20, 20))
    manifest["cube3_facegrid"] = "subdivided_cube(3) on a 20^3 grid, h=1/12, centres on faces and shared edges"

    # full-size configurations: the headline SH surface (65,024 triangles) at 128 and
    # 256 cells on its long axis, and the 262,156-triangle box + torus on the exact-face
    # 256^3 grid and through the API
    pts, tris = W.sh_sphere(nlon=256, nlat=128, seed=3)
    if want("shsphere256"):
        full_case(ref, "shsphere256", pts, tris,
                  [("r126p1", ("api", 126, 1)), ("r254p1", ("api", 254, 1))])
    manifest["shsphere256"] = ("SH star surface on a 256x128-band UV sphere (seed 3, 65,024 triangles); "
                               "resolution 126 pad 1 (128^3) and resolution 254 pad 1 (231x247x256)")
    pts, tris = W.box_and_torus(512, 256)
    h = 2.0 ** -7
    if want("boxtorus512"):
        full_case(ref, "boxtorus512", pts, tris,
                  [("facegrid", ("grid", [-64.5 * h, -64.5 * h, -43.5 * h], h, (256, 256, 256))),
                   ("r254p1", ("api", 254, 1))])
    manifest["boxtorus512"] = ("unit box + torus(R .35, r .12, 512x256 quads; 262,156 triangles) on the "
                               "exact-face 256^3 grid (h=2^-7) and through the API at resolution 254, pad 1")

    if want("predicates"):
        pred_case(ref, "predicates", 4096, seed=21)
    if want("stl"):
        stl_case(ref, manifest)
    if want("detect"):
        detect_case(ref, manifest)
    if want("simplify"):
        simplify_case(ref, manifest)
    if want("sizing"):
        sizing_case(ref, manifest)
    manifest["predicates"] = "4096 orient3d + 4096 insphere queries (25% exact-degenerate, 25% near)"

    with open(path, "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
