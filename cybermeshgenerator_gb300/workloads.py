"""Seeded synthetic inputs for the voxelization path.

Every generator returns float64 points (N, 3) and int32 triangles (M, 3) (or a
list of polygon facets where the fan triangulation itself is under test). The
shapes follow the workloads the voxelizer is measured on:

* ``jittered_icosphere``  — closed icosphere, subdivision 3 (642 vertices, 1280
  triangles), each vertex radially scaled by U(-2%, +2%); voxelized at 64 cells on
  the longest axis (resolution 58, pad 3).
* ``box_and_torus``       — the unit box [0,1]^3 (12 triangles) and a torus
  R=0.35, r=0.12 centred at (0.5, 0.5, 1.2) with 512x256 quads (262,144
  triangles); ``box_torus_face_grid`` is the 256^3 grid whose cell centres land
  exactly on the box faces and edges.
* ``sh_sphere``           — star-shaped surface from a 256x128-band UV sphere
  (65,024 triangles) with radius 1 + a sum of 8 real spherical harmonics of
  degree <= 6 and N(0, 0.05^2) coefficients.
* ``mesh_batch``          — many closed meshes of uneven size (icospheres of
  subdivision 1-5, tori of 16-256 segments per ring) under random scale and
  rotation, each with its own resolution.
* ``ellipsoid_field``     — non-overlapping random ellipsoids (icosphere
  subdivision 3 each) packed in the unit cube.
* ``predicate_stream``    — orient3d / insphere queries in SoA layout, a given
  fraction of them exactly coplanar / cospherical (small-integer and dyadic
  coordinates, so the ties survive rounding).

Transcendental functions differ in the last bit between hosts, so fixtures that
must be bit-identical across machines are serialised (tests/golden) rather than
regenerated.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


# --------------------------------------------------------------------------- #
# basic closed surfaces
# --------------------------------------------------------------------------- #

def icosphere(subdiv: int):
    """Unit icosphere: 10*4^n + 2 vertices, 20*4^n triangles (outward winding)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
         (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts, dtype=np.float64), np.array(faces, dtype=np.int32)


def jittered_icosphere(subdiv: int = 3, jitter: float = 0.02, seed: int = 1):
    pts, tris = icosphere(subdiv)
    rng = np.random.default_rng(seed)
    s = 1.0 + rng.uniform(-jitter, jitter, size=len(pts))
    return pts * s[:, None], tris


def unit_box(side: float = 1.0):
    """Axis-aligned box [0,side]^3, six faces of two triangles each (12)."""
    s = float(side)
    pts = np.array([[0, 0, 0], [s, 0, 0], [s, s, 0], [0, s, 0],
                    [0, 0, s], [s, 0, s], [s, s, s], [0, s, s]], dtype=np.float64)
    tris = []
    for a, b, c, d in [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4),
                       (2, 3, 7, 6), (1, 2, 6, 5), (0, 4, 7, 3)]:
        tris += [(a, b, c), (a, c, d)]
    return pts, np.array(tris, dtype=np.int32)


def brick(X: float, Y: float, Z: float):
    """Box [0,X]x[0,Y]x[0,Z] as 12 triangles."""
    pts = np.array([[0, 0, 0], [X, 0, 0], [X, Y, 0], [0, Y, 0],
                    [0, 0, Z], [X, 0, Z], [X, Y, Z], [0, Y, Z]], dtype=np.float64)
    tris = []
    for a, b, c, d in [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4),
                       (2, 3, 7, 6), (1, 2, 6, 5), (0, 4, 7, 3)]:
        tris += [(a, b, c), (a, c, d)]
    return pts, np.array(tris, dtype=np.int32)


def torus(R: float, r: float, center=(0.0, 0.0, 0.0), nu: int = 64, nv: int = 32):
    """Torus around the z axis: nu segments around the ring, nv around the tube,
    each quad split into two triangles (2*nu*nv)."""
    u = 2.0 * np.pi * np.arange(nu) / nu
    v = 2.0 * np.pi * np.arange(nv) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    x = (R + r * np.cos(V)) * np.cos(U) + center[0]
    y = (R + r * np.cos(V)) * np.sin(U) + center[1]
    z = r * np.sin(V) + center[2]
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    t1 = np.stack([a, b, c], axis=-1).reshape(-1, 3)
    t2 = np.stack([a, c, d], axis=-1).reshape(-1, 3)
    tris = np.empty((2 * nu * nv, 3), dtype=np.int32)
    tris[0::2] = t1
    tris[1::2] = t2
    return pts.astype(np.float64), tris


def merge(*meshes):
    pts, tris, off = [], [], 0
    for p, t in meshes:
        pts.append(p)
        tris.append(t + off)
        off += len(p)
    return np.concatenate(pts).astype(np.float64), np.concatenate(tris).astype(np.int32)


def box_and_torus(nu: int = 512, nv: int = 256):
    """Unit box (12 triangles) plus a torus R=0.35, r=0.12 at (0.5, 0.5, 1.2)."""
    return merge(unit_box(1.0), torus(0.35, 0.12, (0.5, 0.5, 1.2), nu, nv))


def box_torus_face_grid(n: int = 256):
    """Explicit grid with h = 2^-7 whose cell centres land exactly on x, y, z in
    {0, 1}: corner (-64.5h, -64.5h, -43.5h), n^3 cells."""
    h = 2.0 ** -7
    return (np.array([-64.5 * h, -64.5 * h, -43.5 * h]), h, (n, n, n))


# --------------------------------------------------------------------------- #
# spherical-harmonic star-shaped surface
# --------------------------------------------------------------------------- #

def _assoc_legendre(l: int, m: int, x: np.ndarray) -> np.ndarray:
    """P_l^m(x) for m >= 0 (no Condon-Shortley phase), by the standard recurrence."""
    pmm = np.ones_like(x)
    if m > 0:
        somx2 = np.sqrt(np.maximum(0.0, (1.0 - x) * (1.0 + x)))
        fact = 1.0
        for _ in range(m):
            pmm = pmm * fact * somx2
            fact += 2.0
    if l == m:
        return pmm
    pmmp1 = x * (2 * m + 1) * pmm
    if l == m + 1:
        return pmmp1
    pll = pmmp1
    for ll in range(m + 2, l + 1):
        pll = (x * (2 * ll - 1) * pmmp1 - (ll + m - 1) * pmm) / (ll - m)
        pmm, pmmp1 = pmmp1, pll
    return pll


def real_sph_harm(l: int, m: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) /
                     math.factorial(l + am))
    p = _assoc_legendre(l, am, np.cos(theta))
    if m == 0:
        return norm * p
    if m > 0:
        return math.sqrt(2.0) * norm * p * np.cos(am * phi)
    return math.sqrt(2.0) * norm * p * np.sin(am * phi)


def sh_sphere(nlon: int = 256, nlat: int = 128, nharm: int = 8, lmax: int = 6,
              sigma: float = 0.05, seed: int = 3):
    """UV sphere of nlon x nlat bands (pole bands as triangle fans), radius
    1 + sum_i c_i Y_{l_i m_i}, c_i ~ N(0, sigma^2), distinct (l, m) with 1<=l<=lmax.
    nlon=256, nlat=128 gives 65,024 triangles."""
    rng = np.random.default_rng(seed)
    pairs = [(l, m) for l in range(1, lmax + 1) for m in range(-l, l + 1)]
    pick = rng.choice(len(pairs), size=nharm, replace=False)
    coef = rng.normal(0.0, sigma, size=nharm)
    theta = np.pi * np.arange(1, nlat) / nlat
    phi = 2.0 * np.pi * np.arange(nlon) / nlon
    TH, PH = np.meshgrid(theta, phi, indexing="ij")
    th_all = np.concatenate([[0.0], TH.ravel(), [np.pi]])
    ph_all = np.concatenate([[0.0], PH.ravel(), [0.0]])
    r = np.ones_like(th_all)
    for k, idx in enumerate(pick):
        l, m = pairs[idx]
        r = r + coef[k] * real_sph_harm(l, m, th_all, ph_all)
    pts = np.stack([r * np.sin(th_all) * np.cos(ph_all),
                    r * np.sin(th_all) * np.sin(ph_all),
                    r * np.cos(th_all)], axis=1)
    top, bot = 0, len(pts) - 1

    def vid(i, j):  # ring i in 1..nlat-1, column j
        return 1 + (i - 1) * nlon + (j % nlon)

    tris = []
    for j in range(nlon):
        tris.append((top, vid(1, j), vid(1, j + 1)))
    for i in range(1, nlat - 1):
        for j in range(nlon):
            a, b = vid(i, j), vid(i + 1, j)
            c, d = vid(i + 1, j + 1), vid(i, j + 1)
            tris.append((a, b, c))
            tris.append((a, c, d))
    for j in range(nlon):
        tris.append((vid(nlat - 1, j), bot, vid(nlat - 1, j + 1)))
    return pts.astype(np.float64), np.array(tris, dtype=np.int32)


# --------------------------------------------------------------------------- #
# fixtures of the reference's own test suite, restated
# --------------------------------------------------------------------------- #

def subdivided_cube(n: int):
    """Unit cube with each face an n x n grid of quads (two triangle facets each),
    shared vertices, as the reference's tests/test_voxelize.cpp:20-52 builds it."""
    vid = {}
    pts = []

    def vert(x, y, z):
        k = (x, y, z)
        if k not in vid:
            vid[k] = len(pts)
            pts.append((x / n, y / n, z / n))
        return vid[k]

    tris = []

    def quad(a, b, c, d):
        tris.append((a, b, c))
        tris.append((a, c, d))

    for i in range(n):
        for j in range(n):
            quad(vert(i, j, 0), vert(i + 1, j, 0), vert(i + 1, j + 1, 0), vert(i, j + 1, 0))
            quad(vert(i, j, n), vert(i, j + 1, n), vert(i + 1, j + 1, n), vert(i + 1, j, n))
            quad(vert(i, 0, j), vert(i, 0, j + 1), vert(i + 1, 0, j + 1), vert(i + 1, 0, j))
            quad(vert(i, n, j), vert(i + 1, n, j), vert(i + 1, n, j + 1), vert(i, n, j + 1))
            quad(vert(0, i, j), vert(0, i + 1, j), vert(0, i + 1, j + 1), vert(0, i, j + 1))
            quad(vert(n, i, j), vert(n, i, j + 1), vert(n, i + 1, j + 1), vert(n, i + 1, j))
    return np.array(pts, dtype=np.float64), np.array(tris, dtype=np.int32)


def uv_sphere(r: float, nlat: int, nlon: int):
    """Triangulated UV sphere as the reference's tests/test_voxelize.cpp:56-89."""
    pts = [(0.0, 0.0, r)]
    ids = {}
    for i in range(1, nlat):
        th = math.pi * i / nlat
        for j in range(nlon):
            ph = 2 * math.pi * j / nlon
            ids[(i, j)] = len(pts)
            pts.append((r * math.sin(th) * math.cos(ph), r * math.sin(th) * math.sin(ph),
                        r * math.cos(th)))
    bot = len(pts)
    pts.append((0.0, 0.0, -r))
    tris = []
    for j in range(nlon):
        tris.append((0, ids[(1, j)], ids[(1, (j + 1) % nlon)]))
    for i in range(1, nlat - 1):
        for j in range(nlon):
            j1 = (j + 1) % nlon
            tris.append((ids[(i, j)], ids[(i + 1, j)], ids[(i + 1, j1)]))
            tris.append((ids[(i, j)], ids[(i + 1, j1)], ids[(i, j1)]))
    for j in range(nlon):
        tris.append((ids[(nlat - 1, j)], bot, ids[(nlat - 1, (j + 1) % nlon)]))
    return np.array(pts, dtype=np.float64), np.array(tris, dtype=np.int32)


# --------------------------------------------------------------------------- #
# batches and scenes
# --------------------------------------------------------------------------- #

def _rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


@dataclass
class BatchItem:
    points: np.ndarray
    triangles: np.ndarray
    resolution: int
    pad: int = 1
    kind: str = ""


_ICO_CACHE: dict = {}


def mesh_batch(n: int = 512, seed: int = 4, resolutions=(32, 48, 64, 96, 128, 192),
               max_subdiv: int = 5, max_seg: int = 256):
    """n closed meshes: icosphere (subdivision 1..max_subdiv) or torus (R~U(.3,.45),
    r~U(.05,.15), 16..max_seg segments per ring), random scale 0.5-2 and rotation."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        if rng.random() < 0.5:
            s = int(rng.integers(1, max_subdiv + 1))
            if s not in _ICO_CACHE:
                _ICO_CACHE[s] = icosphere(s)
            p, t = _ICO_CACHE[s]
            kind = f"ico{s}"
        else:
            R = rng.uniform(0.3, 0.45)
            r = rng.uniform(0.05, 0.15)
            nu = int(rng.integers(16, max_seg + 1))
            nv = int(rng.integers(16, max_seg + 1))
            p, t = torus(R, r, (0, 0, 0), nu, nv)
            kind = f"torus{nu}x{nv}"
        A = _rotation(rng) * rng.uniform(0.5, 2.0)
        out.append(BatchItem(p @ A.T, t.copy(), int(rng.choice(resolutions)), 1, kind))
    return out


def ellipsoid_field(n: int = 2000, seed: int = 5, subdiv: int = 3,
                    amin: float = 0.01, amax: float = 0.04, max_tries: int = 2_000_000):
    """n non-overlapping ellipsoids (semi-axes U(amin, amax), random rotation) in the
    unit cube, rejection-sampled on bounding spheres; subdivision-3 icospheres give
    1280 triangles each."""
    rng = np.random.default_rng(seed)
    base_p, base_t = icosphere(subdiv)
    centers, radii, pts, tris = [], [], [], []
    tries = 0
    C = np.zeros((0, 3))
    Rr = np.zeros(0)
    while len(centers) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place all ellipsoids")
        ax = rng.uniform(amin, amax, size=3)
        rad = ax.max()
        c = rng.uniform(rad, 1.0 - rad, size=3)
        if len(C) and np.any(np.linalg.norm(C - c, axis=1) < Rr + rad):
            continue
        centers.append(c)
        radii.append(rad)
        C = np.asarray(centers)
        Rr = np.asarray(radii)
        M = _rotation(rng) * ax[None, :]
        pts.append(base_p @ M.T + c)
        tris.append(base_t + len(base_p) * (len(centers) - 1))
    return np.concatenate(pts), np.concatenate(tris).astype(np.int32)


# --------------------------------------------------------------------------- #
# predicate streams
# --------------------------------------------------------------------------- #

def _sphere_lattice_points(N: int) -> np.ndarray:
    r = int(math.isqrt(N))
    out = []
    for x in range(-r, r + 1):
        for y in range(-r, r + 1):
            z2 = N - x * x - y * y
            if z2 < 0:
                continue
            z = int(math.isqrt(z2))
            if z * z == z2:
                out.append((x, y, z))
                if z:
                    out.append((x, y, -z))
    return np.array(out, dtype=np.float64)


def predicate_stream(n: int, kind: str = "orient3d", degenerate: float = 0.1,
                     near: float = 0.1, seed: int = 6) -> np.ndarray:
    """SoA float64 array of shape (12, n) (orient3d: a b c d) or (15, n) (insphere:
    a b c d e). A `degenerate` fraction is exactly coplanar / cospherical (integer
    points scaled by a power of two), a `near` fraction is nearly so (the exact
    case perturbed by a few ulps; a zero coordinate becomes +-k*2^-60, never a
    subnormal, where products would underflow), the rest uniform in [0,1)^3."""
    rng = np.random.default_rng(seed)
    npt = 4 if kind == "orient3d" else 5
    P = rng.random((npt, 3, n))
    nd = int(round(degenerate * n))
    nn = int(round(near * n))
    idx = rng.permutation(n)
    deg = idx[:nd]
    nea = idx[nd:nd + nn]
    both = np.concatenate([deg, nea])
    m = len(both)
    if m:
        scale = 2.0 ** -rng.integers(3, 12, size=m)
        if kind == "orient3d":
            a = rng.integers(-64, 65, size=(3, m)).astype(np.float64)
            b = rng.integers(-64, 65, size=(3, m)).astype(np.float64)
            c = rng.integers(-64, 65, size=(3, m)).astype(np.float64)
            s = rng.integers(-4, 5, size=m).astype(np.float64)
            t = rng.integers(-4, 5, size=m).astype(np.float64)
            d = a + s * (b - a) + t * (c - a)
            pts = [a, b, c, d]
        else:
            lat = _sphere_lattice_points(27625)  # 1152 integer points on the sphere
            sel = rng.integers(0, len(lat), size=(m, 5))
            while True:  # five distinct points per query: redraw rows with a repeat
                srt = np.sort(sel, axis=1)
                dup = (srt[:, 1:] == srt[:, :-1]).any(axis=1)
                if not dup.any():
                    break
                sel[dup] = rng.integers(0, len(lat), size=(int(dup.sum()), 5))
            off = rng.integers(-32, 33, size=(3, m)).astype(np.float64)
            pts = [lat[sel[:, i]].T + off for i in range(5)]
        perm = rng.permutation(npt)
        for i in range(npt):
            P[i][:, both] = pts[perm[i]] * scale
        if nn:
            # nudge one coordinate of the near cases by a few ulps
            k = rng.integers(0, npt, size=nn)
            ax = rng.integers(0, 3, size=nn)
            ulps = rng.integers(1, 4, size=nn) * rng.choice([-1, 1], size=nn)
            v = P[k, ax, nea]
            zero = v == 0.0
            toward = np.where(ulps > 0, np.inf, -np.inf)
            for step in range(1, 4):
                sel_ = ~zero & (np.abs(ulps) >= step)
                v[sel_] = np.nextafter(v[sel_], toward[sel_])
            # a zero coordinate becomes +-k*2^-60, clear of subnormals (no expansion
            # arithmetic there)
            v[zero] = ulps[zero].astype(np.float64) * 2.0 ** -60
            P[k, ax, nea] = v
    return np.ascontiguousarray(P.reshape(npt * 3, n))


# --------------------------------------------------------------------------- #
# STL images
# --------------------------------------------------------------------------- #

def stl_binary(points, triangles, header: bytes = b"cybermeshgenerator stl") -> bytes:
    """Binary STL image: 80-byte header, u32 count, 50-byte records (zero normal,
    three float32 vertices, zero attribute)."""
    p = np.asarray(points, dtype=np.float32)
    t = np.asarray(triangles, dtype=np.int64)
    rec = np.zeros(len(t), dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]))
    rec["v"] = p[t]
    return header[:80].ljust(80, b"\0") + np.uint32(len(t)).tobytes() + rec.tobytes()


def stl_ascii(points, triangles, fmt: str = "{:.9g}", crlf: bool = False,
              comments: bool = False, commas: bool = False, upper: bool = False) -> bytes:
    """ASCII STL image in the reference writer's layout, with optional variations
    its reader accepts (comments, CRLF line ends, comma separators, upper case)."""
    p = np.asarray(points, dtype=np.float64)
    nl = "\r\n" if crlf else "\n"
    sep = ", " if commas else " "
    kw = "VERTEX" if upper else "vertex"
    out = ["solid cmg"]
    for i, t in enumerate(np.asarray(triangles)):
        out.append("  facet normal 0 0 0" + (f"  # facet {i}" if comments else ""))
        out.append("    outer loop")
        for k in t:
            out.append("      " + kw + " " + sep.join(fmt.format(float(c)) for c in p[k]))
        out.append("    endloop")
        out.append("  endfacet")
        if comments and i % 7 == 0:
            out.append("# a comment line")
            out.append("   ")
    out.append("endsolid cmg")
    return (nl.join(out) + nl).encode()


def kuhn_tet_mesh(n: int = 8, jitter: float = 0.0, seed: int = 1, lo=(0.0, 0.0, 0.0),
                  side: float = 1.0):
    """A conforming background tetrahedral mesh of the cube [lo, lo + side]^3: an n^3 grid
    of cells, each split into the six Kuhn tetrahedra around its main diagonal (node
    (i,j,k) -> (i+1,j+1,k+1) through one axis step at a time), interior nodes moved by up
    to `jitter` cell sizes. Returns (points (N, 3) float64, tets (6 n^3, 4) int32)."""
    rng = np.random.default_rng(seed)
    g = np.arange(n + 1, dtype=np.float64) / n
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    if jitter > 0:
        inner = np.all((pts > 0) & (pts < 1), axis=1)
        pts[inner] += rng.uniform(-jitter, jitter, size=(int(inner.sum()), 3)) / n
    pts = np.asarray(lo, dtype=np.float64) + side * pts
    I, J, K = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1)          # cells in (i, j, k) order
    step = np.eye(3, dtype=np.int64)
    nid = lambda v: (v[:, 0] * (n + 1) + v[:, 1]) * (n + 1) + v[:, 2]
    tets = np.empty((len(base), 6, 4), dtype=np.int32)
    for p, perm in enumerate(((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))):
        a = base
        b = a + step[perm[0]]
        c = b + step[perm[1]]
        d = c + step[perm[2]]
        tets[:, p] = np.stack([nid(a), nid(b), nid(c), nid(d)], axis=1)
    return pts, tets.reshape(-1, 4)


def sizing_queries(points, tets, n: int, seed: int = 2, outside: float = 0.1):
    """Queries for a background sizing field: uniform points over the mesh's box grown by
    `outside` of its extent on every side (some fall outside the mesh and take the
    nearest node's size), plus exact nodes, edge midpoints and face centroids (points
    on shared faces, where the first tetrahedron in order must win)."""
    rng = np.random.default_rng(seed)
    lo, hi = points.min(0), points.max(0)
    ext = (hi - lo).max()
    m = n // 2
    q = [rng.uniform(lo - outside * ext, hi + outside * ext, size=(m, 3))]
    k = (n - m) // 3
    q.append(points[rng.integers(0, len(points), size=k)])
    t = tets[rng.integers(0, len(tets), size=k)]
    q.append(0.5 * (points[t[:, 0]] + points[t[:, 1]]))
    t = tets[rng.integers(0, len(tets), size=n - m - 2 * k)]
    q.append((points[t[:, 0]] + points[t[:, 1]] + points[t[:, 2]]) / 3.0)
    return np.ascontiguousarray(np.vstack(q))
