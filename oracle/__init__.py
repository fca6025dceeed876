"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

`load()` opens oracle/liboracle.so, the C restatement of the reference's
voxelization path; `load_ref()` opens oracle/_ref/libcmgref.so, the reference's
own code compiled from its sources (present only where the reference sources
were available at build time). Only the test suite, the smoke check and the
CPU-baseline leg of bench.py use this module; the product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_REF = os.path.join(_HERE, "_ref", "libcmgref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_fp = ctypes.POINTER(ctypes.c_float)
_i8p = ctypes.POINTER(ctypes.c_int8)

COMPAT, EXACT = 0, 1


class Grid(ctypes.Structure):
    _fields_ = [("corner", ctypes.c_double * 3), ("spacing", ctypes.c_double),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int)]

    @property
    def dims(self):
        return (self.nx, self.ny, self.nz)

    @property
    def ncell(self):
        return self.nx * self.ny * self.nz

    def as_tuple(self):
        return (tuple(self.corner), self.spacing, self.dims)


class OccStats(ctypes.Structure):
    _fields_ = [("columns", ctypes.c_int64), ("nudged_columns", ctypes.c_int64),
                ("exhausted_columns", ctypes.c_int64), ("exact_calls", ctypes.c_int64),
                ("orient_calls", ctypes.c_int64), ("crossings", ctypes.c_int64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference harness when `ref`)."""
    r = subprocess.run(["make", "-C", _HERE, "liboracle.so"], capture_output=True, text=True)
    if r.returncode != 0:  # a host without OpenMP: build single-threaded
        r = subprocess.run(["make", "-C", _HERE, "liboracle.so", "OMP="],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    if ref:
        root = os.environ.get("CMG_REFERENCE_ROOT")
        if not root:
            raise RuntimeError("the reference harness needs CMG_REFERENCE_ROOT (the reference source tree)")
        r = subprocess.run(["make", "-C", _HERE, "ref", "REF_ROOT=" + root], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference harness build failed:\n" + r.stdout + r.stderr)


def _ptr(a, t):
    return a.ctypes.data_as(t)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Oracle:
    """The C restatement."""

    def __init__(self, path: str = _LIB):
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        self.L = L
        L.orc_orient3d_fast.restype = ctypes.c_double
        L.orc_insphere_fast.restype = ctypes.c_double
        L.orc_point_tri_dist2.restype = ctypes.c_double
        L.orc_make_grid.restype = ctypes.c_int
        L.orc_fan_triangles.restype = ctypes.c_int64
        L.orc_fan_triangles.argtypes = [_ip, _i64p, ctypes.c_int64, _ip]
        for f in ("orc_orient3d_stream", "orc_insphere_stream"):
            getattr(L, f).argtypes = [ctypes.POINTER(_dp), ctypes.c_int64, ctypes.c_int,
                                      _i8p, ctypes.c_int]

    @staticmethod
    def threads(n=None):
        return int(n or os.cpu_count() or 1)

    # ---- grid ----
    def make_grid(self, pts, resolution, pad) -> Grid:
        pts = _f64(pts)
        g = Grid()
        rc = self.L.orc_make_grid(_ptr(pts, _dp), ctypes.c_int64(len(pts)),
                                  ctypes.c_int(resolution), ctypes.c_int(pad),
                                  ctypes.byref(g))
        if rc != 0:
            raise ValueError("zero-extent point set")
        return g

    @staticmethod
    def grid(corner, spacing, dims) -> Grid:
        g = Grid()
        for a in range(3):
            g.corner[a] = float(corner[a])
        g.spacing = float(spacing)
        g.nx, g.ny, g.nz = (int(d) for d in dims)
        return g

    def fan(self, facets):
        idx = _i32(np.concatenate([np.asarray(f, dtype=np.int32) for f in facets]))
        off = np.zeros(len(facets) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(f) for f in facets])
        n = self.L.orc_fan_triangles(_ptr(idx, _ip), _ptr(off, _i64p),
                                     ctypes.c_int64(len(facets)), None)
        out = np.zeros((n, 3), dtype=np.int32)
        self.L.orc_fan_triangles(_ptr(idx, _ip), _ptr(off, _i64p),
                                 ctypes.c_int64(len(facets)), _ptr(out, _ip))
        return out

    # ---- occupancy ----
    def occupancy(self, pts, tris, g: Grid, mode=COMPAT, threads=None):
        pts, tris = _f64(pts), _i32(tris)
        occ = np.zeros(g.ncell, dtype=np.uint8)
        st = OccStats()
        self.L.orc_occupancy(_ptr(pts, _dp), _ptr(tris, _ip), ctypes.c_int64(len(tris)),
                             ctypes.byref(g), ctypes.c_int(mode), _ptr(occ, _u8p),
                             ctypes.byref(st), ctypes.c_int(self.threads(threads)))
        return occ, st.as_dict()

    # ---- distance ----
    def sdf_ring(self, pts, tris, g: Grid, occ, threads=None):
        """Reference ring-search SDF: (signed float64, float32) over every cell."""
        pts, tris = _f64(pts), _i32(tris)
        occ = np.ascontiguousarray(occ, dtype=np.uint8)
        s64 = np.zeros(g.ncell, dtype=np.float64)
        s32 = np.zeros(g.ncell, dtype=np.float32)
        self.L.orc_sdf_ring(_ptr(pts, _dp), _ptr(tris, _ip), ctypes.c_int64(len(tris)),
                            ctypes.byref(g), _ptr(occ, _u8p), _ptr(s64, _dp),
                            _ptr(s32, _fp), ctypes.c_int(self.threads(threads)))
        return s64, s32

    def sdf_ring_sample(self, pts, tris, g: Grid, vox, threads=None, times=False):
        """Ring-search squared distances at the listed voxels; with times=True also
        (bucket build seconds, query seconds)."""
        pts, tris = _f64(pts), _i32(tris)
        vox = np.ascontiguousarray(vox, dtype=np.int64)
        d2 = np.zeros(len(vox), dtype=np.float64)
        tm = np.zeros(2, dtype=np.float64)
        self.L.orc_sdf_ring_sample(_ptr(pts, _dp), _ptr(tris, _ip),
                                   ctypes.c_int64(len(tris)), ctypes.byref(g),
                                   _ptr(vox, _i64p), ctypes.c_int64(len(vox)),
                                   _ptr(d2, _dp), ctypes.c_int(self.threads(threads)),
                                   _ptr(tm, _dp))
        return (d2, (float(tm[0]), float(tm[1]))) if times else d2

    def sdf_brute(self, pts, tris, g: Grid, vox=None, threads=None):
        """Brute-force nearest (d2, triangle, region) at the listed voxels (all if None)."""
        pts, tris = _f64(pts), _i32(tris)
        n = g.ncell if vox is None else len(vox)
        vp = None
        if vox is not None:
            vox = np.ascontiguousarray(vox, dtype=np.int64)
            vp = _ptr(vox, _i64p)
        d2 = np.zeros(n, dtype=np.float64)
        tri = np.zeros(n, dtype=np.int32)
        reg = np.zeros(n, dtype=np.int32)
        self.L.orc_sdf_brute(_ptr(pts, _dp), _ptr(tris, _ip), ctypes.c_int64(len(tris)),
                             ctypes.byref(g), vp, ctypes.c_int64(n), _ptr(d2, _dp),
                             _ptr(tri, _ip), _ptr(reg, _ip),
                             ctypes.c_int(self.threads(threads)))
        return d2, tri, reg

    def dist2_points(self, pts, tris, q, threads=None):
        pts, tris, q = _f64(pts), _i32(tris), _f64(q)
        d2 = np.zeros(len(q), dtype=np.float64)
        tri = np.zeros(len(q), dtype=np.int32)
        self.L.orc_dist2_points(_ptr(pts, _dp), _ptr(tris, _ip), ctypes.c_int64(len(tris)),
                                _ptr(q, _dp), ctypes.c_int64(len(q)), _ptr(d2, _dp),
                                _ptr(tri, _ip), ctypes.c_int(self.threads(threads)))
        return d2, tri

    def point_tri_dist2(self, p, a, b, c):
        p, a, b, c = (_f64(x) for x in (p, a, b, c))
        r = ctypes.c_int()
        d = self.L.orc_point_tri_dist2(_ptr(p, _dp), _ptr(a, _dp), _ptr(b, _dp),
                                       _ptr(c, _dp), ctypes.byref(r))
        return d, r.value

    def sdf_grad(self, pts, tris, g: Grid, occ, tri, w, t):
        pts, tris = _f64(pts), _i32(tris)
        occ = np.ascontiguousarray(occ, dtype=np.uint8)
        tri = _i32(tri)
        w, t = _f64(w), _f64(t)
        grad = np.zeros((len(pts), 3), dtype=np.float64)
        self.L.orc_sdf_grad(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(tris, _ip),
                            ctypes.byref(g), _ptr(occ, _u8p), _ptr(tri, _ip),
                            _ptr(w, _dp), _ptr(t, _dp), _ptr(grad, _dp))
        return grad

    # ---- predicates ----
    def orient3d_fast(self, a, b, c, d):
        a, b, c, d = (_f64(x) for x in (a, b, c, d))
        return self.L.orc_orient3d_fast(*(_ptr(x, _dp) for x in (a, b, c, d)))

    def stl_read(self, data: bytes):
        """The reference STL reader restated on an in-memory image: (points, triangles,
        error) with error "" on success."""
        if not getattr(self, "_stl_bound", False):
            _stl_bind(self.L, "orc_stl", [ctypes.c_char_p, ctypes.c_size_t])
            self._stl_bound = True
        return _stl_unpack(self.L, "orc_stl", self.L.orc_stl_read(data, len(data)))

    def self_intersections(self, pts, tris):
        """(i, j) pairs, i < j, of crossing triangles (reference order), int64 (k, 2)."""
        pts, tris = _f64(pts), _i32(tris)
        self.L.orc_self_intersections.restype = ctypes.c_int64
        n = self.L.orc_self_intersections(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(tris, _ip),
                                          ctypes.c_int64(len(tris)), None, ctypes.c_int64(0))
        out = np.zeros((max(n, 1), 2), dtype=np.int64)
        self.L.orc_self_intersections(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(tris, _ip),
                                      ctypes.c_int64(len(tris)), _ptr(out, _i64p), ctypes.c_int64(n))
        return out[:n]

    def simplify(self, pts, tris, grid):
        """Grid vertex clustering restated: (points (r,3), triangles (m,3) int32, error)
        with error "" on success (points and triangles None on error)."""
        pts = _f64(pts).reshape(-1, 3)
        tris = _i32(tris).reshape(-1, 3)
        f = self.L.orc_simplify
        f.restype = ctypes.c_int64
        op = np.zeros((max(len(pts), 1), 3))
        ot = np.zeros((max(len(tris), 1), 3), dtype=np.int32)
        m = ctypes.c_int64()
        err = ctypes.create_string_buffer(256)
        r = f(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(tris, _ip), ctypes.c_int64(len(tris)),
              ctypes.c_int(int(grid)), _ptr(op, _dp), _ptr(ot, _ip), ctypes.byref(m), err,
              ctypes.c_size_t(256))
        if r < 0:
            return None, None, err.value.decode()
        return op[:r].copy(), ot[:m.value].copy(), ""

    def orient3d_values(self, soa):
        """robust::orient3d values of n queries; soa is a (12, n) float64 array."""
        soa = _f64(soa)
        n = soa.shape[1]
        rows = (_dp * 12)(*[_ptr(soa[i], _dp) for i in range(12)])
        out = np.zeros(n)
        self.L.orc_orient3d_values(rows, ctypes.c_int64(n), _ptr(out, _dp))
        return out

    def sizing(self, points, tets, sizes, scale, queries, threads=None):
        """The background sizing field at the queries: (sizes (n,), answering tetrahedron
        or -1 per query (n,) int64). Node sizes are padded with 0 or truncated to the
        node count, as the reference does."""
        P = _f64(points).reshape(-1, 3)
        T = _i32(tets).reshape(-1, 4)
        S = np.zeros(len(P))
        sz = np.asarray(sizes, dtype=np.float64).ravel()[: len(P)]
        S[: len(sz)] = sz
        Q = _f64(queries).reshape(-1, 3)
        out = np.zeros(len(Q))
        which = np.zeros(len(Q), dtype=np.int64)
        self.L.orc_sizing_eval(_ptr(P, _dp), ctypes.c_int64(len(P)), _ptr(T, _ip), ctypes.c_int64(len(T)),
                               _ptr(S, _dp), ctypes.c_double(scale), _ptr(Q, _dp), ctypes.c_int64(len(Q)),
                               _ptr(out, _dp), _ptr(which, _i64p), ctypes.c_int(self.threads(threads)))
        return out, which

    def stream(self, kind, soa, mode=COMPAT, threads=None):
        """Signs of n queries; soa is a (12|15, n) float64 array."""
        soa = _f64(soa)
        n = soa.shape[1]
        rows = (_dp * soa.shape[0])(*[_ptr(soa[i], _dp) for i in range(soa.shape[0])])
        out = np.zeros(n, dtype=np.int8)
        fn = self.L.orc_orient3d_stream if kind == "orient3d" else self.L.orc_insphere_stream
        fn(rows, ctypes.c_int64(n), ctypes.c_int(mode), _ptr(out, _i8p),
           ctypes.c_int(self.threads(threads)))
        return out



def _stl_unpack(L, prefix, h):
    """(points (n,3) float64, triangles (m,3) int32, error str) from a reader handle."""
    try:
        err = getattr(L, prefix + "_error")(h).decode()
        if err:
            return None, None, err
        n = int(getattr(L, prefix + "_num_points")(h))
        m = int(getattr(L, prefix + "_num_triangles")(h))
        pts = np.ctypeslib.as_array(getattr(L, prefix + "_points")(h), (n * 3,)).reshape(n, 3).copy() \
            if n else np.zeros((0, 3))
        tri = np.ctypeslib.as_array(getattr(L, prefix + "_triangles")(h), (m * 3,)).reshape(m, 3).copy() \
            if m else np.zeros((0, 3), np.int32)
        return pts, tri.astype(np.int32), ""
    finally:
        getattr(L, prefix + "_free")(h)


def _stl_bind(L, prefix, arg):
    getattr(L, prefix + "_read").restype = ctypes.c_void_p
    getattr(L, prefix + "_read").argtypes = arg
    getattr(L, prefix + "_error").restype = ctypes.c_char_p
    for f, r in (("_num_points", ctypes.c_int64), ("_num_triangles", ctypes.c_int64),
                 ("_points", _dp), ("_triangles", _ip)):
        getattr(L, prefix + f).restype = r
        getattr(L, prefix + f).argtypes = [ctypes.c_void_p]
    getattr(L, prefix + "_error").argtypes = [ctypes.c_void_p]
    getattr(L, prefix + "_free").argtypes = [ctypes.c_void_p]


class Reference:
    """The reference's own code (built from its sources into oracle/_ref)."""

    def __init__(self, path: str = _REF):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        self.L = L
        for f in ("ref_orient3d", "ref_insphere", "ref_orient3dexact", "ref_insphereexact"):
            getattr(L, f).restype = ctypes.c_double

    @staticmethod
    def available() -> bool:
        return os.path.exists(_REF)

    def make_grid(self, pts, resolution, pad):
        pts = _f64(pts)
        corner = np.zeros(3)
        sp = ctypes.c_double()
        dims = np.zeros(3, dtype=np.int32)
        rc = self.L.ref_make_grid(_ptr(pts, _dp), ctypes.c_int64(len(pts)),
                                  ctypes.c_int(resolution), ctypes.c_int(pad),
                                  _ptr(corner, _dp), ctypes.byref(sp), _ptr(dims, _ip))
        return rc, corner, sp.value, tuple(int(d) for d in dims)

    def voxelize(self, pts, facets, resolution, pad, mode):
        """Public cmg::voxelize::voxelize. Returns (status, origin, spacing, dims, data)."""
        pts = _f64(pts)
        idx = _i32(np.concatenate([np.asarray(f, dtype=np.int32) for f in facets])
                   if len(facets) else np.zeros(0, np.int32))
        off = np.zeros(len(facets) + 1, dtype=np.int64)
        if len(facets):
            off[1:] = np.cumsum([len(f) for f in facets])
        origin = np.zeros(3)
        sp = ctypes.c_double()
        dims = np.zeros(3, dtype=np.int32)
        cap = 0
        rc, _, _, d = self.make_grid(pts, max(resolution, 1), pad) if len(pts) else (-1, 0, 0, (0, 0, 0))
        if rc == 0:
            cap = max(d[0] * d[1] * d[2], 0)
        out = np.zeros(max(cap, 1), dtype=np.float32 if mode == 1 else np.uint8)
        st = self.L.ref_voxelize(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(idx, _ip),
                                 _ptr(off, _i64p), ctypes.c_int64(len(facets)),
                                 ctypes.c_int(resolution), ctypes.c_int(pad),
                                 ctypes.c_int(mode), _ptr(origin, _dp), ctypes.byref(sp),
                                 _ptr(dims, _ip), out.ctypes.data_as(ctypes.c_void_p),
                                 ctypes.c_int64(cap))
        dims_t = tuple(int(x) for x in dims)
        return st, origin, sp.value, dims_t, out[:cap] if st == 0 else None

    def occupancy_grid(self, pts, tris, corner, spacing, dims):
        pts, tris = _f64(pts), _i32(tris)
        corner = _f64(corner)
        d = np.asarray(dims, dtype=np.int32)
        occ = np.zeros(int(np.prod(dims)), dtype=np.uint8)
        self.L.ref_occupancy_grid(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(tris, _ip),
                                  ctypes.c_int64(len(tris)), _ptr(corner, _dp),
                                  ctypes.c_double(spacing), _ptr(d, _ip), _ptr(occ, _u8p))
        return occ

    def fill_distance(self, pts, tris, corner, spacing, dims, occ):
        pts, tris = _f64(pts), _i32(tris)
        corner = _f64(corner)
        d = np.asarray(dims, dtype=np.int32)
        occ = np.ascontiguousarray(occ, dtype=np.uint8)
        out = np.zeros(int(np.prod(dims)), dtype=np.float32)
        self.L.ref_fill_distance(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(tris, _ip),
                                 ctypes.c_int64(len(tris)), _ptr(corner, _dp),
                                 ctypes.c_double(spacing), _ptr(d, _ip), _ptr(occ, _u8p),
                                 _ptr(out, _fp))
        return out

    def dist2_brute(self, pts, tris, corner, spacing, dims, vox):
        pts, tris = _f64(pts), _i32(tris)
        corner = _f64(corner)
        d = np.asarray(dims, dtype=np.int32)
        vox = np.ascontiguousarray(vox, dtype=np.int64)
        out = np.zeros(len(vox), dtype=np.float64)
        self.L.ref_dist2_brute(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(tris, _ip),
                               ctypes.c_int64(len(tris)), _ptr(corner, _dp),
                               ctypes.c_double(spacing), _ptr(d, _ip), _ptr(vox, _i64p),
                               ctypes.c_int64(len(vox)), _ptr(out, _dp))
        return out

    def ring_sample(self, pts, tris, corner, spacing, dims, vox):
        pts, tris = _f64(pts), _i32(tris)
        corner = _f64(corner)
        d = np.asarray(dims, dtype=np.int32)
        vox = np.ascontiguousarray(vox, dtype=np.int64)
        out = np.zeros(len(vox), dtype=np.float64)
        self.L.ref_ring_sample(_ptr(pts, _dp), ctypes.c_int64(len(pts)), _ptr(tris, _ip),
                               ctypes.c_int64(len(tris)), _ptr(corner, _dp),
                               ctypes.c_double(spacing), _ptr(d, _ip), _ptr(vox, _i64p),
                               ctypes.c_int64(len(vox)), _ptr(out, _dp))
        return out

    def stl_read(self, path: str):
        """The reference's read_stl on a file: (points, triangles, error)."""
        if not getattr(self, "_stl_bound", False):
            _stl_bind(self.L, "ref_stl", [ctypes.c_char_p])
            self._stl_bound = True
        return _stl_unpack(self.L, "ref_stl", self.L.ref_stl_read(path.encode()))

    def self_intersections(self, pts, tris):
        """The reference's self_intersections on a PLC of one triangle per facet:
        (k, 8) int32 rows (facet_a, facet_b, tri_a[3], tri_b[3]) in its order."""
        pts, tris = _f64(pts), _i32(tris)
        f = self.L.ref_self_intersections
        f.restype = ctypes.c_longlong
        n = f(_ptr(pts, _dp), ctypes.c_longlong(len(pts)), _ptr(tris, _ip), ctypes.c_longlong(len(tris)),
              None, ctypes.c_longlong(0))
        out = np.zeros((max(n, 1), 8), dtype=np.int32)
        f(_ptr(pts, _dp), ctypes.c_longlong(len(pts)), _ptr(tris, _ip), ctypes.c_longlong(len(tris)),
          _ptr(out, _ip), ctypes.c_longlong(n))
        return out[:n]

    def simplify(self, pts, tris, grid):
        """The reference's simplify on a PLC of one triangle per facet: (points,
        triangles, error) as Oracle.simplify."""
        pts = _f64(pts).reshape(-1, 3)
        tris = _i32(tris).reshape(-1, 3)
        f = self.L.ref_simplify
        f.restype = ctypes.c_longlong
        op = np.zeros((max(len(pts), 1), 3))
        ot = np.zeros((max(len(tris), 1), 3), dtype=np.int32)
        m = ctypes.c_longlong()
        err = ctypes.create_string_buffer(256)
        r = f(_ptr(pts, _dp), ctypes.c_longlong(len(pts)), _ptr(tris, _ip), ctypes.c_longlong(len(tris)),
              ctypes.c_int(int(grid)), _ptr(op, _dp), ctypes.c_longlong(len(op)), _ptr(ot, _ip),
              ctypes.c_longlong(len(ot)), ctypes.byref(m), err, ctypes.c_longlong(256))
        if r < 0:
            return None, None, err.value.decode()
        return op[:r].copy(), ot[:m.value].copy(), ""

    def sizing(self, points, tets, sizes, scale, queries):
        """The reference's from_background closure evaluated at each query (sizes as
        given: the reference pads or truncates them itself)."""
        P = _f64(points).reshape(-1, 3)
        T = _i32(tets).reshape(-1, 4)
        S = _f64(np.asarray(sizes, dtype=np.float64).ravel())
        Q = _f64(queries).reshape(-1, 3)
        out = np.zeros(len(Q))
        self.L.ref_sizing_eval(_ptr(P, _dp), ctypes.c_longlong(len(P)), _ptr(T, _ip),
                               ctypes.c_longlong(len(T)), _ptr(S, _dp), ctypes.c_longlong(len(S)),
                               ctypes.c_double(scale), _ptr(Q, _dp), ctypes.c_longlong(len(Q)),
                               _ptr(out, _dp))
        return out

    def pred(self, name, *pts):
        args = [_f64(p) for p in pts]
        return getattr(self.L, "ref_" + name)(*(_ptr(a, _dp) for a in args))
