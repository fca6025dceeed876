"""cybermeshgenerator_gb300 — GB300-native voxelization for CyberMeshGenerator.

The module mirrors the reference binding's surface
(bindings/python/src/cybermesh/__init__.py): ``PLC``, ``voxelize(plc,
resolution, mode, pad) -> VoxelGrid`` with the same argument meaning, array
layout ((nx, ny, nz), C-order per axis after the reference's transpose) and
error behaviour (``RuntimeError`` carrying the C error text, ``ValueError`` /
``TypeError`` for bad Python arguments). Underneath, libcmg_c.so runs the
occupancy and signed-distance kernels on the GPU.

Additions beyond the reference: ``voxelize_ex`` (explicit grid, FP64 and mixed
precision distance fields, exact predicates, nearest-feature checkpoints, run
statistics), ``Batch`` (many meshes in one pipeline, optionally replayed as a
CUDA graph) and, in ``cybermeshgenerator_gb300.torch_sdf``, a differentiable
signed distance field.

    import numpy as np, cybermeshgenerator_gb300 as cm
    plc = cm.PLC().add_points(points)
    for tri in triangles:
        plc.add_facet(tri)
    vg = cm.voxelize(plc, resolution=64, mode="sdf")
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, Optional, Sequence

import numpy as np

from . import _lib as _L

_clib = _L.Lazy()

OUT_OCCUPANCY, OUT_SDF_F32, OUT_SDF_F64, OUT_NEAREST, OUT_ERROR_BOUND = 1, 2, 4, 8, 16
PREC_FP64, PREC_MIXED, PREC_FP64_PLAIN = 0, 1, 2
PRED_COMPAT, PRED_EXACT = 0, 1


def _check(status: int, err) -> None:
    if status != 0:
        raise RuntimeError(err.value.decode() or f"cmg error {status}")


class PLC:
    """A piecewise-linear complex: points and polygon facets (the voxelizer reads
    the facets' fan triangulation)."""

    def __init__(self, _handle: Optional[int] = None) -> None:
        self._handle = _handle if _handle is not None else _clib.cmg_plc_create()
        if not self._handle:
            raise MemoryError("cmg_plc_create failed")

    @property
    def num_points(self) -> int:
        return int(_clib.cmg_plc_num_points(self._handle))

    @property
    def points(self) -> np.ndarray:
        n = self.num_points
        if not n:
            return np.empty((0, 3), dtype=np.float64)
        return np.ctypeslib.as_array(_clib.cmg_plc_points(self._handle), (n, 3)).astype(np.float64).copy()

    @property
    def triangles(self) -> np.ndarray:
        m = int(_clib.cmg_plc_num_triangles(self._handle))
        if not m:
            return np.empty((0, 3), dtype=np.int32)
        return np.ctypeslib.as_array(_clib.cmg_plc_triangles(self._handle), (m, 3)).astype(np.int32).copy()

    def add_points(self, points) -> "PLC":
        """Set the vertex cloud from an (N, 3) array (replaces any previous set)."""
        pts = np.ascontiguousarray(points, dtype=np.float64)
        if pts.ndim != 2 or pts.shape[1] != 3:
            raise ValueError("points must be an (N, 3) array")
        _check(_clib.cmg_plc_set_points(self._handle, pts.ctypes.data_as(_L.c_double_p),
                                       pts.shape[0]), ctypes.create_string_buffer(1))
        return self

    def add_facet(self, vertex_indices: Sequence[int], marker: int = 0) -> "PLC":
        """Append a one-polygon facet (a triangle when three indices)."""
        idx = np.ascontiguousarray(vertex_indices, dtype=np.int32).ravel()
        if idx.size < 3:
            raise ValueError("a facet needs at least 3 vertex indices")
        _check(_clib.cmg_plc_add_facet(self._handle, idx.ctypes.data_as(_L.c_int_p), idx.size,
                                      int(marker)), ctypes.create_string_buffer(1))
        return self

    def add_facets(self, triangles) -> "PLC":
        """Append every row of an (M, k) index array as a facet (one bulk call for
        triangles)."""
        a = np.ascontiguousarray(triangles, dtype=np.int32)
        if a.ndim == 2 and a.shape[1] == 3:
            _check(_clib.cmg_plc_add_triangles(self._handle, a.ctypes.data_as(_L.c_int_p),
                                               len(a), 0), ctypes.create_string_buffer(1))
            return self
        for row in a:
            self.add_facet(row)
        return self

    def add_hole(self, x: float, y: float, z: float) -> "PLC":
        _check(_clib.cmg_plc_add_hole(self._handle, x, y, z), ctypes.create_string_buffer(1))
        return self

    def add_region(self, x: float, y: float, z: float, attribute: float = 0.0,
                   max_volume: float = -1.0) -> "PLC":
        _check(_clib.cmg_plc_add_region(self._handle, x, y, z, attribute, max_volume),
               ctypes.create_string_buffer(1))
        return self

    @classmethod
    def from_arrays(cls, points, triangles) -> "PLC":
        return cls().add_points(points).add_facets(triangles)

    def __del__(self) -> None:
        h = getattr(self, "_handle", None)
        if h:
            _clib.cmg_plc_destroy(h)
            self._handle = None


def read_plc(path: str) -> PLC:
    """Read a PLC boundary from a surface file, as the reference's ``read_plc``
    (bindings/python/src/cybermesh/__init__.py:395-397): .stl is read here (records
    decoded and vertices merged on the GPU); the reference's other formats are outside
    this library (RuntimeError)."""
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(512)
    _check(_clib.cmg_read_plc(str(path).encode(), ctypes.byref(out), err, 512), err)
    return PLC(out.value)


def plc_from_stl(data: bytes) -> PLC:
    """A PLC from an in-memory STL image (binary or ASCII), as read_plc reads a file."""
    buf = bytes(data)
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(512)
    _check(_clib.cmg_plc_from_stl(buf, len(buf), ctypes.byref(out), err, 512), err)
    return PLC(out.value)


def self_intersections(plc: PLC) -> np.ndarray:
    """Crossing pairs of fan triangles of the PLC's facets, as the reference's
    cmg::detect::self_intersections: an (k, 8) int32 array of rows (facet_a, facet_b,
    triangle a's three vertex indices, triangle b's), in the reference's order."""
    if not isinstance(plc, PLC):
        raise TypeError("plc must be a PLC")
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(512)
    _check(_clib.cmg_plc_self_intersections(plc._handle, ctypes.byref(out), err, 512), err)
    try:
        n = int(_clib.cmg_intersections_count(out.value))
        if n == 0:
            return np.zeros((0, 8), dtype=np.int32)
        return np.ctypeslib.as_array(_clib.cmg_intersections_data(out.value), (n * 8,)).reshape(n, 8).copy()
    finally:
        _clib.cmg_intersections_destroy(out.value)


def stl_last_timing() -> Dict[str, float]:
    """Phase times (ms, CUDA events) of the last STL read on the current device."""
    a, b, c = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
    _check(_clib.cmg_stl_last_timing(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
           ctypes.create_string_buffer(1))
    return {"upload_ms": a.value, "merge_ms": b.value, "download_ms": c.value}


def simplify(plc: PLC, grid: int = 34) -> PLC:
    """Simplify a PLC surface by grid vertex clustering and return a new PLC, as the
    reference's ``simplify`` (bindings/python/src/cybermesh/__init__.py:400-413 over
    src/simplify/simplify.cpp:48-112), on the GPU with bit-identical points and the
    same triangles in the same order. ``grid`` is the number of cells along the longest
    bounding-box axis."""
    if not isinstance(plc, PLC):
        raise TypeError("plc must be a PLC")
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(256)
    _check(_clib.cmg_plc_simplify(plc._handle, int(grid), ctypes.byref(out), err, 256), err)
    return PLC(out.value)


def simplify_last_timing() -> Dict[str, float]:
    """Phase times (ms, CUDA events) of the last simplify on the current device."""
    a, b, c = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
    _check(_clib.cmg_simplify_last_timing(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
           ctypes.create_string_buffer(1))
    return {"upload_ms": a.value, "cluster_ms": b.value, "download_ms": c.value}


class SizingField:
    """The background-mesh sizing field of the reference's
    ``cmg::sizing::from_background(mesh, node_sizes, scale)``
    (src/sizing/background.cpp:58-74) on the GPU: ``field(p)`` is the closure's value at
    one point, ``field.eval(queries)`` at many ((n, 3) NumPy array, or a CUDA float64
    torch tensor evaluated on the current stream), bit for bit the reference's: the
    sizes interpolated in the first tetrahedron (in order) that contains the point,
    else the nearest node's, times ``scale``. ``tets`` holds 4 node indices per row;
    ``node_sizes`` is padded with 0 or truncated to the node count."""

    def __init__(self, points, tets, node_sizes, scale: float = 1.0) -> None:
        P = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        T = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1, 4)
        S = np.ascontiguousarray(node_sizes, dtype=np.float64).ravel()
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        self._h = None
        _check(_clib.cmg_sizing_create(P.ctypes.data_as(_L.c_double_p), len(P),
                                       T.ctypes.data_as(_L.c_int_p), len(T),
                                       S.ctypes.data_as(_L.c_double_p), len(S), float(scale),
                                       ctypes.byref(h), err, 256), err)
        self._h = h.value

    def eval(self, queries, which: bool = False):
        """Sizes at the queries; with ``which``, also the answering tetrahedron per query
        (-1: the nearest node's size)."""
        err = ctypes.create_string_buffer(256)
        try:
            import torch
            is_tensor = isinstance(queries, torch.Tensor)
        except ImportError:
            is_tensor = False
        if is_tensor:
            if not queries.is_cuda or queries.dtype != torch.float64:
                raise TypeError("queries must be a CUDA float64 tensor")
            q = queries.reshape(-1, 3).contiguous()
            n = q.shape[0]
            out = torch.empty(n, dtype=torch.float64, device=q.device)
            w = torch.empty(n, dtype=torch.int32, device=q.device) if which else None
            st = torch.cuda.current_stream(q.device).cuda_stream
            _check(_clib.cmg_sizing_eval_device(self._h, q.data_ptr(), n, out.data_ptr(),
                                                w.data_ptr() if which else None, st, err, 256), err)
            return (out, w) if which else out
        q = np.ascontiguousarray(queries, dtype=np.float64).reshape(-1, 3)
        alloc = host_empty if len(q) >= 65536 else (lambda n, dt: np.empty(n, dtype=dt))
        out = alloc(len(q), np.float64)
        w = alloc(len(q), np.int32) if which else None
        _check(_clib.cmg_sizing_eval(self._h, q.ctypes.data_as(_L.c_double_p), len(q),
                                     out.ctypes.data_as(_L.c_double_p),
                                     w.ctypes.data_as(_L.c_int_p) if which else None, err, 256), err)
        return (out, w) if which else out

    def __call__(self, p) -> float:
        return float(self.eval(np.asarray(p, dtype=np.float64).reshape(1, 3))[0])

    def stats(self) -> Dict[str, float]:
        s = _L.SizingStats()
        _check(_clib.cmg_sizing_get_stats(self._h, ctypes.byref(s)), ctypes.create_string_buffer(1))
        return s.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None):
            _clib.cmg_sizing_destroy(self._h)
            self._h = None

    def __del__(self) -> None:
        self.close()


@dataclass
class VoxelGrid:
    """A regular grid from :func:`voxelize`: ``grid`` is (nx, ny, nz), uint8
    occupancy (1 inside) or float32 signed distance (negative inside); ``origin``
    is the centre of cell (0, 0, 0) and ``spacing`` the cubic cell size."""

    grid: np.ndarray
    origin: np.ndarray
    spacing: float
    mode: str

    @property
    def dims(self) -> tuple:
        return tuple(int(d) for d in self.grid.shape)


_VOXEL_MODES = {"occupancy": 0, "sdf": 1}


def _mode(mode):
    if isinstance(mode, str):
        try:
            return _VOXEL_MODES[mode], mode
        except KeyError:
            raise ValueError(f"mode must be one of {sorted(_VOXEL_MODES)} or 0/1")
    code = int(mode)
    if code not in (0, 1):
        raise ValueError("mode must be 'occupancy'/0 or 'sdf'/1")
    return code, "occupancy" if code == 0 else "sdf"


def _to_xyz(flat: np.ndarray, dims) -> np.ndarray:
    nx, ny, nz = dims
    # cells are laid out as idx = (k*ny + j)*nx + i: C order for (nz, ny, nx)
    return flat.reshape((nz, ny, nx)).transpose(2, 1, 0).copy()


def voxelize(plc: PLC, resolution: int = 64, mode="occupancy", pad: int = 1) -> VoxelGrid:
    """Voxelize a PLC (reference semantics: resolution cells on the longest axis,
    pad margin cells; "occupancy"/0 -> uint8, "sdf"/1 -> float32)."""
    if not isinstance(plc, PLC):
        raise TypeError("plc must be a PLC")
    code, name = _mode(mode)
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(256)
    _check(_clib.cmg_plc_voxelize(plc._handle, int(resolution), code, int(pad), ctypes.byref(out),
                                 err, 256), err)
    h = out.value
    try:
        dims, origin, spacing = _geometry(h)
        n = dims[0] * dims[1] * dims[2]
        if code == 0:
            flat = np.ctypeslib.as_array(_clib.cmg_voxels_occupancy(h), (n,)).astype(np.uint8)
        else:
            flat = np.ctypeslib.as_array(_clib.cmg_voxels_distance(h), (n,)).astype(np.float32)
        grid = _to_xyz(flat, dims)
    finally:
        _clib.cmg_voxels_destroy(h)
    return VoxelGrid(grid=grid, origin=origin, spacing=spacing, mode=name)


def _geometry(h):
    nx, ny, nz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _clib.cmg_voxels_dims(h, ctypes.byref(nx), ctypes.byref(ny), ctypes.byref(nz))
    ox, oy, oz = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _clib.cmg_voxels_origin(h, ctypes.byref(ox), ctypes.byref(oy), ctypes.byref(oz))
    return ((nx.value, ny.value, nz.value), np.array([ox.value, oy.value, oz.value]),
            float(_clib.cmg_voxels_spacing(h)))


@dataclass
class VoxelResult:
    """Outputs of :func:`voxelize_ex`, flat in the C layout idx = (k*ny + j)*nx + i
    (``as_xyz`` reshapes to (nx, ny, nz)). ``dims`` counts the layers held; ``layers``
    is (z_begin, z_end, nz of the grid): a slab holds layers z_begin .. z_end-1 of the
    grid whose corner and origin it reports."""

    dims: tuple
    origin: np.ndarray
    corner: np.ndarray
    spacing: float
    occupancy: Optional[np.ndarray] = None
    sdf32: Optional[np.ndarray] = None
    sdf64: Optional[np.ndarray] = None
    nearest_triangle: Optional[np.ndarray] = None
    nearest_region: Optional[np.ndarray] = None
    error_bound: Optional[np.ndarray] = None
    stats: Dict[str, float] = field(default_factory=dict)
    layers: tuple = (0, 0, 0)

    def as_xyz(self, a: np.ndarray) -> np.ndarray:
        return _to_xyz(a, self.dims)


def make_opts(resolution: int = 64, pad: int = 1, outputs: int = OUT_OCCUPANCY,
              precision: int = PREC_FP64, predicates: int = PRED_COMPAT, grid=None,
              band: float = 1.0, brick: int = 0, autotune: bool = False, grab: int = 0,
              stage: int = -1, walk_warps: int = 0, probe: int = 0,
              ctas: int = 0, layers=None) -> _L.VoxelOpts:
    """Options of voxelize_ex / Batch. ``layers=(z_begin, z_end)`` evaluates cell layers
    [z_begin, z_end) of the grid only (a z-slab; equal to those layers of the whole
    grid bit for bit)."""
    o = _L.VoxelOpts()
    _clib.cmg_voxel_opts_init(ctypes.byref(o))
    o.resolution, o.pad, o.outputs = int(resolution), int(pad), int(outputs)
    o.precision, o.predicates = int(precision), int(predicates)
    o.band, o.brick, o.autotune = float(band), int(brick), int(bool(autotune))
    o.grab, o.stage = int(grab), int(stage)
    o.walk_warps, o.probe, o.ctas = int(walk_warps), int(probe), int(ctas)
    if layers is not None:
        o.z_begin, o.z_end = int(layers[0]), int(layers[1])
    if grid is not None:
        corner, spacing, dims = grid
        o.explicit_grid = 1
        for a in range(3):
            o.corner[a] = float(corner[a])
            o.dims[a] = int(dims[a])
        o.spacing = float(spacing)
    return o


class _Owner:
    """Owns a cmg_voxels handle; destroys it when no array views its buffers."""

    def __init__(self, h) -> None:
        self.h = h

    def __del__(self) -> None:
        h, self.h = getattr(self, "h", None), None
        if h:
            _clib.cmg_voxels_destroy(h)


class _View:
    """Array interface over one buffer of an owned handle (keeps the owner alive)."""

    def __init__(self, owner: _Owner, ptr: int, n: int, dtype) -> None:
        self._owner = owner
        self.__array_interface__ = {"shape": (n,), "typestr": np.dtype(dtype).str,
                                    "data": (ptr, False), "version": 3}


def _result_from_handle(h, owner: Optional[_Owner] = None) -> VoxelResult:
    """The grid behind handle h. With an owner, the arrays view the handle's
    buffers (no copy) and the handle lives as long as they do; without, they are
    copies."""
    dims, origin, spacing = _geometry(h)
    cx, cy, cz = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _clib.cmg_voxels_corner(h, ctypes.byref(cx), ctypes.byref(cy), ctypes.byref(cz))
    n = dims[0] * dims[1] * dims[2]

    def grab(fn, dtype):
        p = fn(h)
        if not p:
            return None
        if owner is not None:
            return np.asarray(_View(owner, ctypes.cast(p, ctypes.c_void_p).value, n, dtype))
        return np.ctypeslib.as_array(p, (n,)).astype(dtype, copy=True)

    st = _L.VoxelStats()
    _clib.cmg_voxels_stats(h, ctypes.byref(st))
    z0, z1, nzg = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _clib.cmg_voxels_layers(h, ctypes.byref(z0), ctypes.byref(z1), ctypes.byref(nzg))
    return VoxelResult(
        dims=dims, origin=origin, corner=np.array([cx.value, cy.value, cz.value]), spacing=spacing,
        occupancy=grab(_clib.cmg_voxels_occupancy, np.uint8),
        sdf32=grab(_clib.cmg_voxels_distance, np.float32),
        sdf64=grab(_clib.cmg_voxels_distance_f64, np.float64),
        nearest_triangle=grab(_clib.cmg_voxels_nearest_triangle, np.int32),
        nearest_region=grab(_clib.cmg_voxels_nearest_region, np.uint8),
        error_bound=grab(_clib.cmg_voxels_error_bound, np.float32),
        stats=st.as_dict(), layers=(z0.value, z1.value, nzg.value))


def plc_grid(plc: PLC, resolution: int = 64, pad: int = 1):
    """(corner, spacing, dims) of the grid voxelize(plc, resolution, ., pad) uses (host
    only, no GPU)."""
    if not isinstance(plc, PLC):
        raise TypeError("plc must be a PLC")
    corner = np.zeros(3)
    spacing = ctypes.c_double()
    dims = np.zeros(3, dtype=np.int32)
    err = ctypes.create_string_buffer(256)
    _check(_clib.cmg_plc_grid(plc._handle, int(resolution), int(pad),
                              corner.ctypes.data_as(_L.c_double_p), ctypes.byref(spacing),
                              dims.ctypes.data_as(_L.c_int_p), err, 256), err)
    return corner, spacing.value, tuple(int(d) for d in dims)


def voxelize_ex(plc: PLC, **kw) -> VoxelResult:
    """Voxelize with explicit options (see :func:`make_opts`)."""
    if not isinstance(plc, PLC):
        raise TypeError("plc must be a PLC")
    o = make_opts(**kw)
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(512)
    _check(_clib.cmg_plc_voxelize_ex(plc._handle, ctypes.byref(o), ctypes.byref(out), err, 512), err)
    return _result_from_handle(out.value, _Owner(out.value))


class Batch:
    """Many PLCs voxelized by one pipeline (occupancy and/or SDF), resident on the
    GPU; ``run(graph=True)`` replays a captured CUDA graph after the first pass."""

    def __init__(self, plcs: Sequence[PLC], resolutions=None, pads=None, **kw):
        self._plcs = list(plcs)  # keep the handles alive
        n = len(self._plcs)
        res = np.ascontiguousarray(resolutions if resolutions is not None else [64] * n, dtype=np.int32)
        pad = np.ascontiguousarray(pads if pads is not None else [1] * n, dtype=np.int32)
        arr = (ctypes.c_void_p * n)(*[p._handle for p in self._plcs])
        o = make_opts(**kw)
        out = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        _check(_clib.cmg_batch_create(arr, res.ctypes.data_as(_L.c_int_p),
                                     pad.ctypes.data_as(_L.c_int_p), n, ctypes.byref(o),
                                     ctypes.byref(out), err, 512), err)
        self._h = out.value

    def __len__(self) -> int:
        return int(_clib.cmg_batch_size(self._h))

    @property
    def cells(self) -> int:
        return int(_clib.cmg_batch_cells(self._h))

    def run(self, graph: bool = False) -> "Batch":
        err = ctypes.create_string_buffer(512)
        _check(_clib.cmg_batch_run(self._h, int(graph), err, 512), err)
        return self

    def sync(self) -> "Batch":
        err = ctypes.create_string_buffer(512)
        _check(_clib.cmg_batch_sync(self._h, err, 512), err)
        return self

    def result(self, i: int) -> VoxelResult:
        out = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        _check(_clib.cmg_batch_get(self._h, int(i), ctypes.byref(out), err, 512), err)
        return _result_from_handle(out.value, _Owner(out.value))

    @property
    def stream(self) -> int:
        """The cudaStream_t (as an integer) the batch's kernels run on."""
        return int(_clib.cmg_batch_stream(self._h) or 0)

    def set_timing(self, on: bool = True) -> "Batch":
        _clib.cmg_batch_set_timing(self._h, int(on))
        return self

    def timing(self) -> Dict[str, float]:
        t = _L.BatchTiming()
        err = ctypes.create_string_buffer(512)
        _check(_clib.cmg_batch_get_timing(self._h, ctypes.byref(t), err, 512), err)
        return t.as_dict()

    def work_model(self) -> Dict[str, float]:
        w = _L.WorkModel()
        err = ctypes.create_string_buffer(512)
        _check(_clib.cmg_batch_work_model(self._h, ctypes.byref(w), err, 512), err)
        return w.as_dict()

    def stats(self) -> Dict[str, float]:
        st = _L.VoxelStats()
        err = ctypes.create_string_buffer(512)
        _check(_clib.cmg_batch_stats(self._h, ctypes.byref(st), err, 512), err)
        return st.as_dict()

    def __del__(self) -> None:
        h = getattr(self, "_h", None)
        if h:
            _clib.cmg_batch_destroy(h)
            self._h = None


MEM_HOST, MEM_DEVICE = 0, 1


class _HostBlock:
    """A page-locked block of the library's host pool, returned to the pool when the
    last array viewing it is collected."""

    def __init__(self, nbytes: int) -> None:
        self.ptr = _clib.cmg_host_alloc(max(int(nbytes), 1))
        if not self.ptr:
            raise MemoryError(f"cmg_host_alloc({nbytes}) failed")

    def __del__(self) -> None:
        if getattr(self, "ptr", None) and _clib is not None:
            _clib.cmg_host_free(self.ptr)
            self.ptr = None


def host_empty(n: int, dtype=np.int8) -> np.ndarray:
    """An uninitialised 1-D array in pooled page-locked host memory (the library
    writes into it without first-touch page faults; the block is reused after the
    array is collected)."""
    dt = np.dtype(dtype)
    blk = _HostBlock(n * dt.itemsize)
    return np.asarray(_View(blk, blk.ptr, n, dt))


def _stream_call(fn, npt, soa, mode, stream=None):
    """soa: (3*npt, n) float64 NumPy array (host) or a list of device pointers with n."""
    if isinstance(soa, np.ndarray):
        soa = np.ascontiguousarray(soa, dtype=np.float64)
        if soa.shape[0] != 3 * npt:
            raise ValueError(f"expected {3 * npt} coordinate rows")
        n = soa.shape[1]
        rows = (ctypes.c_void_p * (3 * npt))(*[soa[k].ctypes.data for k in range(3 * npt)])
        out = host_empty(n, np.int8) if n >= 65536 else np.zeros(n, dtype=np.int8)
        st = _L.PredStats()
        err = ctypes.create_string_buffer(512)
        _check(fn(rows, n, int(mode), MEM_HOST, out.ctypes.data_as(ctypes.c_void_p),
                  ctypes.byref(st), None, err, 512), err)
        return out, st.as_dict()
    ptrs, n, out_ptr = soa
    rows = (ctypes.c_void_p * (3 * npt))(*ptrs)
    st = _L.PredStats()
    err = ctypes.create_string_buffer(512)
    _check(fn(rows, int(n), int(mode), MEM_DEVICE, ctypes.c_void_p(out_ptr), ctypes.byref(st),
              ctypes.c_void_p(stream or 0), err, 512), err)
    return None, st.as_dict()


def orient3d_stream(soa, mode: int = PRED_COMPAT, stream=None):
    """Signs of orient3d queries: soa is a (12, n) float64 array (a, b, c, d in SoA),
    or (device pointers [12], n, device out pointer). Returns (signs int8, stats)."""
    return _stream_call(_clib.cmg_orient3d_stream, 4, soa, mode, stream)


def insphere_stream(soa, mode: int = PRED_COMPAT, stream=None):
    """Signs of insphere queries: soa is a (15, n) float64 array (a..e in SoA)."""
    return _stream_call(_clib.cmg_insphere_stream, 5, soa, mode, stream)


def orient3d_signs(points, tets) -> np.ndarray:
    """robust::orient3d_signs on the GPU: points (N, 3), tets (M, 4) indices."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    t = np.ascontiguousarray(tets, dtype=np.int32)
    out = np.zeros(len(t), dtype=np.int32)
    st = _clib.cmg_orient3d_signs(pts.ctypes.data_as(_L.c_double_p), len(pts),
                                  t.ctypes.data_as(_L.c_int_p), len(t),
                                  out.ctypes.data_as(_L.c_int_p))
    if st != 0:
        raise RuntimeError(f"cmg_orient3d_signs failed with status {st}")
    return out


def orient3d_batch(points, tets) -> np.ndarray:
    """robust::orient3d_batch on the GPU: the orient3d value of each candidate
    tetrahedron (tets (M, 4) indices into points (N, 3)), bit for bit the reference's."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    t = np.ascontiguousarray(tets, dtype=np.int32)
    out = np.zeros(len(t))
    st = _clib.cmg_orient3d_batch(pts.ctypes.data_as(_L.c_double_p), len(pts),
                                  t.ctypes.data_as(_L.c_int_p), len(t),
                                  out.ctypes.data_as(_L.c_double_p))
    if st != 0:
        raise RuntimeError(f"cmg_orient3d_batch failed with status {st}")
    return out


def gpu_launches() -> int:
    """Kernels launched by the library in this process."""
    return int(_clib.cmg_gpu_launches())


def peak_flops(fp64: bool) -> float:
    """Measured FMA throughput of the current GPU in FLOP/s (FMA = 2)."""
    v = ctypes.c_double()
    err = ctypes.create_string_buffer(512)
    _check(_clib.cmg_gpu_peak_flops(int(fp64), ctypes.byref(v), err, 512), err)
    return v.value


def version() -> str:
    return _clib.cmg_version().decode()


def gpu_version() -> str:
    return _clib.cmg_gpu_version().decode()


def library_path() -> str:
    return _L.library_path()


__all__ = ["orient3d_stream", "insphere_stream", "host_empty", "orient3d_signs", "orient3d_batch", "PLC", "VoxelGrid", "VoxelResult", "voxelize", "voxelize_ex", "plc_grid", "make_opts", "Batch",
           "version", "gpu_version", "library_path", "OUT_OCCUPANCY", "OUT_SDF_F32", "OUT_SDF_F64",
           "OUT_NEAREST", "OUT_ERROR_BOUND", "PREC_FP64", "PREC_MIXED", "PRED_COMPAT", "PRED_EXACT",
           "read_plc", "plc_from_stl", "self_intersections", "simplify", "stl_last_timing",
           "simplify_last_timing", "SizingField"]
