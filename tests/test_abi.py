"""The C ABI surface on the CPU: the library loads, exports every symbol the
headers declare, and answers the reference's validation errors without touching
a GPU (no compute call is made here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "cmg_c", h) for h in ("cmg_c.h", "cmg_gpu.h")]

# the 41 symbols the reference's ctypes binding touches at import
# (bindings/python/src/cybermesh/__init__.py:58-157)
REFERENCE_BOUND = """cmg_delaunay cmg_mesh_destroy cmg_mesh_face_markers cmg_mesh_faces
cmg_mesh_num_faces cmg_mesh_num_points cmg_mesh_num_tets cmg_mesh_points cmg_mesh_tet_markers
cmg_mesh_tets cmg_options_create cmg_options_destroy cmg_options_set_max_volume
cmg_options_set_plc cmg_options_set_preserve_edges cmg_options_set_quality cmg_plc_add_facet
cmg_plc_add_hole cmg_plc_add_region cmg_plc_create cmg_plc_destroy cmg_plc_num_points
cmg_plc_num_triangles cmg_plc_points cmg_plc_set_points cmg_plc_simplify cmg_plc_triangles
cmg_plc_voxelize cmg_read_mesh cmg_read_plc cmg_read_points cmg_tetrahedralize cmg_version
cmg_voxels_destroy cmg_voxels_dims cmg_voxels_distance cmg_voxels_occupancy cmg_voxels_origin
cmg_voxels_spacing cmg_write_mesh cmg_write_plc""".split()


@pytest.fixture(scope="module")
def lib():
    from cybermeshgenerator_gb300 import build, _lib
    build.build()
    return _lib.load()


def declared():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(cmg_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_reference_symbols_declared():
    assert len(REFERENCE_BOUND) == 41
    assert set(REFERENCE_BOUND) <= set(declared())


def test_every_declared_symbol_exported(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing


def test_null_and_resolution_errors(lib):
    out = ctypes.c_void_p(123)
    err = ctypes.create_string_buffer(64)
    assert lib.cmg_plc_voxelize(None, 8, 0, 1, ctypes.byref(out), err, 64) == 1
    assert out.value is None
    plc = lib.cmg_plc_create()
    try:
        assert lib.cmg_plc_voxelize(plc, 0, 0, 1, ctypes.byref(out), err, 64) == 1
        assert err.value == b"resolution must be >= 1"
        small = ctypes.create_string_buffer(8)
        assert lib.cmg_plc_voxelize(plc, 0, 0, 1, ctypes.byref(out), small, 8) == 1
        assert small.value == b"resolut"  # truncated to len-1 chars, NUL-terminated
        assert lib.cmg_plc_voxelize(plc, 8, 0, 1, None, err, 64) == 1
    finally:
        lib.cmg_plc_destroy(plc)


def test_empty_plc_is_invalid_input(lib):
    # voxelize.cpp:366-372: no points / no boundary triangles -> InvalidInput,
    # answered before any GPU work
    from cybermeshgenerator_gb300 import _lib as L
    plc = lib.cmg_plc_create()
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(128)
    try:
        assert lib.cmg_plc_voxelize(plc, 8, 0, 1, ctypes.byref(out), err, 128) == 1
        assert err.value == b"voxelize: PLC has no points"
        pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=np.float64)
        lib.cmg_plc_set_points(plc, pts.ctypes.data_as(L.c_double_p), 3)
        assert lib.cmg_plc_voxelize(plc, 8, 0, 1, ctypes.byref(out), err, 128) == 1
        assert err.value == b"voxelize: PLC has no boundary triangles"
        bad = np.array([0, 1, 7], dtype=np.int32)
        lib.cmg_plc_add_facet(plc, bad.ctypes.data_as(L.c_int_p), 3, 0)
        assert lib.cmg_plc_voxelize(plc, 8, 0, 1, ctypes.byref(out), err, 128) == 1
        assert b"out of range" in err.value
    finally:
        lib.cmg_plc_destroy(plc)


def test_simplify_validation(lib):
    # simplify.cpp:49-54: no points, then grid < 1 -> InvalidInput, answered before any
    # GPU work
    from cybermeshgenerator_gb300 import _lib as L
    plc = lib.cmg_plc_create()
    out = ctypes.c_void_p(123)
    err = ctypes.create_string_buffer(128)
    try:
        assert lib.cmg_plc_simplify(None, 8, ctypes.byref(out), err, 128) == 1
        assert out.value is None
        assert lib.cmg_plc_simplify(plc, 0, ctypes.byref(out), err, 128) == 1
        assert err.value == b"simplify: PLC has no points"
        pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=np.float64)
        lib.cmg_plc_set_points(plc, pts.ctypes.data_as(L.c_double_p), 3)
        assert lib.cmg_plc_simplify(plc, 0, ctypes.byref(out), err, 128) == 1
        assert err.value == b"simplify: grid must be >= 1"
        assert lib.cmg_plc_simplify(plc, 8, None, err, 128) == 1
    finally:
        lib.cmg_plc_destroy(plc)


def test_sizing_validation(lib):
    # a non-finite node or an index outside the nodes is refused before any GPU work
    from cybermeshgenerator_gb300 import _lib as L
    out = ctypes.c_void_p(123)
    err = ctypes.create_string_buffer(128)
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    tet = np.array([0, 1, 2, 4], dtype=np.int32)
    sz = np.ones(4)
    args = lambda p, t: (p.ctypes.data_as(L.c_double_p), 4, t.ctypes.data_as(L.c_int_p), 1,
                         sz.ctypes.data_as(L.c_double_p), 4, 1.0, ctypes.byref(out), err, 128)
    assert lib.cmg_sizing_create(*args(pts, tet)) == 1
    assert err.value == b"sizing: tetrahedron vertex index out of range"
    assert out.value is None
    bad = pts.copy()
    bad[2, 1] = np.nan
    assert lib.cmg_sizing_create(*args(bad, np.array([0, 1, 2, 3], dtype=np.int32))) == 1
    assert err.value == b"sizing: non-finite background point"
    assert lib.cmg_sizing_create(None, 4, None, 0, None, 0, 1.0, ctypes.byref(out), err, 128) == 1
    assert lib.cmg_sizing_eval(None, None, 0, None, None, err, 128) == 1


def test_facet_validation_and_readback(lib):
    from cybermeshgenerator_gb300 import _lib as L
    plc = lib.cmg_plc_create()
    try:
        pts = np.arange(15, dtype=np.float64).reshape(5, 3)
        assert lib.cmg_plc_set_points(plc, pts.ctypes.data_as(L.c_double_p), 5) == 0
        two = np.array([0, 1], dtype=np.int32)
        assert lib.cmg_plc_add_facet(plc, two.ctypes.data_as(L.c_int_p), 2, 0) == 1
        quad = np.array([0, 1, 2, 3, 4], dtype=np.int32)
        assert lib.cmg_plc_add_facet(plc, quad.ctypes.data_as(L.c_int_p), 5, 7) == 0
        n = lib.cmg_plc_num_triangles(plc)
        tri = np.ctypeslib.as_array(lib.cmg_plc_triangles(plc), (n * 3,))
        # fan (v0, v[i-1], v[i]) as voxelize.cpp:29-38
        assert tri.tolist() == [0, 1, 2, 0, 2, 3, 0, 3, 4]
        assert lib.cmg_plc_num_points(plc) == 5
        back = np.ctypeslib.as_array(lib.cmg_plc_points(plc), (15,))
        assert np.array_equal(back, pts.ravel())
    finally:
        lib.cmg_plc_destroy(plc)


def test_out_of_scope_entry_points(lib):
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(256)
    opts = lib.cmg_options_create()
    plc = lib.cmg_plc_create()
    try:
        assert lib.cmg_tetrahedralize(plc, opts, ctypes.byref(out), err, 256) == 5
        assert lib.cmg_read_plc(b"x.poly", ctypes.byref(out), err, 256) == 5
        # .stl is read here: a missing file is the reference's error, before any GPU work
        assert lib.cmg_read_plc(b"no_such_dir/x.stl", ctypes.byref(out), err, 256) == 1
        assert err.value == b"cannot open file for reading: no_such_dir/x.stl"
        assert lib.cmg_read_plc(b"x.xyz", ctypes.byref(out), err, 256) == 1
        assert err.value == b"unsupported file format for x.xyz"
        assert lib.cmg_mesh_num_points(None) == 0 and not lib.cmg_mesh_points(None)
        assert lib.cmg_options_set_plc(opts, 1) == 0
    finally:
        lib.cmg_plc_destroy(plc)
        lib.cmg_options_destroy(opts)


def test_getters_tolerate_null(lib):
    nx = ctypes.c_int(5)
    lib.cmg_voxels_dims(None, ctypes.byref(nx), None, None)
    assert nx.value == 0 and lib.cmg_voxels_spacing(None) == 0.0
    assert not lib.cmg_voxels_occupancy(None) and not lib.cmg_voxels_distance(None)
    assert lib.cmg_version() == b"0.5.0"


def test_bulk_triangles_equal_single_facets(lib):
    """cmg_plc_add_triangles appends the same facets as one cmg_plc_add_facet call
    per triangle (same fan triangulation readback), after any earlier polygon."""
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.icosphere(2)
    quad = [0, 1, 2, 3]
    a = cm.PLC().add_points(pts).add_facet(quad)
    for t in tris:
        a.add_facet(t)
    b = cm.PLC().add_points(pts).add_facet(quad).add_facets(tris)
    assert len(a.triangles) == len(b.triangles) == len(tris) + 2
    assert np.array_equal(a.triangles, b.triangles)
    assert np.array_equal(b.triangles[2:], tris)


def test_host_blocks_without_gpu(lib):
    """cmg_host_alloc hands out ordinary heap memory where nothing can be page-locked
    (no GPU here): the array over it is writable, and its block goes back to the
    library when the array is collected; a NULL free is ignored."""
    import gc
    import cybermeshgenerator_gb300 as cm
    for _ in range(3):
        a = cm.host_empty(1 << 20, np.float32)
        a[:] = 1.5
        assert a.dtype == np.float32 and a.shape == (1 << 20,) and float(a.sum()) == 1.5 * (1 << 20)
        del a
        gc.collect()
    lib.cmg_host_free(None)


def test_large_triangle_plc_readback(lib):
    """A PLC of triangles only, with arrays above the 1 MiB pool threshold: points and
    fan triangles read back as given (the fan of a triangle is itself, copied as
    stored), and an appended quad switches the readback to the general fan."""
    import cybermeshgenerator_gb300 as cm
    rng = np.random.default_rng(7)
    pts = rng.random((200_000, 3))
    tris = rng.integers(0, len(pts), size=(400_000, 3)).astype(np.int32)
    plc = cm.PLC.from_arrays(pts, tris)
    assert np.array_equal(plc.points, pts)
    assert np.array_equal(plc.triangles, tris)
    plc.add_facet([0, 1, 2, 3])
    t = plc.triangles
    assert len(t) == len(tris) + 2 and np.array_equal(t[:-2], tris)
    assert t[-2:].tolist() == [[0, 1, 2], [0, 2, 3]]


@pytest.mark.parametrize("name", ["icosphere_s3_r58p3", "brick312_r20p1", "shsphere64_r30p1"])
def test_plc_grid_equals_reference_grid(lib, golden, name):
    """cmg_plc_grid is the reference's make_grid (host only): corner, spacing and dims
    of the fixture's grid, bit for bit."""
    import cybermeshgenerator_gb300 as cm
    g = golden(name)
    corner, spacing, dims = cm.plc_grid(cm.PLC.from_arrays(g["points"], g["triangles"]),
                                        int(g["resolution"]), int(g["pad"]))
    assert np.array_equal(corner, g["corner"]) and spacing == float(g["spacing"])
    assert dims == tuple(int(d) for d in g["dims"])
    with pytest.raises(RuntimeError, match="resolution must be >= 1"):
        cm.plc_grid(cm.PLC.from_arrays(g["points"], g["triangles"]), 0, 1)


def test_layers_validation_without_gpu(lib, golden):
    """Slab options answer their errors on the host, before any GPU call."""
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import _lib as L
    g = golden("cube4_r16p1")
    plc = cm.PLC.from_arrays(g["points"], g["triangles"])
    nz = int(g["dims"][2])
    for layers in ((5, 3), (-1, 4), (0, nz + 1), (nz, 0)):
        with pytest.raises(RuntimeError, match="cell layers"):
            cm.voxelize_ex(plc, resolution=16, pad=1, layers=layers)
    with pytest.raises(RuntimeError, match="whole meshes"):
        cm.Batch([plc], [16], [1], layers=(0, 4))
    o = cm.make_opts(grid=(g["corner"], g["spacing"], g["dims"]), layers=(0, 4))
    out = ctypes.c_void_p()
    err = ctypes.create_string_buffer(256)
    pts = np.ascontiguousarray(g["points"], np.float64)
    tri = np.ascontiguousarray(g["triangles"], np.int32)
    assert lib.cmg_sdf_plan_create(pts.ctypes.data_as(L.c_double_p), len(pts),
                                   tri.ctypes.data_as(L.c_int_p), len(tri), ctypes.byref(o),
                                   ctypes.byref(out), err, 256) == 3
    assert b"whole grid" in err.value and not out.value
