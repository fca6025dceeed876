"""The drop-in entry point cmg_plc_voxelize (bindings/c/src/cmg_c.cpp:242-267) and the
Python mirror voxelize() on the GPU, with the reference's semantics:

* one output per mode (src/voxelize/voxelize.cpp:393-396): occupancy grids carry no
  distance view and distance grids no occupancy view; any mode other than 1 means
  occupancy (cmg_c.cpp:254-255);
* outputs equal to the reference's own (tests/golden fixtures);
* the reference binding's checks (bindings/python/tests/test_cybermesh_voxelize.py:44-97)
  restated on this package: axis order on non-cubic grids, dtypes, mode spellings,
  occupied volume, SDF sign;
* the reference's binding itself, run against this library through CMG_C_LIB, where
  the reference source tree is present (CMG_REFERENCE_ROOT).
"""
import ctypes
import hashlib
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import unpack_occ

pytestmark = pytest.mark.gpu

CASES = ["cube4_r16p1", "brick312_r20p1", "icosphere_s3_r58p3", "shsphere64_r30p1",
         "cube4deg_r16p1"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _c_voxelize(cm, plc, resolution, mode, pad):
    """cmg_plc_voxelize through the C ABI: (handle, status, error text)."""
    from cybermeshgenerator_gb300 import _lib
    L = _lib.load()
    out = ctypes.c_void_p(123)
    err = ctypes.create_string_buffer(256)
    st = L.cmg_plc_voxelize(plc._handle, resolution, mode, pad, ctypes.byref(out), err, 256)
    return L, out.value, st, err.value.decode()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("mode", [0, 1, 7])
def test_cmg_plc_voxelize_one_output_per_mode(cm, golden, name, mode):
    g = golden(name)
    plc = cm.PLC.from_arrays(g["points"], g["triangles"])
    L, h, st, msg = _c_voxelize(cm, plc, int(g["resolution"]), mode, int(g["pad"]))
    assert st == 0, msg
    try:
        nx, ny, nz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.cmg_voxels_dims(h, ctypes.byref(nx), ctypes.byref(ny), ctypes.byref(nz))
        dims = (nx.value, ny.value, nz.value)
        assert dims == tuple(int(d) for d in g["dims"])
        o = [ctypes.c_double() for _ in range(3)]
        L.cmg_voxels_origin(h, *(ctypes.byref(x) for x in o))
        assert np.array_equal([x.value for x in o], g["origin"])
        assert L.cmg_voxels_spacing(h) == float(g["spacing"])
        n = int(np.prod(dims))
        occ_p, dist_p = L.cmg_voxels_occupancy(h), L.cmg_voxels_distance(h)
        if mode == 1:
            assert not occ_p
            d = np.ctypeslib.as_array(dist_p, (n,)).copy()
            assert _sha(d) == str(g["sdf32_sha"])
        else:
            assert not dist_p
            occ = np.ctypeslib.as_array(occ_p, (n,)).copy()
            assert np.array_equal(occ, unpack_occ(g))
    finally:
        L.cmg_voxels_destroy(h)


@pytest.mark.parametrize("name", CASES)
def test_python_voxelize_axis_order_and_dtypes(cm, golden, name):
    g = golden(name)
    plc = cm.PLC.from_arrays(g["points"], g["triangles"])
    nx, ny, nz = (int(d) for d in g["dims"])
    want = unpack_occ(g).reshape(nz, ny, nx).transpose(2, 1, 0)
    for mode in ("occupancy", 0):
        vg = cm.voxelize(plc, resolution=int(g["resolution"]), mode=mode, pad=int(g["pad"]))
        assert vg.grid.dtype == np.uint8 and vg.grid.shape == (nx, ny, nz) == vg.dims
        assert np.array_equal(vg.grid, want) and vg.mode == "occupancy"
        assert vg.origin.dtype == np.float64 and np.array_equal(vg.origin, g["origin"])
    sdf = cm.voxelize(plc, resolution=int(g["resolution"]), mode="sdf", pad=int(g["pad"]))
    assert sdf.grid.dtype == np.float32 and sdf.grid.shape == (nx, ny, nz)
    flat = np.ascontiguousarray(sdf.grid.transpose(2, 1, 0)).ravel()
    assert _sha(flat) == str(g["sdf32_sha"]) and sdf.mode == "sdf"


# ---- the reference binding's checks, restated -------------------------------------
def _box(cm, X, Y, Z):
    """Watertight box [0,X]x[0,Y]x[0,Z], each face split into two triangles."""
    p = cm.PLC().add_points([[0, 0, 0], [X, 0, 0], [X, Y, 0], [0, Y, 0],
                            [0, 0, Z], [X, 0, Z], [X, Y, Z], [0, Y, Z]])
    for a, b, c, d in [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5),
                       (0, 4, 7, 3)]:
        p.add_facet([a, b, c])
        p.add_facet([a, c, d])
    return p


@pytest.mark.parametrize("X,Y,Z", [(2.0, 1.0, 1.0), (1.0, 2.0, 1.0), (1.0, 1.0, 2.0),
                                   (3.0, 1.0, 2.0)])
def test_grid_axes_on_non_cubic_boxes(cm, X, Y, Z):
    vg = cm.voxelize(_box(cm, X, Y, Z), resolution=20, pad=1)
    nx, ny, nz = vg.dims
    assert vg.dims[int(np.argmax([X, Y, Z]))] == max(vg.dims)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cx, cy, cz = (vg.origin[a] + idx * vg.spacing for a, idx in enumerate((i, j, k)))
    inside = ((cx > 0) & (cx < X) & (cy > 0) & (cy < Y) & (cz > 0) & (cz < Z)).astype(np.uint8)
    assert float((inside == vg.grid).mean()) > 0.98


def test_cube_volume_modes_and_sign(cm):
    cube = _box(cm, 2.0, 2.0, 2.0)
    vg = cm.voxelize(cube, resolution=32, mode="occupancy", pad=1)
    assert vg.grid.dtype == np.uint8 and vg.grid.ndim == 3 and vg.grid.shape == vg.dims
    assert vg.origin.shape == (3,) and vg.origin.dtype == np.float64 and vg.spacing > 0
    occupied, total = int(vg.grid.sum()), int(vg.grid.size)
    assert 0 < occupied < total
    assert abs(occupied * vg.spacing ** 3 - 8.0) / 8.0 < 0.15
    assert np.array_equal(cm.voxelize(cube, resolution=32, mode=0, pad=1).grid, vg.grid)
    sdf = cm.voxelize(cube, resolution=32, mode="sdf", pad=1)
    assert sdf.grid.dtype == np.float32 and sdf.grid.shape == vg.grid.shape
    assert (sdf.grid < 0).any() and (sdf.grid > 0).any()
    assert float((sdf.grid[vg.grid.astype(bool)] <= sdf.spacing).mean()) > 0.9
    with pytest.raises(ValueError):
        cm.voxelize(cube, resolution=32, mode="surface")
    with pytest.raises(RuntimeError, match="resolution must be >= 1"):
        cm.voxelize(cube, resolution=0)


def _reference_binding():
    root = os.environ.get("CMG_REFERENCE_ROOT")
    test = os.path.join(root or "", "bindings", "python", "tests", "test_cybermesh_voxelize.py")
    if not root or not os.path.exists(test):
        pytest.skip("the reference source tree (CMG_REFERENCE_ROOT) is not present")
    return os.path.join(root, "bindings", "python", "src"), test


def test_reference_binding_runs_on_this_library(cm):
    """The unmodified reference binding and its voxelize test, with CMG_C_LIB pointing
    at this library."""
    src, test = _reference_binding()
    env = dict(os.environ, CMG_C_LIB=cm.library_path(),
               PYTHONPATH=src + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, test], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASS: voxelize" in r.stdout
