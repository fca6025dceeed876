"""Failed device allocations, made on the host (a fake of cudaMalloc's failure through
cmg_debug_fail_device_allocs; no GPU fault is involved): every call that meets one
returns CMG_ERR_INTERNAL with "out of memory" in its error buffer, and the next call
works and gives the same results as before. Covered: each of a batch's four workspace
arenas (inputs, outputs, bucket entries, candidate lists), the shared workspace of
single calls growing for a larger input, and the adjoint plan's own buffers."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def fail(cm):
    from cybermeshgenerator_gb300 import _lib
    L = _lib.load()

    def set_(skip, count):
        assert L.cmg_debug_fail_device_allocs(skip, count) == 0
    yield set_
    L.cmg_debug_fail_device_allocs(0, 0)


def _mesh(golden, name):
    g = golden(name)
    return g["points"], g["triangles"], int(g["resolution"]), int(g["pad"])


def _batch(cm, plc, res, pad):
    b = cm.Batch([plc], [res], [pad], outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F64,
                 precision=cm.PREC_MIXED)
    r = b.run().sync().result(0)
    return np.array(r.occupancy), np.array(r.sdf64)


def test_batch_arena_failures(cm, golden, fail):
    pts, tris, res, pad = _mesh(golden, "shsphere64_r30p1")
    plc = cm.PLC.from_arrays(pts, tris)
    occ0, sdf0 = _batch(cm, plc, res, pad)
    failed = 0
    for skip in range(6):
        fail(skip, 1)
        try:
            _batch(cm, plc, res, pad)
        except RuntimeError as e:
            assert "out of memory" in str(e)
            failed += 1
        fail(0, 0)
        occ, sdf = _batch(cm, plc, res, pad)
        assert np.array_equal(occ, occ0) and np.array_equal(sdf.view(np.uint64), sdf0.view(np.uint64))
    assert failed >= 4  # inputs, outputs, bucket entries, candidate lists


def test_shared_workspace_growth_failure(cm, golden, fail):
    small = _mesh(golden, "cube4_r16p1")
    big = _mesh(golden, "icosphere_s3_r58p3")
    outs = cm.OUT_OCCUPANCY | cm.OUT_SDF_F32
    cm.voxelize_ex(cm.PLC.from_arrays(small[0], small[1]), resolution=small[2], pad=small[3],
                   outputs=outs)
    plc = cm.PLC.from_arrays(big[0], big[1])
    # a larger input than the shared workspace has held makes it grow: fail that
    fail(0, 4)
    with pytest.raises(RuntimeError, match="out of memory"):
        cm.voxelize_ex(plc, resolution=1024, pad=1, outputs=outs)
    fail(0, 0)
    r = cm.voxelize_ex(plc, resolution=big[2], pad=big[3], outputs=outs)
    g = golden("icosphere_s3_r58p3")
    from conftest import unpack_occ
    assert np.array_equal(r.occupancy, unpack_occ(g))
    import hashlib
    assert hashlib.sha256(r.sdf32.tobytes()).hexdigest() == str(g["sdf32_sha"])


def test_plan_allocation_failure(cm, golden, fail):
    from cybermeshgenerator_gb300 import _lib
    L = _lib.load()
    g = golden("uvsphere16_r20p1")
    pts = np.ascontiguousarray(g["points"], np.float64)
    tri = np.ascontiguousarray(g["triangles"], np.int32)
    o = cm.make_opts(grid=(g["corner"], g["spacing"], g["dims"]))
    err = ctypes.create_string_buffer(512)
    for skip in range(8):
        fail(skip, 1)
        out = ctypes.c_void_p()
        st = L.cmg_sdf_plan_create(pts.ctypes.data_as(_lib.c_double_p), len(pts),
                                   tri.ctypes.data_as(_lib.c_int_p), len(tri), ctypes.byref(o),
                                   ctypes.byref(out), err, 512)
        fail(0, 0)
        if st != 0:
            assert st == 6 and b"out of memory" in err.value and not out.value
        else:
            L.cmg_sdf_plan_destroy(out.value)
    out = ctypes.c_void_p()
    assert L.cmg_sdf_plan_create(pts.ctypes.data_as(_lib.c_double_p), len(pts),
                                 tri.ctypes.data_as(_lib.c_int_p), len(tri), ctypes.byref(o),
                                 ctypes.byref(out), err, 512) == 0
    L.cmg_sdf_plan_destroy(out.value)
