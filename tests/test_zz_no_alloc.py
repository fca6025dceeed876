"""cmg_gpu_occupancy_static: occupancy for callers that cannot allocate device
memory (a framework that owns the device memory through its own pool, a loop that
may not allocate after start-up). The caller passes device buffers; the library's
working memory is a fixed static array. Its output must equal the allocating entry
point's (cmg_plc_voxelize_ex) bit for bit, on two calls in a row (the second call
finds the first call's leftovers in the shared array). This file is collected
last so that a run stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from conftest import unpack_occ

pytestmark = pytest.mark.gpu


def _call(cm, torch, points, tris, corner, spacing, dims, predicates=0):
    from cybermeshgenerator_gb300 import _lib as L
    lib = L.load()
    d_pts = torch.tensor(np.ascontiguousarray(points, np.float64), device="cuda")
    d_tri = torch.tensor(np.ascontiguousarray(tris, np.int32), device="cuda")
    n = int(np.prod(dims))
    d_occ = torch.full((n,), 7, dtype=torch.uint8, device="cuda")  # garbage: every cell is written
    c = np.ascontiguousarray(corner, np.float64)
    d = np.ascontiguousarray(dims, np.int32)
    err = ctypes.create_string_buffer(256)
    st = lib.cmg_gpu_occupancy_static(
        ctypes.c_void_p(d_pts.data_ptr()), len(points), ctypes.c_void_p(d_tri.data_ptr()), len(tris),
        c.ctypes.data_as(L.c_double_p), float(spacing), d.ctypes.data_as(L.c_int_p), predicates,
        ctypes.c_void_p(d_occ.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
        err, 256)
    return st, err.value.decode(), d_occ.cpu().numpy()


def test_static_scratch_matches_allocating_entry_point(cm, golden):
    torch = pytest.importorskip("torch")
    # two calls in a row on different meshes and grids
    for name in ("boxtorus64_facegrid", "icosphere_s3_r58p3"):
        g = golden(name)
        grid = (g["corner"], float(g["spacing"]), tuple(int(x) for x in g["dims"]))
        want = cm.voxelize_ex(cm.PLC.from_arrays(g["points"], g["triangles"]), grid=grid,
                              outputs=cm.OUT_OCCUPANCY).occupancy
        st, msg, got = _call(cm, torch, g["points"], g["triangles"], *grid)
        assert st == 0, msg
        assert np.array_equal(got, want)
        assert np.array_equal(got, unpack_occ(g))


def test_static_scratch_rejects_oversized_input(cm, golden):
    torch = pytest.importorskip("torch")
    g = golden("cube4_r16p1")
    st, msg, _ = _call(cm, torch, g["points"], g["triangles"], g["corner"], float(g["spacing"]),
                       (4096, 4096, 1))
    assert st == 1 and "static scratch" in msg


def test_static_scratch_rejects_a_stream_being_captured(cm, golden):
    """The call synchronises its stream, so on a stream being captured into a CUDA graph
    it returns CMG_ERR_UNSUPPORTED_OPTION before any device work: the capture goes on
    (its graph replays), and the next call on an ordinary stream is correct."""
    torch = pytest.importorskip("torch")
    from cybermeshgenerator_gb300 import _lib as L
    lib = L.load()
    g = golden("cube4_r16p1")
    d_pts = torch.tensor(np.ascontiguousarray(g["points"], np.float64), device="cuda")
    d_tri = torch.tensor(np.ascontiguousarray(g["triangles"], np.int32), device="cuda")
    dims = np.ascontiguousarray(g["dims"], np.int32)
    corner = np.ascontiguousarray(g["corner"], np.float64)
    d_occ = torch.zeros(int(np.prod(dims)), dtype=torch.uint8, device="cuda")
    x = torch.zeros(16, device="cuda")
    err = ctypes.create_string_buffer(256)
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        graph.capture_begin()
        st = lib.cmg_gpu_occupancy_static(
            ctypes.c_void_p(d_pts.data_ptr()), len(g["points"]), ctypes.c_void_p(d_tri.data_ptr()),
            len(g["triangles"]), corner.ctypes.data_as(L.c_double_p), float(g["spacing"]),
            dims.ctypes.data_as(L.c_int_p), 0, ctypes.c_void_p(d_occ.data_ptr()),
            ctypes.c_void_p(side.cuda_stream), err, 256)
        x.add_(1.0)
        graph.capture_end()
    assert st == 3 and "being captured" in err.value.decode()
    graph.replay()
    torch.cuda.synchronize()
    assert float(x[0].item()) == 1.0
    st, msg, got = _call(cm, torch, g["points"], g["triangles"], corner, float(g["spacing"]),
                         tuple(int(v) for v in dims))
    assert st == 0, msg
    assert np.array_equal(got, unpack_occ(g))
