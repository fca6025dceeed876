"""Loading and binding libcmg_c.so (the GPU voxelization library).

The library is looked up as the reference binding does it
(bindings/python/src/cybermesh/__init__.py:45-56): the ``CMG_C_LIB``
environment variable first, then the copy built in this package directory.
There is no fallback: if the library is missing, importing fails with the build
command to run.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
IN_TREE = os.path.join(HERE, "libcmg_c.so")

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)
c_void_pp = ctypes.POINTER(ctypes.c_void_p)
c_ubyte_p = ctypes.POINTER(ctypes.c_ubyte)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_int64_p = ctypes.POINTER(ctypes.c_int64)


class VoxelOpts(ctypes.Structure):
    """Mirror of ``cmg_voxel_opts`` (include/cmg_c/cmg_gpu.h)."""
    _fields_ = [("resolution", ctypes.c_int), ("pad", ctypes.c_int), ("mode", ctypes.c_int),
                ("outputs", ctypes.c_int), ("precision", ctypes.c_int),
                ("predicates", ctypes.c_int), ("explicit_grid", ctypes.c_int),
                ("corner", ctypes.c_double * 3), ("spacing", ctypes.c_double),
                ("dims", ctypes.c_int * 3), ("band", ctypes.c_double), ("brick", ctypes.c_int),
                ("autotune", ctypes.c_int), ("grab", ctypes.c_int), ("stage", ctypes.c_int),
                ("walk_warps", ctypes.c_int), ("probe", ctypes.c_int), ("ctas", ctypes.c_int),
                ("z_begin", ctypes.c_int), ("z_end", ctypes.c_int)]


class VoxelStats(ctypes.Structure):
    """Mirror of ``cmg_voxel_stats`` (include/cmg_c/cmg_gpu.h)."""
    _fields_ = [("cells", ctypes.c_int64), ("flagged_columns", ctypes.c_int64),
                ("nudged_columns", ctypes.c_int64), ("exhausted_columns", ctypes.c_int64),
                ("exact_calls", ctypes.c_int64), ("bucket_entries", ctypes.c_int64),
                ("candidates", ctypes.c_int64), ("evaluations", ctypes.c_int64),
                ("fp64_evaluations", ctypes.c_int64), ("band_cells", ctypes.c_int64),
                ("filtered", ctypes.c_int64), ("brick", ctypes.c_int), ("grab", ctypes.c_int),
                ("max_error_bound", ctypes.c_double), ("walk_warps", ctypes.c_int),
                ("probe", ctypes.c_int), ("ctas", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchTiming(ctypes.Structure):
    _fields_ = [("occupancy_ms", ctypes.c_float), ("sdf_prep_ms", ctypes.c_float),
                ("eval_ms", ctypes.c_float), ("total_ms", ctypes.c_float)]

    def as_dict(self):
        return {k: float(getattr(self, k)) for k, _ in self._fields_}


class WorkModel(ctypes.Structure):
    _fields_ = [("sum_k", ctypes.c_double), ("sum_k_band", ctypes.c_double),
                ("band_cells", ctypes.c_double), ("orient_calls", ctypes.c_double),
                ("crossings", ctypes.c_double)]

    def as_dict(self):
        return {k: float(getattr(self, k)) for k, _ in self._fields_}


class PredStats(ctypes.Structure):
    _fields_ = [("queries", ctypes.c_int64), ("fp64_queries", ctypes.c_int64),
                ("exact_queries", ctypes.c_int64), ("expansion_queries", ctypes.c_int64),
                ("fp32_pass_ms", ctypes.c_float), ("tma_reruns", ctypes.c_int32)]

    def as_dict(self):
        return {k: (float if k.endswith("_ms") else int)(getattr(self, k)) for k, _ in self._fields_}


class SizingStats(ctypes.Structure):
    _fields_ = [("binned_pairs", ctypes.c_int64), ("global_tets", ctypes.c_int64),
                ("far_tets", ctypes.c_int64),
                ("inside", ctypes.c_int64), ("nearest", ctypes.c_int64), ("slow", ctypes.c_int64),
                ("tests", ctypes.c_int64), ("candidates", ctypes.c_int64),
                ("upload_ms", ctypes.c_float), ("eval_ms", ctypes.c_float),
                ("download_ms", ctypes.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def library_path() -> str:
    return os.environ.get("CMG_C_LIB") or IN_TREE


def _bind(lib: ctypes.CDLL) -> None:
    V, I, D, S, Z = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_size_t

    def sig(name, res, args):
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args

    # reference surface (bindings/python/src/cybermesh/__init__.py:58-159)
    sig("cmg_plc_create", V, [])
    sig("cmg_plc_destroy", None, [V])
    sig("cmg_options_create", V, [])
    sig("cmg_options_destroy", None, [V])
    sig("cmg_mesh_destroy", None, [V])
    sig("cmg_plc_set_points", I, [V, c_double_p, Z])
    sig("cmg_plc_add_facet", I, [V, c_int_p, Z, I])
    sig("cmg_plc_add_triangles", I, [V, c_int_p, Z, I])
    sig("cmg_plc_from_stl", I, [V, Z, ctypes.POINTER(V), S, Z])
    sig("cmg_plc_self_intersections", I, [V, ctypes.POINTER(V), S, Z])
    sig("cmg_intersections_count", ctypes.c_int64, [V])
    sig("cmg_intersections_data", c_int_p, [V])
    sig("cmg_intersections_destroy", None, [V])
    sig("cmg_self_intersections_last_ms", ctypes.c_float, [])
    sig("cmg_sizing_create", I, [c_double_p, ctypes.c_int64, c_int_p, ctypes.c_int64, c_double_p,
                                 ctypes.c_int64, D, ctypes.POINTER(V), S, Z])
    sig("cmg_sizing_eval", I, [V, c_double_p, ctypes.c_int64, c_double_p, c_int_p, S, Z])
    sig("cmg_sizing_eval_device", I, [V, V, ctypes.c_int64, V, V, V, S, Z])
    sig("cmg_sizing_get_stats", I, [V, ctypes.POINTER(SizingStats)])
    sig("cmg_sizing_destroy", None, [V])
    F = ctypes.POINTER(ctypes.c_float)
    sig("cmg_stl_last_timing", I, [F, F, F])
    sig("cmg_simplify_last_timing", I, [F, F, F])
    sig("cmg_plc_add_hole", I, [V, D, D, D])
    sig("cmg_plc_add_region", I, [V, D, D, D, D, D])
    sig("cmg_options_set_plc", I, [V, I])
    sig("cmg_options_set_max_volume", I, [V, D])
    sig("cmg_options_set_quality", I, [V, D, D])
    sig("cmg_options_set_preserve_edges", I, [V, I])
    sig("cmg_options_from_switches", I, [V, S, S, Z])
    sig("cmg_tetrahedralize", I, [V, V, c_void_pp, S, Z])
    sig("cmg_delaunay", I, [c_double_p, Z, V, c_void_pp, S, Z])
    for n in ("cmg_mesh_num_points", "cmg_mesh_num_tets", "cmg_mesh_num_faces"):
        sig(n, Z, [V])
    sig("cmg_mesh_points", c_double_p, [V])
    sig("cmg_mesh_tets", c_int_p, [V])
    sig("cmg_mesh_faces", c_int_p, [V])
    sig("cmg_mesh_tet_markers", c_int_p, [V])
    sig("cmg_mesh_face_markers", c_int_p, [V])
    for n in ("cmg_read_plc", "cmg_read_points", "cmg_read_mesh"):
        sig(n, I, [S, c_void_pp, S, Z])
    sig("cmg_write_mesh", I, [S, V, S, Z])
    sig("cmg_write_plc", I, [S, V, S, Z])
    sig("cmg_plc_num_points", Z, [V])
    sig("cmg_plc_points", c_double_p, [V])
    sig("cmg_plc_num_triangles", Z, [V])
    sig("cmg_plc_triangles", c_int_p, [V])
    sig("cmg_plc_simplify", I, [V, I, c_void_pp, S, Z])
    sig("cmg_plc_voxelize", I, [V, I, I, I, c_void_pp, S, Z])
    sig("cmg_voxels_destroy", None, [V])
    sig("cmg_voxels_dims", None, [V, c_int_p, c_int_p, c_int_p])
    sig("cmg_voxels_origin", None, [V, c_double_p, c_double_p, c_double_p])
    sig("cmg_voxels_spacing", D, [V])
    sig("cmg_voxels_occupancy", c_ubyte_p, [V])
    sig("cmg_voxels_distance", c_float_p, [V])
    sig("cmg_version", S, [])
    # GPU additions (include/cmg_c/cmg_gpu.h)
    sig("cmg_voxel_opts_init", None, [ctypes.POINTER(VoxelOpts)])
    sig("cmg_plc_voxelize_ex", I, [V, ctypes.POINTER(VoxelOpts), c_void_pp, S, Z])
    sig("cmg_voxels_distance_f64", c_double_p, [V])
    sig("cmg_voxels_nearest_triangle", c_int_p, [V])
    sig("cmg_voxels_nearest_region", c_ubyte_p, [V])
    sig("cmg_voxels_error_bound", c_float_p, [V])
    sig("cmg_voxels_corner", None, [V, c_double_p, c_double_p, c_double_p])
    sig("cmg_voxels_layers", None, [V, c_int_p, c_int_p, c_int_p])
    sig("cmg_plc_grid", I, [V, I, I, c_double_p, c_double_p, c_int_p, S, Z])
    sig("cmg_debug_fail_device_allocs", I, [I, I])
    sig("cmg_debug_fail_pred_wait", I, [ctypes.c_int64])
    sig("cmg_voxels_stats", None, [V, ctypes.POINTER(VoxelStats)])
    sig("cmg_batch_create", I, [ctypes.POINTER(V), c_int_p, c_int_p, I,
                                ctypes.POINTER(VoxelOpts), c_void_pp, S, Z])
    sig("cmg_batch_run", I, [V, I, S, Z])
    sig("cmg_batch_sync", I, [V, S, Z])
    sig("cmg_batch_get", I, [V, I, c_void_pp, S, Z])
    sig("cmg_batch_size", I, [V])
    sig("cmg_batch_cells", ctypes.c_int64, [V])
    sig("cmg_batch_destroy", None, [V])
    sig("cmg_gpu_version", S, [])
    sig("cmg_batch_stream", V, [V])
    sig("cmg_batch_set_timing", I, [V, I])
    sig("cmg_batch_get_timing", I, [V, ctypes.POINTER(BatchTiming), S, Z])
    sig("cmg_batch_work_model", I, [V, ctypes.POINTER(WorkModel), S, Z])
    sig("cmg_batch_stats", I, [V, ctypes.POINTER(VoxelStats), S, Z])
    sig("cmg_gpu_launches", ctypes.c_longlong, [])
    sig("cmg_gpu_peak_flops", I, [I, c_double_p, S, Z])
    for n in ("cmg_orient3d_stream", "cmg_insphere_stream"):
        sig(n, I, [ctypes.POINTER(V), ctypes.c_int64, I, I, V, ctypes.POINTER(PredStats), V, S, Z])
    sig("cmg_orient3d_signs", I, [c_double_p, I, c_int_p, I, c_int_p])
    sig("cmg_orient3d_batch", I, [c_double_p, I, c_int_p, I, c_double_p])
    sig("cmg_host_alloc", V, [Z])
    sig("cmg_host_free", None, [V])
    sig("cmg_gpu_occupancy_static", I, [V, ctypes.c_int64, V, ctypes.c_int64, c_double_p, D,
                                        c_int_p, I, V, V, S, Z])
    # differentiable signed distance
    sig("cmg_sdf_plan_create", I, [c_double_p, ctypes.c_int64, c_int_p, ctypes.c_int64, V,
                                   ctypes.POINTER(V), S, Z])
    sig("cmg_sdf_plan_forward", I, [V, V, V, S, Z])
    sig("cmg_sdf_plan_outputs", I, [V, ctypes.POINTER(V), ctypes.POINTER(V), ctypes.POINTER(V),
                                    ctypes.POINTER(V)])
    sig("cmg_sdf_plan_cells", ctypes.c_int64, [V])
    sig("cmg_sdf_plan_copy_outputs", I, [V, V, V, V, V, V, S, Z])
    sig("cmg_sdf_plan_backward", I, [V, V, V, V, V, V, V, V, S, Z])
    sig("cmg_sdf_plan_destroy", None, [V])


_LIB = None


class Lazy:
    """Attribute access loads and binds the library on first use, so that the
    package (and its build and workload modules) import without it; a call then
    fails loudly if the library is missing."""

    def __getattr__(self, name):
        return getattr(load(), name)


def load() -> ctypes.CDLL:
    """The bound library (loaded once)."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise ImportError(
                f"libcmg_c.so not found at {path}; build it with "
                "`python -m cybermeshgenerator_gb300.build` (or set CMG_C_LIB)")
        lib = ctypes.CDLL(path)
        _bind(lib)
        _LIB = lib
    return _LIB
