"""ctypes binding of libmcgpu.so (include/mcgpu.h).

The library is built in-tree by model3d_gb300/build.py.  There is no
fallback: if the library is missing or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmcgpu.so")

# mc_status values (include/mcgpu.h)
MC_OK = 0
MC_ERR_INVALID_BOUNDS = 1
MC_ERR_BOUNDS_INSIDE = 2
MC_ERR_NOT_ON_EDGE = 3
MC_ERR_EDGE_INDEX = 4
MC_ERR_BAD_PROGRAM = 5
MC_ERR_NOT_LOWERABLE = 6
MC_ERR_OOM = 7
MC_ERR_TIMEOUT = 8
MC_ERR_CUDA = 9
MC_ERR_ARG = 10
MC_ERR_GRID = 11
MC_ERR_LIMIT = 12

MC_PREC_FP64 = 0
MC_PREC_FP32_FILTERED = 1

EXPORTS = [
    "mc_status_string", "mc_last_error", "mc_create", "mc_destroy", "mc_solid_create",
    "mc_solid_destroy", "mc_solid_bounds", "mc_spacer_axis", "mc_search", "mc_mesh_free",
    "mc_search_device", "mc_result_device", "mc_result_copy", "mc_contains", "mc_search_batch",
    "mc_case_table", "mc_version", "mc_search_noalloc", "mc_autotune",
    "mc_measure_peaks", "mc_result_interior_copy", "mc_result_transform", "mc_result_stl",
    "mc_program_check", "mc_result_keys", "mc_result_group", "mc_result_stl_grouped", "mc_mesh_group",
    "mc_mesh_stl_grouped",
]


class MCProgramInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "n_ops", "n_leaves", "n_metaballs", "n_balls", "n_boxes", "n_colliders", "max_stack")] + [
        ("threshold", ctypes.c_double), ("root_min", ctypes.c_double * 3), ("root_max", ctypes.c_double * 3),
        ("digest", ctypes.c_uint64)]


class MCStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "nx", "ny", "nz", "corners", "vertices", "triangles", "leaf_evals", "escalations",
        "tiles", "tiles_const", "bvh_nodes", "bvh_tris")] + [
        (n, ctypes.c_double) for n in ("ms_classify", "ms_count", "ms_emit", "ms_search",
                                       "ms_total")] + [
        (n, ctypes.c_int64) for n in ("h2d_bytes", "d2h_bytes", "flops_classify", "flops_search")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class MCMesh(ctypes.Structure):
    _fields_ = [("vertices", ctypes.POINTER(ctypes.c_double)),
                ("triangles", ctypes.POINTER(ctypes.c_int32)),
                ("n_vertices", ctypes.c_int64), ("n_triangles", ctypes.c_int64),
                ("stats", MCStats)]


class MCOpts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("cull", ctypes.c_int32),
                ("tile_y", ctypes.c_int32), ("tile_z", ctypes.c_int32),
                ("interior", ctypes.c_int32), ("z_begin", ctypes.c_int32), ("z_end", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class MCTriSet(ctypes.Structure):
    _fields_ = [("tris", ctypes.c_void_p), ("n", ctypes.c_int64),
                ("grouped", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class MCJob(ctypes.Structure):
    _fields_ = [("solid", ctypes.c_void_p), ("delta", ctypes.c_double),
                ("iters", ctypes.c_int32), ("reserved", ctypes.c_int32)]


_lib = None
_lock = threading.Lock()


def lib():
    """Load libmcgpu.so (building it first if the sources are newer)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        from . import build as _build
        if not _build.up_to_date():
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libmcgpu.so missing at {LIB_PATH}; run model3d_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
        L.mc_status_string.restype = ctypes.c_char_p
        L.mc_status_string.argtypes = [ctypes.c_int]
        L.mc_last_error.restype = ctypes.c_char_p
        L.mc_last_error.argtypes = [vp]
        L.mc_version.restype = ctypes.c_char_p
        L.mc_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int]
        L.mc_destroy.argtypes = [vp]
        L.mc_destroy.restype = None
        L.mc_solid_create.argtypes = [vp, vp, ctypes.c_size_t, vp, ctypes.c_size_t, ctypes.POINTER(vp)]
        L.mc_solid_destroy.argtypes = [vp]
        L.mc_solid_destroy.restype = None
        L.mc_solid_bounds.argtypes = [vp, vp, vp]
        L.mc_spacer_axis.argtypes = [dbl, dbl, dbl, vp, i64, ctypes.POINTER(i64)]
        L.mc_search.argtypes = [vp, vp, dbl, i32, ctypes.POINTER(MCOpts), ctypes.POINTER(MCMesh)]
        L.mc_mesh_free.argtypes = [ctypes.POINTER(MCMesh)]
        L.mc_mesh_free.restype = None
        L.mc_search_device.argtypes = [vp, vp, dbl, i32, ctypes.POINTER(MCOpts),
                                       ctypes.POINTER(i64), ctypes.POINTER(i64),
                                       ctypes.POINTER(MCStats)]
        L.mc_result_device.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        L.mc_result_copy.argtypes = [vp, vp, vp]
        L.mc_result_interior_copy.argtypes = [vp, vp]
        L.mc_result_keys.argtypes = [vp, vp]
        L.mc_result_transform.argtypes = [vp, vp, ctypes.c_size_t, i32]
        L.mc_result_stl.argtypes = [vp, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        L.mc_result_group.argtypes = [vp, vp]
        L.mc_result_stl_grouped.argtypes = [vp, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        L.mc_mesh_group.argtypes = [vp, vp, i64, vp, i64, vp]
        L.mc_mesh_stl_grouped.argtypes = [vp, vp, i64, vp, i64, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        L.mc_contains.argtypes = [vp, vp, vp, i64, ctypes.POINTER(MCOpts), vp]
        L.mc_search_batch.argtypes = [vp, ctypes.POINTER(MCJob), ctypes.c_size_t,
                                      ctypes.POINTER(MCOpts), ctypes.POINTER(MCMesh), vp]
        L.mc_case_table.argtypes = [vp, vp]
        L.mc_measure_peaks.argtypes = [vp, ctypes.POINTER(dbl), ctypes.POINTER(dbl), ctypes.POINTER(dbl)]
        L.mc_program_check.argtypes = [vp, ctypes.c_size_t, vp, ctypes.c_size_t, ctypes.POINTER(MCProgramInfo),
                                       ctypes.c_char_p, ctypes.c_size_t]
        L.mc_autotune.argtypes = [vp, vp, dbl, i32, ctypes.POINTER(MCOpts), ctypes.POINTER(MCOpts),
                                  ctypes.POINTER(dbl)]
        L.mc_search_noalloc.argtypes = [vp, ctypes.c_size_t, dbl, i32, ctypes.POINTER(MCOpts), vp,
                                        vp, i64, vp, i64, ctypes.POINTER(i64), ctypes.POINTER(i64)]
        for name in EXPORTS:
            getattr(L, name)  # every declared entry point must be exported
        _lib = L
        return L


def status_string(status: int) -> str:
    return lib().mc_status_string(status).decode()
