"""ctypes binding of include/analyticmesh_gb300.h (libamgb300.so).

The library is built in-tree by ``analyticmesh_gb300.build``.  There is no
fallback: if the library is missing or fails to load, every entry point
raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_LIB = None


class AmStats(C.Structure):
    _fields_ = [
        ("num_regions", C.c_int64), ("num_faces", C.c_int64), ("num_seeds", C.c_int64),
        ("num_nostart", C.c_int64), ("num_open", C.c_int64), ("num_truncated", C.c_int64),
        ("num_singular", C.c_int64), ("mesh_num_verts", C.c_int64), ("mesh_num_faces", C.c_int64),
        ("mesh_num_indices", C.c_int64), ("chunks", C.c_int32), ("max_polygon_verts", C.c_int32),
        ("am_time_ms", C.c_double), ("compose_ms", C.c_double), ("polygon_ms", C.c_double),
        ("frontier_ms", C.c_double), ("kernel_launches", C.c_int64),
        ("max_abs_f", C.c_double), ("max_vertex_err", C.c_double), ("error_faces", C.c_int64),
        ("num_fp64_walks", C.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AmErrorReport(C.Structure):
    """am_error_report_t: max |f(v)| and vertex error of a result against FP64."""
    _fields_ = [("faces", C.c_int64), ("vertices", C.c_int64), ("vertices_singular", C.c_int64),
                ("max_abs_f", C.c_double), ("max_vertex_err", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AmRunArgs(C.Structure):
    """am_run_args: the arguments of am_analytic_marching for one network of a batch."""
    _fields_ = [
        ("weights", C.c_void_p), ("biases", C.c_void_p), ("states", C.c_void_p), ("points", C.c_void_p),
        ("num_points", C.c_int), ("arc_tm", C.c_void_p), ("arc_tm_shapes", C.c_void_p), ("num_arc_tm", C.c_int),
        ("w_extra", C.c_void_p), ("b_extra", C.c_void_p), ("iso", C.c_double), ("flip_insideout", C.c_int),
    ]


AM_OPT_CHUNK = 1
AM_OPT_PHASE_TIMING = 2
AM_OPT_WELD = 3
AM_OPT_GRAPH = 4
AM_OPT_MAX_REGIONS = 5
AM_OPT_COMPOSE_TILE = 6
AM_OPT_FACE_WARPS = 7
AM_OPT_TABLE_SLOTS = 8
AM_OPT_INJECT_ERROR = 9
AM_OPT_PRUNE_ROWS = 10

# device error bits (AM_OPT_INJECT_ERROR)
ERR_TABLE_FULL, ERR_WAIT, ERR_CAPACITY, ERR_NONFINITE = 1, 2, 4, 8

# status codes (am_status)
AM_OK, AM_ERR_INVALID_ARGUMENT, AM_ERR_NOT_INITIALIZED, AM_ERR_CUDA, AM_ERR_OUT_OF_MEMORY = 0, 1, 2, 3, 4
AM_ERR_TABLE_FULL, AM_ERR_NO_RESULT, AM_ERR_IO, AM_ERR_CAPACITY = 5, 6, 7, 8


class AmError(RuntimeError):
    """A failed call; ``status`` is the am_status code."""

    def __init__(self, msg, status=None):
        super().__init__(msg)
        self.status = status


def lib():
    """Load libamgb300.so (building it when the sources are newer)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path) or os.environ.get("AM_REBUILD"):
        path = _build.build()
    L = C.CDLL(path)
    vp, i32p = C.c_void_p, C.POINTER(C.c_int32)
    L.am_init.argtypes = [C.POINTER(vp), C.c_char_p, i32p, C.c_int, i32p, C.c_int, C.c_int, C.c_int]
    L.am_analytic_marching.argtypes = [vp, vp, vp, vp, vp, C.c_int, vp, i32p, C.c_int, vp, vp, C.c_double, C.c_int, vp]
    L.am_combine_mesh.argtypes = [vp, C.c_double, C.POINTER(C.c_double)]
    L.am_export_mesh.argtypes = [vp, C.c_char_p, C.c_int, C.c_int]
    L.am_destroy.argtypes = [vp]
    L.am_strerror.restype = C.c_char_p
    L.am_strerror.argtypes = [C.c_int]
    L.am_last_error.restype = C.c_char_p
    L.am_last_error.argtypes = [vp]
    L.am_get_stats.argtypes = [vp, C.POINTER(AmStats)]
    L.am_get_mesh.argtypes = [vp, vp, vp, vp]
    L.am_get_regions.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    L.am_set_option.argtypes = [vp, C.c_int, C.c_int64]
    L.am_region_rows.argtypes = [vp, C.c_int64, C.c_int, vp, vp]
    L.am_run_batch.argtypes = [vp, C.POINTER(AmRunArgs), C.c_int, C.POINTER(C.c_double)]
    L.am_compose_rows_noalloc.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int, C.c_double, vp, vp, vp]
    L.am_autotune.argtypes = [vp, C.POINTER(AmRunArgs), C.c_int64, C.POINTER(C.c_int32)]
    L.am_error_report.argtypes = [vp, C.c_int64, C.POINTER(AmErrorReport)]
    _LIB = L
    return L


def check(rc: int, handle=None):
    if rc != 0:
        L = lib()
        detail = L.am_last_error(handle).decode() if handle else ""
        raise AmError("%s%s" % (L.am_strerror(rc).decode(), (": " + detail) if detail else ""), rc)


def vert_capacity() -> int:
    return lib().am_vert_capacity()
