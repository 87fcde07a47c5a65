"""ctypes declarations for libwolkenbase_gb300.so (include/wolkenbase_gb300.h).

The library is built in-tree by wolkenbase_gb300/_build.py.  There is no CPU
fallback: if the shared library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwolkenbase_gb300.so")

WB_OK, WB_EINVAL, WB_ENOMEM, WB_ECUDA, WB_EDEPTH, WB_ESTATE, WB_ETIMEDOUT, WB_ENOTFOUND = 0, -1, -2, -3, -4, -5, -6, -7
WB_EBUSY, WB_ECANCELED, WB_EIO = -8, -9, -10
ERROR_NAMES = {WB_EINVAL: "WB_EINVAL", WB_ENOMEM: "WB_ENOMEM", WB_ECUDA: "WB_ECUDA", WB_EDEPTH: "WB_EDEPTH",
               WB_ESTATE: "WB_ESTATE", WB_ETIMEDOUT: "WB_ETIMEDOUT", WB_ENOTFOUND: "WB_ENOTFOUND",
               WB_EBUSY: "WB_EBUSY", WB_ECANCELED: "WB_ECANCELED", WB_EIO: "WB_EIO"}

WB_FLUSH_EAGER, WB_FLUSH_FULL = 0, 1
WB_PRECISION_EXACT, WB_PRECISION_FP32 = 0, 1
(WB_JOB_QUEUED, WB_JOB_PREP, WB_JOB_READY, WB_JOB_CLASSIFY, WB_JOB_DONE, WB_JOB_FAILED,
 WB_JOB_CANCELLED) = range(7)


class wb_params(C.Structure):
    _fields_ = [("tile_size", C.c_double), ("max_slope", C.c_double), ("thickness", C.c_double),
                ("min_hyp_size", C.c_double)]


class wb_cloud(C.Structure):
    _fields_ = [("records", C.c_void_p), ("n", C.c_uint64), ("stride", C.c_uint32),
                ("device_resident", C.c_uint32), ("scale", C.c_double * 3), ("offset", C.c_double * 3),
                ("unit", C.c_double), ("minc", C.c_double * 3), ("maxc", C.c_double * 3)]


class wb_octree_stats(C.Structure):
    _fields_ = [("n_points", C.c_uint64), ("n_distinct", C.c_uint64), ("n_leaves", C.c_uint64),
                ("max_depth", C.c_uint32), ("pad", C.c_uint32), ("root_center", C.c_double * 3),
                ("root_side", C.c_double), ("tile_center", C.c_double * 3), ("tile_side", C.c_double),
                ("spacing", C.c_double), ("n_tiles", C.c_uint64), ("tile_lo", C.c_int32), ("tile_hi", C.c_int32)]


class wb_tile(C.Structure):
    _fields_ = [("ex", C.c_int32), ("ey", C.c_int32), ("n_points", C.c_int32), ("n_ground", C.c_int32),
                ("tree_flags", C.c_int32), ("pad", C.c_int32), ("density", C.c_double), ("h_scan", C.c_double),
                ("hyperboloid_size", C.c_double), ("height", C.c_double)]


WB_N_SHAPES = 8
WB_SHAPE_CYLINDER, WB_SHAPE_HYPERBOLOID = 1, 2


class wb_shape(C.Structure):
    _fields_ = [("kind", C.c_int), ("pad", C.c_int), ("v", C.c_double * 3), ("r", C.c_double), ("s", C.c_double)]


class wb_tuning(C.Structure):
    _fields_ = [("shape", C.c_int), ("chunk", C.c_int), ("grid_points", C.c_double)]


class wb_server_config(C.Structure):
    _fields_ = [("device", C.c_int), ("prep_slots", C.c_int), ("hbm_budget", C.c_uint64), ("flush", C.c_int),
                ("max_batch", C.c_int), ("shape", C.c_int), ("chunk", C.c_int), ("grid_points", C.c_double),
                ("autotune", C.c_int), ("pad", C.c_int), ("host_budget", C.c_uint64)]


class wb_job(C.Structure):
    _fields_ = [("cloud", wb_cloud), ("params", wb_params), ("cls", C.c_void_p), ("tag", C.c_uint64)]


class wb_job_status(C.Structure):
    _fields_ = [("state", C.c_int), ("rc", C.c_int), ("tag", C.c_uint64), ("n_points", C.c_uint64),
                ("n_ground", C.c_uint64), ("n_ambiguous", C.c_uint64), ("reserved_bytes", C.c_uint64),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_ready", C.c_double),
                ("t_done", C.c_double), ("batch_jobs", C.c_int), ("pad", C.c_int)]


class wb_server_stats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("cancelled", C.c_uint64), ("points", C.c_uint64), ("fused_launches", C.c_uint64),
                ("fused_jobs", C.c_uint64), ("held_bytes", C.c_uint64), ("peak_bytes", C.c_uint64),
                ("budget", C.c_uint64), ("kernel_launches", C.c_uint64), ("contexts", C.c_int),
                ("queued", C.c_int), ("running", C.c_int), ("pad", C.c_int), ("now", C.c_double),
                ("tuned", C.c_int), ("shape", C.c_int), ("chunk", C.c_int), ("pad2", C.c_int),
                ("grid_points", C.c_double), ("tune_ms", C.c_double)]


LAS_POINT_FIELDS = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("intensity", C.c_uint16),
                    ("return_num", C.c_uint16), ("n_returns", C.c_uint16), ("scan_direction", C.c_uint8),
                    ("edge_line", C.c_uint8), ("classification", C.c_uint16), ("class_flags", C.c_uint16),
                    ("scanner_channel", C.c_uint16), ("user_data", C.c_uint16), ("scan_angle", C.c_int32),
                    ("point_source", C.c_uint16), ("gps_time", C.c_double), ("red", C.c_uint16),
                    ("green", C.c_uint16), ("blue", C.c_uint16), ("nir", C.c_uint16)]


class wb_las_points(C.Structure):
    _fields_ = [(name, C.c_void_p) for name, _ in LAS_POINT_FIELDS]


class wb_las_output(C.Structure):
    _fields_ = [("point_format", C.c_int32), ("separate_classes", C.c_int32), ("n_input_files", C.c_int32),
                ("creation_day", C.c_int32), ("creation_year", C.c_int32), ("pad", C.c_int32),
                ("points_per_file", C.c_uint64), ("unit", C.c_double), ("min_cor", C.c_double * 3),
                ("max_cor", C.c_double * 3), ("scale", C.c_double * 3), ("software", C.c_char_p)]


class wb_las_file(C.Structure):
    _fields_ = [("class_id", C.c_int32), ("index", C.c_int32), ("name_digits", C.c_int32),
                ("point_format", C.c_int32), ("first", C.c_uint64), ("n_points", C.c_uint64 * 16),
                ("scale", C.c_double * 3), ("offset", C.c_double * 3), ("min", C.c_double * 3),
                ("max", C.c_double * 3)]


# name -> (restype, argtypes); every symbol include/wolkenbase_gb300.h declares
SIGNATURES = {
    "wb_open": (C.c_void_p, [C.c_int, C.c_size_t]),
    "wb_close": (None, [C.c_void_p]),
    "wb_last_error": (C.c_char_p, [C.c_void_p]),
    "wb_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wb_synchronize": (C.c_int, [C.c_void_p]),
    "wb_set_paging": (C.c_int, [C.c_void_p, C.c_size_t]),
    "wb_paging_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "wb_octree_build": (C.c_int, [C.c_void_p, C.POINTER(wb_cloud)]),
    "wb_octree_info": (C.c_int, [C.c_void_p, C.POINTER(wb_octree_stats)]),
    "wb_octree_leaves": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "wb_octree_point_leaf": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wb_octree_store_order": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wb_octree_find_block": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "wb_octree_find_block_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "wb_classify_ex": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "wb_find_blocks": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "wb_points_in": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_uint64, C.c_void_p]),
    "wb_scan_tiles": (C.c_int, [C.c_void_p, C.POINTER(wb_params)]),
    "wb_tiles": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "wb_classify": (C.c_int, [C.c_void_p, C.POINTER(wb_params), C.c_void_p, C.c_int]),
    "wb_classify_cloud": (C.c_int, [C.c_void_p, C.POINTER(wb_cloud), C.POINTER(wb_params), C.c_void_p]),
    "wb_stage_times": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)]),
    "wb_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "wb_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "wb_check_atan2i": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p]),
    "wb_check_hypot": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p]),
    "wb_check_dir_f32": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_uint64, C.c_void_p]),
    "wb_check_hyperboloid": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_uint64, C.c_void_p]),
    "wb_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(wb_tuning)]),
    "wb_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(wb_tuning)]),
    "wb_autotune": (C.c_int, [C.c_void_p, C.POINTER(wb_params)]),
    "wb_set_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "wb_tile_planes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "wb_tile_residuals": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "wb_class_totals": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wb_duplicates": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_void_p]),
    "wb_las_write_classes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_int, C.c_int, C.c_void_p]),
    "wb_las_split_by_class": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_int, C.c_int, C.c_void_p,
                                        C.c_void_p]),
    "wb_preview": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                             C.c_void_p]),
    "wb_las_point_length": (C.c_int, [C.c_int]),
    "wb_las_decode": (C.c_int, [C.c_void_p, C.POINTER(wb_cloud), C.c_int, C.POINTER(wb_las_points)]),
    "wb_las_join_point_format": (C.c_int, [C.c_void_p, C.c_int]),
    "wb_las_combine_scales": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "wb_las_write_output": (C.c_int, [C.c_void_p, C.POINTER(wb_cloud), C.c_int, C.c_void_p, C.POINTER(wb_las_output),
                                      C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "wb_las_header_bytes": (C.c_int, [C.POINTER(wb_las_output), C.POINTER(wb_las_file), C.c_void_p]),
    "wb_las_file_name": (C.c_int, [C.POINTER(wb_las_output), C.POINTER(wb_las_file), C.c_char_p, C.c_char_p,
                                   C.c_size_t]),
    "wb_las_write_files": (C.c_int, [C.c_void_p, C.POINTER(wb_cloud), C.c_int, C.c_void_p, C.POINTER(wb_las_output),
                                     C.c_char_p, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "wb_server_open": (C.c_void_p, [C.POINTER(wb_server_config)]),
    "wb_server_close": (None, [C.c_void_p]),
    "wb_server_error": (C.c_char_p, [C.c_void_p]),
    "wb_submit": (C.c_int64, [C.c_void_p, C.POINTER(wb_job)]),
    "wb_poll": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(wb_job_status)]),
    "wb_wait": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.POINTER(wb_job_status)]),
    "wb_cancel": (C.c_int, [C.c_void_p, C.c_int64]),
    "wb_release": (C.c_int, [C.c_void_p, C.c_int64]),
    "wb_server_stats_get": (C.c_int, [C.c_void_p, C.POINTER(wb_server_stats)]),
    "wb_classify_batch": (C.c_int, [C.c_void_p, C.POINTER(wb_job), C.c_int, C.c_void_p]),
}

_lib = None


def load():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run wolkenbase_gb300/_build.py (nvcc, sm_103a) first; "
                              "there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib
