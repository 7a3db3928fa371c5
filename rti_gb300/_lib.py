"""ctypes bindings of librtg.so (the C ABI in include/rtg.h).

The library is loaded from this package directory only; there is no fallback.
If it is missing, build it with ``python -m rti_gb300.build`` (nvcc, sm_103a).
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librtg.so")

RTG_OK = 0
RTG_ERR_INVALID_ARGUMENT = 1
RTG_ERR_CUDA = 2
RTG_ERR_OUT_OF_MEMORY = 3
RTG_ERR_NO_GEOMETRY = 4
RTG_ERR_BUDGET = 5
RTG_ERR_ABORTED = 6
RTG_ERR_INTERNAL = 7

RTG_BOUND_REFLECTIVE = 0
RTG_BOUND_PERIODIC = 1
RTG_REFLECT_DIFFUSE = 0
RTG_REFLECT_SPECULAR = 1
RTG_REFLECT_MIXED = 2
RTG_BOX_FROM_GEOMETRY = 0
RTG_BOX_EXPLICIT = 1

# every function include/rtg.h declares (checked by the tests)
EXPORTS = [
    "rtg_config_default", "rtg_abi_version", "rtg_create", "rtg_destroy", "rtg_last_error",
    "rtg_upload_discs", "rtg_upload_triangles", "rtg_upload_mixed", "rtg_update_discs", "rtg_update_vertices",
    "rtg_set_config", "rtg_get_config", "rtg_get_box", "rtg_set_sticking", "rtg_set_sticking_field",
    "rtg_trace", "rtg_trace_range", "rtg_synchronize", "rtg_request_abort", "rtg_trace_rays",
    "rtg_num_primitives", "rtg_get_mc_estimates", "rtg_get_hit_counts", "rtg_get_accumulators",
    "rtg_get_exposed_areas", "rtg_get_relative_error", "rtg_get_vov", "rtg_get_tally", "rtg_set_accumulators",
    "rtg_get_neighbors", "rtg_get_device_view", "rtg_device_run", "rtg_get_mc_estimates_noalloc",
    "rtg_set_sticking_field_device", "rtg_adjoint", "rtg_adjoint_host",
    "rtg_batch_create", "rtg_batch_destroy", "rtg_batch_last_error", "rtg_batch_add", "rtg_batch_num_jobs",
    "rtg_batch_run", "rtg_batch_run_sequential", "rtg_batch_synchronize", "rtg_batch_get_results",
    "rtg_batch_get_tally", "rtg_launch_config_default", "rtg_set_launch_config", "rtg_get_launch_config",
    "rtg_get_tree_depth", "rtg_autotune", "rtg_batch_set_launch_config", "rtg_batch_get_launch_config",
    "rtg_batch_autotune", "rtg_write_vtp", "rtg_write_vtp_discs", "rtg_write_vtp_triangles", "rtg_write_vtp_mixed",
    "rtg_read_point_cloud", "rtg_read_triangles", "rtg_set_tree_builder", "rtg_get_tree_builder",
    "rtg_set_deposit_mode", "rtg_get_deposit_mode", "rtg_set_accumulation", "rtg_get_accumulation",
    "rtg_set_visit_limit", "rtg_get_visit_limit", "rtg_inject_alloc_failure", "rtg_set_node_width",
    "rtg_get_node_width", "rtg_get_traversal_width", "rtg_set_segment_log", "rtg_get_segment_log",
    "rtg_write_segment_log_vtp", "rtg_write_vtp_segments", "rtg_read_point_cloud_vtu", "rtg_read_triangles_vtu",
]

RTG_ADJ_HELD = 0
RTG_ADJ_UNBIASED = 1
RTG_SCHED_MEGAKERNEL = 0
RTG_SCHED_WAVEFRONT = 1
RTG_SCHED_PLAIN = 2
RTG_TREE_KARRAS = 0
RTG_LEAF_IMMEDIATE = 0
RTG_LEAF_POSTPONED = 1
RTG_TREE_PLOC = 1
RTG_STACK_AUTO = 0
RTG_STACK_LOCAL = 1
RTG_STACK_SHARED = 2
RTG_ACCUM_FP64 = 0
RTG_ACCUM_FIXED = 1
RTG_DEPOSIT_NEIGHBORS = 0
RTG_DEPOSIT_WINDOW = 1
RTG_VTU_AREA = 1
RTG_VTU_SPACING = 2
RTG_NODES_AUTO = 0
RTG_NODES_BINARY = 2
RTG_NODES_WIDE = 8


class RtgConfig(C.Structure):
    _fields_ = [
        ("x_bound", C.c_int32),
        ("y_bound", C.c_int32),
        ("reflection", C.c_int32),
        ("specular_fraction", C.c_float),
        ("sticking", C.c_float),
        ("source_exponent", C.c_float),
        ("box_mode", C.c_int32),
        ("box_lo", C.c_float * 3),
        ("box_hi", C.c_float * 3),
        ("tnear", C.c_float),
        ("roulette_threshold", C.c_double),
        ("roulette_weight", C.c_double),
        ("max_segments", C.c_uint32),
        ("job", C.c_uint32),
    ]


class RtgTally(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in
                ("num_rays", "hitc", "nonhitc", "total", "segments", "truncated", "nb_deposits", "errors")] + [
        ("trace_ms", C.c_double), ("kernel_ms", C.c_double)]


RTG_SEG_HIT = 0
RTG_SEG_BACKFACE = 1
RTG_SEG_BOUNDARY = 2
RTG_SEG_ESCAPE = 3


class RtgSegment(C.Structure):
    """One record of the segment log (rtg_segment)."""
    _fields_ = [("ray", C.c_uint64), ("segment", C.c_uint32), ("kind", C.c_int32), ("org", C.c_float * 3),
                ("end", C.c_float * 3), ("primitive", C.c_int32), ("weight", C.c_float)]


# numpy view of an array of RtgSegment (48 bytes each)
SEGMENT_DTYPE = [("ray", "<u8"), ("segment", "<u4"), ("kind", "<i4"), ("org", "<f4", (3,)), ("end", "<f4", (3,)),
                 ("primitive", "<i4"), ("weight", "<f4")]


class RtgDeviceView(C.Structure):
    _fields_ = [("s1", C.c_void_p), ("s2", C.c_void_p), ("s3", C.c_void_p), ("s4", C.c_void_p),
                ("counts", C.c_void_p), ("areas", C.c_void_p), ("estimates", C.c_void_p), ("n", C.c_int64)]


class RtgLaunchConfig(C.Structure):
    _fields_ = [("threads_per_block", C.c_int32), ("packet", C.c_int32), ("stack_depth", C.c_int32),
                ("scheduling", C.c_int32), ("leaf_tests", C.c_int32), ("stack_memory", C.c_int32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class RtgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"rtg error {code}: {msg}")
        self.code = code


_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_u64p = C.POINTER(C.c_uint64)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)
_ctx = C.c_void_p

_lib = None


def load(path: str | None = None):
    """Loads librtg.so; raises if it has not been built (there is no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"librtg.so not found at {p}; build it with `python -m rti_gb300.build`")
    L = C.CDLL(p)
    sig = {
        "rtg_config_default": (None, [C.POINTER(RtgConfig)]),
        "rtg_abi_version": (C.c_int, []),
        "rtg_create": (C.c_int, [C.POINTER(_ctx), C.c_int]),
        "rtg_destroy": (C.c_int, [_ctx]),
        "rtg_last_error": (C.c_char_p, [_ctx]),
        "rtg_upload_discs": (C.c_int, [_ctx, _f32p, _f32p, _f32p, C.c_int64]),
        "rtg_upload_triangles": (C.c_int, [_ctx, _f32p, _u32p, C.c_int64, C.c_int64]),
        "rtg_upload_mixed": (C.c_int, [_ctx, _f32p, _f32p, _f32p, C.c_int64, _f32p, _u32p, C.c_int64, C.c_int64]),
        "rtg_update_discs": (C.c_int, [_ctx, _f32p, _f32p, _f32p, C.c_int64]),
        "rtg_update_vertices": (C.c_int, [_ctx, _f32p, C.c_int64]),
        "rtg_set_config": (C.c_int, [_ctx, C.POINTER(RtgConfig)]),
        "rtg_get_config": (C.c_int, [_ctx, C.POINTER(RtgConfig)]),
        "rtg_get_box": (C.c_int, [_ctx, _f32p, _f32p]),
        "rtg_set_sticking": (C.c_int, [_ctx, C.c_float]),
        "rtg_set_sticking_field": (C.c_int, [_ctx, _f32p, C.c_int64]),
        "rtg_set_sticking_field_device": (C.c_int, [_ctx, C.c_void_p, C.c_int64, C.c_void_p]),
        "rtg_adjoint": (C.c_int, [_ctx, C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p,
                                  C.c_void_p, C.c_void_p]),
        "rtg_adjoint_host": (C.c_int, [_ctx, _f64p, C.c_uint64, C.c_uint64, C.c_int, _f64p, _f64p, _f64p]),
        "rtg_trace": (C.c_int, [_ctx, C.c_uint64, C.c_uint64, C.c_void_p]),
        "rtg_trace_range": (C.c_int, [_ctx, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]),
        "rtg_synchronize": (C.c_int, [_ctx]),
        "rtg_request_abort": (C.c_int, [_ctx]),
        "rtg_trace_rays": (C.c_int, [_ctx, _f32p, C.c_int64, C.c_float, _i32p, _f32p]),
        "rtg_num_primitives": (C.c_int, [_ctx, _i64p]),
        "rtg_get_mc_estimates": (C.c_int, [_ctx, _f32p]),
        "rtg_get_mc_estimates_noalloc": (C.c_int, [_ctx, C.c_void_p, C.c_void_p]),
        "rtg_get_hit_counts": (C.c_int, [_ctx, _u64p]),
        "rtg_get_accumulators": (C.c_int, [_ctx, _f64p, _f64p, _f64p, _f64p]),
        "rtg_get_exposed_areas": (C.c_int, [_ctx, _f32p]),
        "rtg_get_relative_error": (C.c_int, [_ctx, _f64p]),
        "rtg_get_vov": (C.c_int, [_ctx, _f64p]),
        "rtg_get_tally": (C.c_int, [_ctx, C.POINTER(RtgTally)]),
        "rtg_set_accumulators": (C.c_int, [_ctx, _f64p, _f64p, _f64p, _f64p, _u64p, C.POINTER(RtgTally)]),
        "rtg_get_neighbors": (C.c_int, [_ctx, _i64p, _i32p, C.c_int64, _i64p]),
        "rtg_get_device_view": (C.c_int, [_ctx, C.POINTER(RtgDeviceView)]),
        "rtg_device_run": (C.c_int, [_f32p, _f32p, _f32p, C.c_int64, C.POINTER(RtgConfig), _f32p, C.c_uint64,
                                     C.c_uint64, _f32p, _u64p, C.c_int]),
        "rtg_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
        "rtg_batch_destroy": (C.c_int, [C.c_void_p]),
        "rtg_batch_last_error": (C.c_char_p, [C.c_void_p]),
        "rtg_batch_add": (C.c_int, [C.c_void_p, _ctx, C.POINTER(RtgConfig), C.c_uint64, C.c_uint64, _i32p]),
        "rtg_batch_num_jobs": (C.c_int, [C.c_void_p, _i32p]),
        "rtg_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
        "rtg_batch_run_sequential": (C.c_int, [C.c_void_p, C.c_void_p]),
        "rtg_batch_synchronize": (C.c_int, [C.c_void_p, _f64p]),
        "rtg_batch_get_results": (C.c_int, [C.c_void_p, C.c_int32, _f64p, _u64p, _f32p]),
        "rtg_batch_get_tally": (C.c_int, [C.c_void_p, C.POINTER(RtgTally)]),
        "rtg_launch_config_default": (None, [C.POINTER(RtgLaunchConfig)]),
        "rtg_set_launch_config": (C.c_int, [_ctx, C.POINTER(RtgLaunchConfig)]),
        "rtg_get_launch_config": (C.c_int, [_ctx, C.POINTER(RtgLaunchConfig)]),
        "rtg_get_tree_depth": (C.c_int, [_ctx, _i32p]),
        "rtg_autotune": (C.c_int, [_ctx, C.c_uint64, C.c_uint64, C.POINTER(RtgLaunchConfig), _f64p]),
        "rtg_batch_set_launch_config": (C.c_int, [C.c_void_p, C.POINTER(RtgLaunchConfig)]),
        "rtg_batch_get_launch_config": (C.c_int, [C.c_void_p, C.POINTER(RtgLaunchConfig)]),
        "rtg_batch_autotune": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(RtgLaunchConfig), _f64p]),
        "rtg_write_vtp": (C.c_int, [_ctx, C.c_char_p, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_int32]),
        "rtg_write_vtp_discs": (C.c_int, [C.c_char_p, C.c_int64, _f32p, _f32p, _f32p, _f64p, _u64p, _f32p, _f64p,
                                          _f64p, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_int32]),
        "rtg_write_vtp_triangles": (C.c_int, [C.c_char_p, C.c_int64, _f32p, C.c_int64, _u32p, _f64p, _u64p, _f32p,
                                              _f64p, _f64p, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p),
                                              C.c_int32]),
        "rtg_write_vtp_mixed": (C.c_int, [C.c_char_p, C.c_int64, _f32p, _f32p, _f32p, C.c_int64, _f32p, C.c_int64,
                                          _u32p, _f64p, _u64p, _f32p, _f64p, _f64p, C.POINTER(C.c_char_p),
                                          C.POINTER(C.c_char_p), C.c_int32]),
        "rtg_read_point_cloud": (C.c_int, [C.c_char_p, _i64p, _f32p, _f32p, _f32p, C.c_char_p, C.c_int32]),
        "rtg_read_triangles": (C.c_int, [C.c_char_p, _i64p, _f32p, _i64p, _u32p, C.c_char_p, C.c_int32]),
        "rtg_read_point_cloud_vtu": (C.c_int, [C.c_char_p, C.c_int32, _i64p, _f32p, _f32p, _f32p, C.c_char_p,
                                               C.c_int32]),
        "rtg_read_triangles_vtu": (C.c_int, [C.c_char_p, _i64p, _f32p, _i64p, _u32p, _f32p, C.c_char_p,
                                             C.c_int32]),
        "rtg_set_tree_builder": (C.c_int, [_ctx, C.c_int32]),
        "rtg_get_tree_builder": (C.c_int, [_ctx, _i32p]),
        "rtg_set_node_width": (C.c_int, [_ctx, C.c_int32]),
        "rtg_get_node_width": (C.c_int, [_ctx, _i32p]),
        "rtg_get_traversal_width": (C.c_int, [_ctx, _i32p]),
        "rtg_set_segment_log": (C.c_int, [_ctx, C.c_uint64, C.c_uint64, C.c_uint64]),
        "rtg_get_segment_log": (C.c_int, [_ctx, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64),
                                          C.POINTER(C.c_uint64)]),
        "rtg_write_segment_log_vtp": (C.c_int, [_ctx, C.c_char_p]),
        "rtg_write_vtp_segments": (C.c_int, [C.c_char_p, C.c_void_p, C.c_int64]),
        "rtg_set_deposit_mode": (C.c_int, [_ctx, C.c_int32, C.c_float]),
        "rtg_get_deposit_mode": (C.c_int, [_ctx, _i32p, _f32p]),
        "rtg_set_visit_limit": (C.c_int, [_ctx, C.c_uint64]),
        "rtg_get_visit_limit": (C.c_int, [_ctx, _u64p]),
        "rtg_inject_alloc_failure": (C.c_int, [_ctx, C.c_int64]),
        "rtg_set_accumulation": (C.c_int, [_ctx, C.c_int32]),
        "rtg_get_accumulation": (C.c_int, [_ctx, _i32p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def default_config() -> RtgConfig:
    c = RtgConfig()
    load().rtg_config_default(C.byref(c))
    return c
