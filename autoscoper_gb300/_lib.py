"""ctypes binding of libautoscoper_gb300.so (the C ABI in
include/autoscoper_gb300.h).  Loading fails loudly when the library has not
been built: there is no CPU fallback."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.environ.get("ASC_LIB_PATH") or os.path.join(HERE, "libautoscoper_gb300.so")
TUNING = os.path.join(HERE, "tuning.txt")

vp = C.c_void_p
i32 = C.c_int
f32 = C.c_float
f64 = C.c_double
P = C.POINTER

ASC_OK = 0
ASC_STORE_U16, ASC_STORE_F16, ASC_STORE_BF16, ASC_STORE_F32 = 0, 1, 2, 3
ASC_SUM_TREE, ASC_SUM_FULL = 0, 1
ASC_OPT_EMPTY_SKIP = 1
ASC_CURVE_X, ASC_CURVE_Y, ASC_CURVE_Z, ASC_CURVE_ROT, ASC_CURVE_ALL = 1, 2, 4, 8, 15
COST_FN = C.CFUNCTYPE(f64, P(f64), vp)
BATCH_COST_FN = C.CFUNCTYPE(i32, i32, P(i32), P(f64), P(f64), vp)


class OptParams(C.Structure):
    _fields_ = [("method", i32), ("n_particles", i32), ("n_iter", i32), ("w", f64), ("c1", f64), ("c2", f64),
                ("lo", f64), ("hi", f64), ("seed", C.c_uint64), ("offsets", f64 * 6), ("ftol", f64),
                ("max_stall", i32)]


class TrackParams(C.Structure):
    _fields_ = [("opt", OptParams), ("repeats", i32), ("guess", i32), ("dframe", i32), ("keyed", P(i32))]


class FilterDesc(C.Structure):
    _fields_ = [("kind", i32), ("enabled", i32), ("p0", f32), ("p1", f32), ("p2", f32)]


class ViewDesc(C.Structure):
    _fields_ = [("frame", f64 * 12), ("viewport", f64 * 4), ("image_plane", f64 * 12), ("radiograph", vp),
                ("background", vp), ("bg_threshold", f32), ("n_drr_filters", i32), ("n_rad_filters", i32),
                ("drr_filters", FilterDesc * 8), ("rad_filters", FilterDesc * 8)]


class LaunchConfig(C.Structure):
    _fields_ = [("ray_blocks_per_sm", i32), ("view_blocks_per_sm", i32), ("ray_shape", i32)]


class BoneDesc(C.Structure):
    _fields_ = [("volume", vp), ("pivot", f64 * 12), ("base_pose", f64 * 6), ("step", f32 * 4),
                ("intensity", f32 * 4), ("cutoff", f32 * 4)]


# name: (restype, argtypes)
SIGNATURES = {
    "asc_set_option": (i32, [i32, i32]),
    "asc_version": (C.c_char_p, []),
    "asc_status_string": (C.c_char_p, [i32]),
    "asc_last_error": (C.c_char_p, []),
    "asc_malloc": (i32, [P(vp), C.c_size_t]),
    "asc_free": (i32, [vp]),
    "asc_memcpy_h2d": (i32, [vp, vp, C.c_size_t, vp]),
    "asc_memcpy_d2h": (i32, [vp, vp, C.c_size_t, vp]),
    "asc_memcpy_d2d": (i32, [vp, vp, C.c_size_t, vp]),
    "asc_memset": (i32, [vp, i32, C.c_size_t, vp]),
    "asc_stream_sync": (i32, [vp]),
    "asc_device_sync": (i32, []),
    "asc_set_device": (i32, [i32]),
    "asc_stream_create": (i32, [P(vp)]),
    "asc_stream_destroy": (i32, [vp]),
    "asc_event_create": (i32, [P(vp)]),
    "asc_event_record": (i32, [vp, vp]),
    "asc_event_elapsed": (i32, [vp, vp, P(f32)]),
    "asc_event_destroy": (i32, [vp]),
    "asc_host_alloc": (i32, [P(vp), C.c_size_t]),
    "asc_host_free": (i32, [vp]),
    "asc_mem_info": (i32, [P(C.c_size_t), P(C.c_size_t)]),
    "asc_probe_read_bandwidth": (i32, [C.c_size_t, i32, P(f64), P(f32)]),
    "asc_volume_create": (i32, [vp, i32, i32, i32, i32, P(f64), P(i32), i32, P(vp)]),
    "asc_volume_info": (i32, [vp, P(f32), P(f32), P(f64), P(f32), P(f32), P(i32)]),
    "asc_volume_destroy": (i32, [vp]),
    "asc_raycast": (i32, [vp, P(f64), P(f32), f32, f32, f32, i32, vp, i32, i32, vp]),
    "asc_image_create": (i32, [vp, i32, i32, i32, P(vp)]),
    "asc_image_update": (i32, [vp, vp, vp]),
    "asc_image_destroy": (i32, [vp]),
    "asc_rad_render": (i32, [vp, P(f32), P(f32), vp, i32, i32, vp]),
    "asc_background_render": (i32, [vp, P(f32), P(f32), f32, vp, i32, i32, vp]),
    "asc_drr_background": (i32, [vp, vp, i32, i32, vp]),
    "asc_multiply": (i32, [vp, vp, vp, i32, i32, vp]),
    "asc_merge": (i32, [vp, vp, vp, i32, i32, vp]),
    "asc_composite": (i32, [vp, vp, vp, vp, vp, i32, i32, vp]),
    "asc_fill": (i32, [vp, C.c_size_t, f32, vp]),
    "asc_sobel": (i32, [vp, vp, i32, i32, f32, f32, vp]),
    "asc_contrast": (i32, [vp, vp, i32, i32, f32, f32, i32, vp]),
    "asc_gaussian": (i32, [vp, vp, i32, i32, f32, vp]),
    "asc_sharpen": (i32, [vp, vp, i32, i32, f32, f32, f32, vp]),
    "asc_ncc_init": (i32, [C.c_uint]),
    "asc_ncc": (i32, [vp, vp, vp, C.c_uint, i32, vp, vp]),
    "asc_hdist": (i32, [vp, vp, vp, C.c_uint, i32, vp, vp]),
    "asc_ncc_noalloc": (i32, [vp, vp, vp, C.c_uint, i32, vp, vp]),
    "asc_ncc_host": (i32, [vp, vp, vp, C.c_uint, i32, P(f64), vp]),
    "asc_hdist_host": (i32, [vp, vp, vp, C.c_uint, i32, P(f64), vp]),
    "asc_engine_create": (i32, [i32, P(ViewDesc), i32, P(BoneDesc), i32, i32, i32, i32, i32, P(vp)]),
    "asc_engine_destroy": (i32, [vp]),
    "asc_engine_set_launch": (i32, [vp, P(LaunchConfig)]),
    "asc_engine_get_launch": (i32, [vp, P(LaunchConfig), P(i32)]),
    "asc_engine_workload_class": (i32, [vp, P(i32)]),
    "asc_tuning_load": (i32, [C.c_char_p]),
    "asc_engine_set_view": (i32, [vp, i32, P(ViewDesc), i32, i32]),
    "asc_engine_set_bone": (i32, [vp, i32, P(BoneDesc), i32, P(i32)]),
    "asc_engine_set_base_pose": (i32, [vp, i32, P(f64)]),
    "asc_engine_set_radiograph": (i32, [vp, i32, vp]),
    "asc_engine_set_visible": (i32, [vp, i32, i32]),
    "asc_engine_eval": (i32, [vp, i32, vp, vp, vp, vp, vp]),
    "asc_engine_eval_host": (i32, [vp, i32, P(i32), P(f64), P(f64), P(f64), vp]),
    "asc_engine_eval_plain": (i32, [vp, i32, P(i32), P(f64), P(f64), P(f64), vp]),
    "asc_engine_debug": (i32, [vp, P(vp), P(vp)]),
    "asc_engine_profile": (i32, [vp, i32]),
    "asc_engine_stats": (i32, [vp, P(f32), P(C.c_ulonglong), P(C.c_ulonglong)]),
    "asc_engine_counters": (i32, [vp, P(C.c_ulonglong)]),
    "asc_engine_exact_rays": (i32, [vp, P(i32)]),
    "asc_engine_pso": (i32, [vp, i32, i32, f64, f64, f64, f64, f64, C.c_uint64, P(f64), P(f64),
                             P(C.c_longlong), vp]),
    "asc_engine_pso_stall": (i32, [vp, i32, i32, i32, f64, f64, f64, f64, f64, C.c_uint64, P(f64), P(f64),
                                   P(C.c_longlong), P(i32), vp]),
    "asc_pso_sequential": (i32, [COST_FN, vp, i32, f32, f32, C.c_uint, C.c_uint, C.c_uint, P(f32), P(f32)]),
    "asc_amoeba": (i32, [COST_FN, vp, P(f64), P(f64), i32, f64, P(i32)]),
    "asc_amoeba_batch": (i32, [BATCH_COST_FN, vp, i32, P(f64), P(f64), i32, f64, P(i32)]),
    "asc_engine_optimize_frame": (i32, [vp, P(OptParams), P(f64), P(f64), P(C.c_longlong), vp]),
    "asc_engine_optimize_frame_ex": (i32, [vp, P(OptParams), P(f64), P(f64), P(f64), P(C.c_longlong), vp]),
    "asc_keycurve_store": (i32, [P(f64), P(f64)]),
    "asc_engine_optimize_curves": (i32, [vp, P(vp), i32, i32, P(TrackParams), P(f64), P(C.c_longlong), vp]),
    "asc_pose_to_matrix": (i32, [P(f64), P(f64)]),
    "asc_pose_from_matrix": (i32, [P(f64), P(f64)]),
    "asc_pose_curve_create": (i32, [P(vp)]),
    "asc_pose_curve_destroy": (i32, [vp]),
    "asc_pose_curve_clear": (i32, [vp]),
    "asc_pose_curve_insert": (i32, [vp, i32, P(f64), i32]),
    "asc_pose_curve_erase": (i32, [vp, i32, i32]),
    "asc_pose_curve_keys": (i32, [vp, i32, P(i32)]),
    "asc_pose_curve_eval": (i32, [vp, i32, P(f64)]),
    "asc_background_from_frames": (i32, [P(vp), i32, vp, vp]),
    "asc_engine_render_drr": (i32, [vp, i32, P(f64), P(f64), vp, vp]),
    "asc_engine_image_data": (i32, [vp, i32, i32, P(f64), vp, vp, vp, P(i32), P(i32), vp]),
    "asc_engine_track": (i32, [vp, i32, P(vp), P(TrackParams), P(f64), P(f64), P(C.c_longlong), vp]),
}

_LIB = None


class AscError(RuntimeError):
    def __init__(self, fn, status):
        lib = _LIB
        msg = lib.asc_status_string(status).decode() if lib else str(status)
        last = lib.asc_last_error().decode() if lib else ""
        super().__init__(f"{fn} failed: {msg} ({status}){': ' + last if last else ''}")
        self.status = status


def load(path: str = SO):
    """Loads the library (once) and declares every entry point."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(path):
            raise ImportError(f"{path} is missing: build it with `python -m autoscoper_gb300.build` "
                              "(there is no CPU fallback)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        # the autotuner's launch shapes per workload class, for the engines created from here on
        if os.path.exists(TUNING):
            check("asc_tuning_load", lib.asc_tuning_load(TUNING.encode()))
    return _LIB


def check(fn: str, status: int):
    if status != ASC_OK:
        raise AscError(fn, status)
    return status


def call(name: str, *args):
    return check(name, getattr(load(), name)(*args))
