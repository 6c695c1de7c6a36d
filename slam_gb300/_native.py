"""Loader for the native libraries built in-tree by slam_gb300/_build.py.

There is no fallback: if libslam_gb300.so is missing or fails to load, every
entry point raises.
"""
import ctypes
import os

from . import _build

_LIB = None
_SYNTH = None


class NativeError(RuntimeError):
    pass


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Returns the ctypes handle of libslam_gb300.so (declaring every C-ABI
    function's signature)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise NativeError("libslam_gb300.so is not built (run __graft_entry__.build())")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    _declare(L)
    _LIB = L
    return L


def load_synth(build_if_missing=True):
    global _SYNTH
    if _SYNTH is not None:
        return _SYNTH
    if not os.path.exists(_build.SYNTH_LIB):
        if not build_if_missing:
            raise NativeError("libslam_synth.so is not built")
        _build.build()
    S = ctypes.CDLL(_build.SYNTH_LIB)
    _SYNTH = S
    return S


c_int, c_float, c_double, c_void_p, c_size_t = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t
P = ctypes.POINTER


class OdoStats(ctypes.Structure):
    _fields_ = [("lastICPError", c_float), ("lastICPCount", c_float), ("lastRGBError", c_float),
                ("lastRGBCount", c_float), ("lastSO3Error", c_float), ("lastSO3Count", c_float),
                ("lastA", c_double * 36), ("lastb", c_double * 6)]


class OdoPair(ctypes.Structure):
    _fields_ = [("width", c_int), ("height", c_int), ("fx", c_float), ("fy", c_float), ("cx", c_float),
                ("cy", c_float), ("distThresh", c_float), ("angleThresh", c_float), ("depthCutoff", c_float),
                ("levels", c_int), ("iterations", c_int * 3), ("model_verts", c_void_p), ("model_norms", c_void_p), ("model_pitch", c_size_t),
                ("model_rgba", c_void_p), ("model_rgba_pitch", c_size_t), ("depth", c_void_p),
                ("depth_pitch", c_size_t), ("rgba", c_void_p), ("rgba_pitch", c_size_t), ("prev_rgba", c_void_p),
                ("prev_rgba_pitch", c_size_t), ("pose", c_float * 16), ("live_verts", c_void_p),
                ("live_norms", c_void_p), ("live_pitch", c_size_t)]


class OdoPairResult(ctypes.Structure):
    _fields_ = [("pose", c_float * 16), ("lastICPError", c_float), ("lastICPCount", c_float),
                ("lastRGBError", c_float), ("lastRGBCount", c_float), ("lastSO3Error", c_float),
                ("lastSO3Count", c_float), ("iterations", c_int * 4), ("done_us", c_double),
                ("lastA", c_double * 36), ("lastb", c_double * 6)]


class OdoPredictParams(ctypes.Structure):
    _fields_ = [("width", c_int), ("height", c_int), ("cx", c_float), ("cy", c_float), ("fx", c_float),
                ("fy", c_float), ("maxDepth", c_float), ("confThreshold", c_float), ("time", c_int),
                ("maxTime", c_int), ("timeDelta", c_int)]


class OdoVerifyParams(ctypes.Structure):
    _fields_ = [("rgbOnly", c_int), ("icpWeight", c_float), ("fastOdom", c_int), ("so3", c_int),
                ("max_icp_error", c_float), ("min_icp_count", c_float), ("max_covariance", c_double)]


class OdoWarmParams(ctypes.Structure):
    _fields_ = [("levels", c_int), ("iterations", c_int * 3), ("residual_limit", c_float),
                ("max_disagree", c_float), ("rgbOnly", c_int), ("icpWeight", c_float), ("fastOdom", c_int)]


# (name, restype, argtypes) of every function declared in include/slam_gb300.h
SIGNATURES = [
    ("odo_create", c_int, [c_int, c_int, c_float, c_float, c_float, c_float, c_float, c_float, P(c_void_p)]),
    ("odo_destroy", c_int, [c_void_p]),
    ("odo_set_stream", c_int, [c_void_p, c_void_p]),
    ("odo_init_icp_depth", c_int, [c_void_p, c_void_p, c_size_t, c_float]),
    ("odo_init_icp_maps", c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_float]),
    ("odo_init_icp_raw_depth", c_int, [c_void_p, c_void_p, c_size_t, c_float, c_float]),
    ("odo_model_predict_scratch_bytes", c_size_t, [c_int, c_int]),
    ("odo_model_predict", c_int, [c_void_p, c_int, P(c_float), P(OdoPredictParams), c_void_p, c_void_p, c_size_t,
                                  c_void_p, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p]),
    ("odo_fill_in", c_int, [c_void_p, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p, c_size_t,
                            c_int, c_int, c_float, c_float, c_float, c_float, c_int, c_void_p, c_void_p, c_size_t,
                            c_void_p, c_size_t, c_void_p]),
    ("odo_png_unfilter", c_int, [c_void_p, c_int, c_size_t, c_int, c_void_p]),
    ("odo_host_copy", c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    ("odo_filter_depth", c_int, [c_void_p, c_size_t, c_void_p, c_size_t, c_int, c_int, c_float, c_void_p]),
    ("odo_depth_metric", c_int, [c_void_p, c_size_t, c_void_p, c_size_t, c_int, c_int, c_float, c_void_p]),
    ("odo_init_icp_model", c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_float, P(c_float)]),
    ("odo_init_rgb", c_int, [c_void_p, c_void_p, c_size_t]),
    ("odo_init_rgb_model", c_int, [c_void_p, c_void_p, c_size_t]),
    ("odo_init_first_rgb", c_int, [c_void_p, c_void_p, c_size_t]),
    ("odo_get_incremental_transformation", c_int,
     [c_void_p, P(c_float), P(c_float), c_int, c_float, c_int, c_int, c_int]),
    ("odo_get_covariance", c_int, [c_void_p, P(c_double)]),
    ("odo_get_stats", c_int, [c_void_p, P(OdoStats)]),
    ("odo_get_iterations", c_int, [c_void_p, P(c_int)]),
    ("odo_set_mode", c_int, [c_void_p, c_int]),
    ("odo_set_precision", c_int, [c_void_p, c_int]),
    ("odo_state_bytes", c_size_t, []),
    ("odo_last_error", ctypes.c_char_p, [c_void_p]),
    ("odo_status_string", ctypes.c_char_p, [c_int]),
    ("odo_debug_download", c_int, [c_void_p, c_int, c_int, c_void_p, c_size_t]),
    ("odo_debug_upload", c_int, [c_void_p, c_int, c_int, c_void_p, c_size_t]),
    ("odo_debug_icp_step", c_int, [c_void_p, c_int, P(c_float), P(c_float), P(c_float), P(c_float), c_void_p,
                                   P(c_double)]),
    ("odo_debug_icp_sums", c_int, [c_void_p, c_int, P(c_float), P(c_float), P(c_float), P(c_float), P(c_double)]),
    ("odo_debug_rgb_sums", c_int, [c_void_p, c_int, c_float, P(c_double)]),
    ("odo_debug_rgb_residual", c_int, [c_void_p, c_int, P(c_float), P(c_float), P(ctypes.c_int32)]),
    ("odo_debug_rgb_step", c_int, [c_void_p, c_int, c_float, P(c_double)]),
    ("odo_debug_so3_step", c_int, [c_void_p, P(c_float), P(c_float), P(c_float), P(c_double)]),
    ("odo_debug_derivatives", c_int, [c_void_p]),
    ("odo_debug_time_iteration", c_int, [c_void_p, c_int, c_int, P(c_float)]),
    ("odo_batch_debug_set_split", c_int, [c_void_p, c_int]),
    ("odo_debug_profile", c_int, [c_void_p, P(c_double), c_int]),
    ("odo_debug_set_wait_limit", c_int, [c_void_p, ctypes.c_longlong, c_int]),
    ("odo_debug_history", c_int, [c_void_p, P(c_double), c_int]),
    ("odo_cnn_param_count", c_size_t, []),
    ("odo_cnn_create", c_int, [c_int, P(c_void_p)]),
    ("odo_cnn_destroy", c_int, [c_void_p]),
    ("odo_cnn_set_stream", c_int, [c_void_p, c_void_p]),
    ("odo_cnn_init_params", c_int, [c_void_p, ctypes.c_uint64]),
    ("odo_cnn_set_params", c_int, [c_void_p, P(c_float)]),
    ("odo_cnn_get_params", c_int, [c_void_p, P(c_float)]),
    ("odo_cnn_set_loss_metric", c_int, [c_void_p, P(c_float)]),
    ("odo_cnn_forward", c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    ("odo_cnn_train_step", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_float, P(c_float)]),
    ("odo_cnn_pack_input", c_int, [c_void_p, P(OdoPair), c_int, c_void_p]),
    ("odo_synth_render", c_int, [c_void_p, c_int, P(c_int), P(c_float), P(ctypes.c_uint64), c_int, c_int, c_int,
                                 c_float, c_float, c_float, c_float, c_float, c_float, c_int, c_int, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p]),
    ("odo_cnn_propose", c_int, [c_void_p, P(OdoPair), c_int, c_void_p]),
    ("odo_cnn_event", c_void_p, [c_void_p]),
    ("odo_cnn_wait", c_int, [c_void_p]),
    ("odo_batch_track_warm", c_int, [c_void_p, c_void_p, P(OdoPair), c_int, P(OdoWarmParams), P(OdoPairResult),
                                     P(c_int)]),
    ("odo_cnn_gradients", c_int, [c_void_p, c_void_p, c_void_p, c_int, P(c_float), P(c_float)]),
    ("odo_cnn_last_error", ctypes.c_char_p, [c_void_p]),
    ("odo_cnn_debug_gemm", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p]),
    ("odo_batch_create", c_int, [c_int, P(c_void_p)]),
    ("odo_batch_destroy", c_int, [c_void_p]),
    ("odo_batch_set_stream", c_int, [c_void_p, c_void_p]),
    ("odo_batch_set_launch", c_int, [c_void_p, c_int, c_int]),
    ("odo_batch_track", c_int, [c_void_p, P(OdoPair), c_int, c_int, c_float, c_int, c_int, P(OdoPairResult)]),
    ("odo_batch_debug_time_iteration", c_int, [c_void_p, c_int, c_int, P(c_float)]),
    ("odo_batch_track_init", c_int, [c_void_p, P(OdoPair), c_int, c_void_p, c_int, c_float, c_int, P(OdoPairResult)]),
    ("odo_batch_verify", c_int, [c_void_p, c_void_p, c_int, P(OdoVerifyParams), c_void_p, P(c_double), P(c_int)]),
    ("odo_batch_autotune", c_int, [c_void_p, P(OdoPair), c_int, c_int, c_float, c_int, c_int, P(OdoPairResult),
                                   P(c_int), P(c_int), P(c_float)]),
    ("odo_batch_last_error", ctypes.c_char_p, [c_void_p]),
    ("odo_icp_step_noalloc", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_int, P(c_float),
                                     c_float, c_float, P(c_float), P(c_float), P(c_float), P(c_float), c_void_p,
                                     P(c_float), P(c_float), P(c_float)]),
]


def _declare(L):
    for name, res, args in SIGNATURES:
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
