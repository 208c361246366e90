"""ctypes mirror of include/gcr.h and the loader of libgcr.so.

The library is built in-tree (``graph-cut-ransac_gb300/_build/libgcr.so``) by
``build.py``; importing this module never compiles anything. A missing library
raises ``ImportError`` with the build command: there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libgcr.so")

GCR_OK = 0
GCR_INVALID_ARG = 1
GCR_TOO_FEW_POINTS = 2
GCR_NO_MODEL = 3
GCR_DEVICE_ERROR = 4
GCR_TIMEOUT = 5
GCR_CAPACITY = 6
GCR_UNSUPPORTED = 7

STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "TOO_FEW_POINTS", 3: "NO_MODEL",
    4: "DEVICE_ERROR", 5: "TIMEOUT", 6: "CAPACITY", 7: "UNSUPPORTED",
}

GCR_SCORING_MSAC = 0
GCR_SCORING_MAGSAC = 1

GCR_SAMPLER_UNIFORM = 0
GCR_SAMPLER_PROSAC = 1
GCR_SAMPLER_PNAPSAC = 2
GCR_SAMPLER_IMPORTANCE = 3
GCR_SAMPLER_AR = 4

GCR_LO_FP64 = 0
GCR_LO_FP32 = 1

GCR_HOMOGRAPHY = 0
GCR_FUNDAMENTAL = 1
GCR_ESSENTIAL = 2
GCR_HOMOGRAPHY_AFFINE = 3  # rows of 8: points, then the local affine map
GCR_FUNDAMENTAL_AFFINE = 4  # rows of 8
GCR_FUNDAMENTAL_SIFT = 5  # rows of 8: points, then scales and orientations (q1, q2, o1, o2)
GCR_HOMOGRAPHY_SIFT = 6  # rows of 8: points, then scales and orientations (q1, q2, o1, o2)
GCR_ESSENTIAL_PLANAR = 7  # rows of 4; planar camera motion

GCR_FLAG_LO_APPLIED = 1
GCR_FLAG_IRLS_APPLIED = 2
GCR_FLAG_DEGENSAC_SKIPPED = 4


class ImageSize(ctypes.Structure):
    _fields_ = [("h1", ctypes.c_int32), ("w1", ctypes.c_int32),
                ("h2", ctypes.c_int32), ("w2", ctypes.c_int32)]


class Params(ctypes.Structure):
    _fields_ = [
        ("threshold", ctypes.c_double),
        ("confidence", ctypes.c_double),
        ("spatial_coherence_weight", ctypes.c_double),
        ("neighborhood_size", ctypes.c_double),
        ("max_iterations", ctypes.c_int64),
        ("min_iterations", ctypes.c_int64),
        ("sampler", ctypes.c_int32),
        ("neighborhood", ctypes.c_int32),
        ("lo_number", ctypes.c_int32),
        ("scoring", ctypes.c_int32),
        ("use_sprt", ctypes.c_int32),
        ("use_space_partitioning", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("min_inlier_ratio_for_sprt", ctypes.c_double),
        ("sampler_variance", ctypes.c_double),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("max_n", ctypes.c_int32), ("batch_calls", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("order", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [
        ("iteration_number", ctypes.c_int64),
        ("graph_cut_number", ctypes.c_int64),
        ("local_optimization_number", ctypes.c_int64),
        ("inlier_number", ctypes.c_int64),
        ("score", ctypes.c_double),
        ("status", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("models_scored", ctypes.c_int64),
    ]


# numpy dtype with the same layout as gcr_stats (for batched outputs)
STATS_DTYPE = np.dtype([
    ("iteration_number", np.int64), ("graph_cut_number", np.int64),
    ("local_optimization_number", np.int64), ("inlier_number", np.int64),
    ("score", np.float64), ("status", np.int32), ("flags", np.int32), ("models_scored", np.int64),
])
SIZE_DTYPE = np.dtype([("h1", np.int32), ("w1", np.int32), ("h2", np.int32), ("w2", np.int32)])

assert ctypes.sizeof(Stats) == STATS_DTYPE.itemsize == 56
assert ctypes.sizeof(Params) == 96

_P = ctypes.c_void_p
_EXPORTS = {
    "gcr_default_params": (None, [ctypes.c_int, _P]),
    "gcr_find_homography": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P]),
    "gcr_find_fundamental": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P]),
    "gcr_find_essential": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "gcr_find_homography_affine": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P]),
    "gcr_find_fundamental_affine": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P]),
    "gcr_find_fundamental_sift": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P]),
    "gcr_find_homography_sift": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P]),
    "gcr_find_essential_planar": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "gcr_find_batch": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "gcr_context_create": (ctypes.c_int, [_P]),
    "gcr_context_destroy": (ctypes.c_int, [_P]),
    "gcr_batch_run_device": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P,
                                            _P, _P, _P]),
    "gcr_find_homography_device_noalloc": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, ctypes.c_uint64, _P, _P, _P,
                                                          _P]),
    "gcr_batch_prepare": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "gcr_batch_launch": (ctypes.c_int, [_P, _P]),
    "gcr_context_set_pair_times": (ctypes.c_int, [_P, _P]),
    "gcr_context_set_probabilities": (ctypes.c_int, [_P, _P]),
    "gcr_context_set_flow_step_limit": (ctypes.c_int, [_P, ctypes.c_int64]),
    "gcr_context_set_sample_tape": (ctypes.c_int, [_P, _P, ctypes.c_int64]),
    "gcr_set_sample_tape": (ctypes.c_int, [_P, ctypes.c_int64]),
    "gcr_context_set_tuning": (ctypes.c_int, [_P, _P, ctypes.c_int32]),
    "gcr_context_last_tuning": (ctypes.c_int, [_P, _P]),
    "gcr_context_set_lo_precision": (ctypes.c_int, [_P, ctypes.c_int32]),
    "gcr_run": (ctypes.c_int, [ctypes.c_int, _P, _P, ctypes.c_int64, _P, ctypes.c_int32, _P, _P, _P, _P, _P]),
    "gcr_run_with_probabilities": (ctypes.c_int, [ctypes.c_int, _P, _P, ctypes.c_int64, _P, ctypes.c_int32, _P, _P,
                                                  _P, _P, _P, _P]),
    "gcr_learned_param_count": (ctypes.c_int64, []),
    "gcr_learned_feature_width": (ctypes.c_int32, []),
    "gcr_learned_features": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64, _P, _P]),
    "gcr_learned_params_to_bf16": (ctypes.c_int, [_P, _P, _P]),
    "gcr_learned_forward": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P]),
    "gcr_learned_backward": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P, _P, _P, _P, _P, ctypes.c_float, _P,
                                            _P]),
    "gcr_learned_adam": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_float, ctypes.c_int64, _P]),
    "gcr_learned_order": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P, _P]),
    "gcr_learned_propose": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _P, _P, _P,
                                           _P, _P, _P]),
    "gcr_learned_unpermute_mask": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int64, _P, _P]),
    "gcr_last_launch_count": (ctypes.c_int64, []),
    "gcr_last_error_string": (ctypes.c_char_p, []),
}

_lib = None


def load():
    """Returns the loaded libgcr.so, raising ImportError when it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"libgcr.so not found at {LIB_PATH}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python graph-cut-ransac_gb300/build.py`")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_EXPORTS)


def ptr(a):
    """Address of a numpy array's data (None -> NULL). The returned pointer
    object holds a reference to the array, so a temporary passed straight into
    a call stays alive until the call returns."""
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def last_error():
    msg = load().gcr_last_error_string()
    return msg.decode() if msg else ""
