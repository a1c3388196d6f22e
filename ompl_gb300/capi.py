"""ctypes declarations of libgbompl.so (include/gbompl.h). Loading fails loudly when the library is
missing: there is no CPU fallback anywhere in this package."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbompl.so")

OK, ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_NO_DEVICE, ERR_OUT_OF_MEMORY, ERR_TIMEOUT, ERR_UNSUPPORTED = range(7)
LAYOUT_SOA, LAYOUT_AOS = 0, 1
SPACE_REAL_VECTOR, SPACE_SO2, SPACE_KINEMATIC_CHAIN, SPACE_WRAP_L2 = 0, 1, 2, 3
CHECK_ALL_VALID, CHECK_CIRCLES, CHECK_CHAIN_SEGMENTS, CHECK_DH_SPHERES, CHECK_DH_BOXES = 0, 1, 2, 3, 4
PRECISION_FP64, PRECISION_FP32_GUARDED = 0, 1
SCHEDULE_PLAIN, SCHEDULE_TILE, SCHEDULE_WARP, SCHEDULE_AUTO = 0, 1, 2, 3
REQ_VALIDITY, REQ_MOTION, REQ_KNN = 0, 1, 2


class Request(C.Structure):
    """gbo_request (include/gbompl.h)."""
    _fields_ = [("kind", C.c_int), ("checker", C.c_void_p), ("nn", C.c_void_p), ("states", C.c_void_p),
                ("states2", C.c_void_p), ("n", C.c_int64), ("k", C.c_int), ("schedule", C.c_int),
                ("ok", C.c_void_p), ("first_j", C.c_void_p), ("nd", C.c_void_p), ("idx", C.c_void_p),
                ("dist", C.c_void_p)]

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I64 = C.c_int64

# name: (restype, argtypes)
SIGNATURES = {
    "gbo_status_string": (C.c_char_p, [C.c_int]),
    "gbo_last_error": (C.c_char_p, []),
    "gbo_device_check": (C.c_int, [C.POINTER(C.c_int)] * 3),
    "gbo_space_create": (C.c_int, [C.c_int, C.c_int, _D, _D, C.c_double, C.c_double, C.c_double, C.c_uint,
                                   C.POINTER(_P)]),
    "gbo_space_destroy": (C.c_int, [_P]),
    "gbo_space_info": (C.c_int, [_P, _D, _D]),
    "gbo_space_distance": (C.c_int, [_P, _P, _P, _I64, _I64, C.c_int, _P, _P]),
    "gbo_space_interpolate": (C.c_int, [_P, _P, _P, _P, _I64, _I64, C.c_int, _P, _P]),
    "gbo_get_motion_states": (C.c_int, [_P, _P, _P, _I64, _I64, C.c_int, C.c_uint, C.c_int, _P, _I64, _P]),
    "gbo_checker_create": (C.c_int, [_P, C.c_int, _D, _I64, _D, C.c_int, C.c_int, C.c_double, C.POINTER(_P)]),
    "gbo_checker_destroy": (C.c_int, [_P]),
    "gbo_checker_set_precision": (C.c_int, [_P, C.c_int]),
    "gbo_checker_stats": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "gbo_is_valid": (C.c_int, [_P, _P, _I64, _I64, C.c_int, _P, _P]),
    "gbo_check_motion": (C.c_int, [_P, _P, _P, _I64, _I64, C.c_int, C.c_int, _P, _P, _P, _P]),
    "gbo_last_valid": (C.c_int, [_P, _P, _P, _P, _P, _I64, _I64, C.c_int, _P, _P, _P]),
    "gbo_check_motion_states": (C.c_int, [_P, _P, _I64, _I64, C.c_int, _P, _P, _P]),
    "gbo_is_valid_host": (C.c_int, [_P, _P, _I64, _P]),
    "gbo_check_motion_host": (C.c_int, [_P, _P, _P, _I64, _P, _P, _P]),
    "gbo_sampler_create": (C.c_int, [_P, C.c_uint32, C.POINTER(_P)]),
    "gbo_sampler_destroy": (C.c_int, [_P]),
    "gbo_sample_uniform": (C.c_int, [_P, _I64, _P, _I64, C.c_int, _P]),
    "gbo_sample_uniform_near": (C.c_int, [_P, _P, C.c_double, _I64, _I64, C.c_int, _P, _P]),
    "gbo_sample_gaussian": (C.c_int, [_P, _P, C.c_double, _I64, _I64, C.c_int, _P, _P]),
    "gbo_sample_valid": (C.c_int, [_P, _P, _I64, C.c_uint, _P, _I64, C.c_int, _P, _P]),
    "gbo_sample_valid_host": (C.c_int, [_P, _P, _I64, C.c_uint, _P, _P]),
    "gbo_nn_create": (C.c_int, [_P, _I64, C.POINTER(_P)]),
    "gbo_nn_destroy": (C.c_int, [_P]),
    "gbo_nn_set_precision": (C.c_int, [_P, C.c_int]),
    "gbo_nn_add": (C.c_int, [_P, _P, _I64, _I64, C.c_int, C.POINTER(_I64), _P]),
    "gbo_nn_remove": (C.c_int, [_P, _P, _I64, _P]),
    "gbo_nn_clear": (C.c_int, [_P]),
    "gbo_nn_size": (C.c_int, [_P, C.POINTER(_I64)]),
    "gbo_nn_nearest_k": (C.c_int, [_P, _P, _I64, _I64, C.c_int, C.c_int, _P, _P, _P, _P]),
    "gbo_nn_nearest_r_count": (C.c_int, [_P, _P, _I64, _I64, C.c_int, C.c_double, _P, _P]),
    "gbo_nn_nearest_r_fill": (C.c_int, [_P, _P, _I64, _I64, C.c_int, C.c_double, _P, _P, _P, _P]),
    "gbo_nn_stats": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "gbo_nn_nearest_k_noalloc": (C.c_int, [_P, _P, _I64, _I64, C.c_int, C.c_int, _P, _P, _P, _P]),
    "gbo_nn_add_host": (C.c_int, [_P, _P, _I64, C.POINTER(_I64)]),
    "gbo_nn_remove_host": (C.c_int, [_P, _P, _I64]),
    "gbo_nn_nearest_k_host": (C.c_int, [_P, _P, _I64, C.c_int, _P, _P]),
    "gbo_nn_nearest_r_host": (C.c_int, [_P, _P, C.c_double, _I64, C.POINTER(_I64), _P, _P]),
    "gbo_sample_uniform_host": (C.c_int, [_P, _I64, _P]),
    "gbo_sample_uniform_near_host": (C.c_int, [_P, _P, C.c_double, _I64, _P]),
    "gbo_sample_gaussian_host": (C.c_int, [_P, _P, C.c_double, _I64, _P]),
    "gbo_server_create": (C.c_int, [C.c_int, _I64, C.POINTER(_P)]),
    "gbo_server_destroy": (C.c_int, [_P]),
    "gbo_server_submit": (C.c_int, [_P, _P, C.POINTER(C.c_uint64)]),
    "gbo_server_wait": (C.c_int, [_P, C.c_uint64, C.c_double, _D]),
    "gbo_server_stats": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(_I64),
                                   C.POINTER(C.c_int)]),
    "gbo_measure_fp32_peak": (C.c_int, [_D, _P]),
    "gbo_measure_fp64_peak": (C.c_int, [_D, _P]),
    "gbo_sincos32": (C.c_int, [_P, _I64, _P, _P, _P]),
    "gbo_launch_count": (C.c_uint64, []),
    "gbo_selftest_bounded_wait": (C.c_int, [_I64, C.POINTER(C.c_double)]),
    "gbo_nn_error_stats": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "gbo_checker_counters": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "gbo_checker_precision_stats": (C.c_int, [_P, _P, _I64, _I64, C.c_int, _P, _P]),
    "gbo_sincos_cr": (C.c_int, [_P, _I64, _P, _P, _P]),
    "gbo_log_rn": (C.c_int, [_P, _I64, _P, _P]),
    "gbo_prm_component_roots": (C.c_int, [_P, _P, _I64, _I64, _P]),
    "gbo_mt19937_discard": (C.c_int, [_P, _P, C.c_uint64]),
    "gbo_nn_nearest_sqrt_approx": (C.c_int, [_P, _P, _I64, _I64, C.c_int, _P, _P, _P, _P]),
    "gbo_nn_nearest_sqrt_approx_host": (C.c_int, [_P, _P, _I64, _P, _P, _P]),
    "gbo_nn_search_bytes": (C.c_int, [_P, _P]),
}


class PrecisionStats(C.Structure):
    """gbo_precision_stats (include/gbompl.h)."""
    _fields_ = [("states", C.c_uint64), ("flips", C.c_uint64), ("ambiguous", C.c_uint64),
                ("max_abs_err", C.c_double)]


class GboError(RuntimeError):
    """Raised for a non-OK status (OMPL raises ompl::Exception for the same misconfigurations)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                              f"g.build()\"` (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int):
    if status != OK:
        L = lib()
        raise GboError(status, L.gbo_last_error().decode() or L.gbo_status_string(status).decode())
    return status
