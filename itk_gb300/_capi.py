"""ctypes binding of the C ABI in ``include/itk_gb300.h``.

The library ``itk_gb300/_lib/libitk_gb300.so`` is built in-tree by
``itk_gb300.build``.  There is no CPU fallback: if the library is missing or
no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

GB_OK = 0
GB_ERR_BAD_ARG = 1
GB_ERR_NO_VALID_POINTS = 2
GB_ERR_JOINT_PDF_SUM_ZERO = 3
GB_ERR_FIXED_CONSTANT = 4
GB_ERR_MOVING_CONSTANT = 5
GB_ERR_FIXED_EMPTY = 6
GB_ERR_MOVING_EMPTY = 7
GB_ERR_OUT_OF_MEMORY = 8
GB_ERR_CUDA = 9
GB_ERR_TIMEOUT = 10
GB_ERR_NOT_INITIALIZED = 11
GB_ERR_UNSUPPORTED = 12
GB_ERR_ADMISSION = 13

GB_METRIC_MEAN_SQUARES = 0
GB_METRIC_MATTES = 1
GB_METRIC_CORRELATION = 2
GB_METRIC_JOINT_HISTOGRAM_MI = 3
GB_IMAGE_FIXED = 0
GB_IMAGE_MOVING = 1
GB_TRANSFORM_AFFINE = 0
GB_TRANSFORM_BSPLINE = 1
GB_TRANSFORM_COMPOSITE = 2
GB_TRANSFORM_DISPLACEMENT_FIELD = 3
GB_GRADIENT_IMAGE = 0
GB_GRADIENT_CENTRAL_DIFFERENCE = 1
GB_GRADIENT_RECURSIVE_GAUSSIAN = 2

# gb_metric_set_fault_injection
GB_FAULT_NONE = 0
GB_FAULT_STALLED_COPY = 1

# MetricSamplingStrategyEnum
GB_SAMPLING_NONE = 0
GB_SAMPLING_REGULAR = 1
GB_SAMPLING_RANDOM = 2

# StopConditionObjectToObjectOptimizerEnum
GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS = 0
GB_STOP_COSTFUNCTION_ERROR = 1
GB_STOP_UPDATE_PARAMETERS_ERROR = 2
GB_STOP_STEP_TOO_SMALL = 3
GB_STOP_CONVERGENCE_CHECKER_PASSED = 4
GB_STOP_GRADIENT_MAGNITUDE_TOLERANCE = 5
GB_STOP_OTHER_ERROR = 6


class RegularStepSettings(ctypes.Structure):
    """gb_regular_step_settings."""
    _fields_ = [("learning_rate", ctypes.c_double), ("relaxation_factor", ctypes.c_double),
                ("minimum_step_length", ctypes.c_double), ("gradient_magnitude_tolerance", ctypes.c_double),
                ("number_of_iterations", ctypes.c_int64), ("return_best_parameters_and_value", ctypes.c_int)]


class OptimizerReport(ctypes.Structure):
    """gb_optimizer_report."""
    _fields_ = [("stop_condition", ctypes.c_int), ("metric_status", ctypes.c_int), ("iterations", ctypes.c_int64),
                ("value", ctypes.c_double), ("current_step_length", ctypes.c_double),
                ("gradient_magnitude", ctypes.c_double), ("learning_rate_relaxation", ctypes.c_double)]

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_D = ctypes.c_double

# name -> argtypes (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "gb_last_error": [],
    "gb_metric_last_error": [_P],
    "gb_version": [],
    "gb_ctx_create": [_I, _P],
    "gb_ctx_destroy": [_P],
    "gb_ctx_info": [_P, _P, _P, _P],
    "gb_metric_create": [_P, _I, _P],
    "gb_metric_destroy": [_P],
    "gb_metric_set_number_of_histogram_bins": [_P, _U64],
    "gb_metric_set_joint_pdf_smoothing_variance": [_P, _D],
    "gb_metric_set_floating_point_correction": [_P, _I, _D],
    "gb_metric_set_image": [_P, _I, _P, _P, _P, _P, _P],
    "gb_metric_set_image_device": [_P, _I, _P, _P, _P, _P, _P],
    "gb_metric_set_gradient_source": [_P, _I],
    "gb_metric_set_moving_gradient_image": [_P, _P],
    "gb_metric_set_virtual_domain": [_P, _P, _P, _P, _P],
    "gb_metric_set_level_smoothing": [_P, _D, _I],
    "gb_metric_set_level_shrink": [_P, _P],
    "gb_smooth_recursive_gaussian": [_P, _U64, _P, _P, _P, _P, _P],
    "gb_gradient_recursive_gaussian": [_P, _U64, _P, _P, _P, _P, _P, _D, _I, _I],
    "gb_smooth_recursive_gaussian_host": [_P, _P, _P, _P, _P, _P],
    "gb_gradient_recursive_gaussian_host": [_P, _P, _P, _P, _P, _P, _D, _I, _I],
    "gb_shrink_geometry": [_P, _P, _P, _P, _P, _P, _P, _P],
    "gb_metric_set_sampled_points": [_P, _P, _I64, _I],
    "gb_metric_use_sampled_point_set": [_P, _I],
    "gb_metric_set_moving_transform": [_P, _I, _P, _I64, _P, _I64],
    "gb_metric_set_parameters": [_P, _P, _I64],
    "gb_metric_update_transform_parameters": [_P, _P, _I64, _D],
    "gb_metric_get_parameters": [_P, _P, _I64],
    "gb_metric_get_number_of_parameters": [_P, _P],
    "gb_metric_initialize": [_P],
    "gb_metric_get_value_and_derivative": [_P, _P, _P, _I64],
    "gb_metric_get_value": [_P, _P],
    "gb_metric_get_number_of_valid_points": [_P, _P],
    "gb_metric_get_number_of_domain_points": [_P, _P],
    "gb_metric_get_joint_pdf": [_P, _P, _I64],
    "gb_metric_get_mattes_state": [_P, _P],
    "gb_metric_get_stream": [_P, _P],
    "gb_metric_get_device_bytes": [_P, _P],
    "gb_metric_evaluate_device": [_P, _P, _P, _I],
    "gb_metric_synchronize": [_P],
    "gb_msq_affine_noalloc": [_P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _U64],
    "gb_metric_set_profiling": [_P, _I],
    "gb_metric_set_fault_injection": [_P, _I],
    "gb_metric_get_kernel_times": [_P, _P, _I, _P],
    "gb_metric_optimize_regular_step": [_P, _P, _P, _I64, _P],
    "gb_metric_set_optimizer_graphs": [_P, _I],
    "gb_batch_create": [_P, _P],
    "gb_batch_destroy": [_P],
    "gb_batch_add": [_P, _P, _P, _P, _I64, _P],
    "gb_batch_run": [_P, _I64, _P],
    "gb_batch_result": [_P, _I64, _P, _P],
    "gb_batch_set_samples_per_block": [_P, _P],
    "gb_batch_get_samples_per_block": [_P, _P],
    "gb_batch_autotune": [_P, _I, _P],
    "gb_batch_set_graphs": [_P, _I],
    "gb_batch_set_persistent": [_P, _I],
    "gb_batch_get_stats": [_P, _P, _P, _P],
    "gb_sample_count": [_I, _P, _D, _P],
    "gb_sample_points": [_I, _P, _P, _P, _P, _D, ctypes.c_int32, _P, _I64, _P, _P],
}
_RESTYPES = {"gb_last_error": ctypes.c_char_p, "gb_version": ctypes.c_char_p,
             "gb_metric_last_error": ctypes.c_char_p}

_lib = None
_lock = threading.Lock()


class ExceptionObject(RuntimeError):
    """Raised for a non-zero status; mirrors itk::ExceptionObject."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def library_path() -> str:
    return _build.LIB_PATH


def lib():
    """Loads the CUDA library (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            if not os.path.exists(path):
                raise ImportError(f"itk_gb300 CUDA library missing at {path}")
            L = ctypes.CDLL(path)
            for name, args in SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = _RESTYPES.get(name, ctypes.c_int)
            _lib = L
    return _lib


def last_error() -> str:
    msg = lib().gb_last_error()
    return msg.decode() if msg else ""


def metric_last_error(handle) -> str:
    msg = lib().gb_metric_last_error(handle)
    return msg.decode() if msg else ""


def check(rc: int) -> int:
    if rc != GB_OK:
        raise ExceptionObject(rc, last_error() or f"status {rc}")
    return rc


def ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return ctypes.c_void_p(a)
    return a.ctypes.data_as(ctypes.c_void_p)


def f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def i64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64))
