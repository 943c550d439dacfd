"""ctypes binding of libgwgpu.so (include/gwgpu.h).

The library is built in-tree by ``libgwmodel_gb300.build``.  There is no
fallback: if the library cannot be loaded, or a call needs a GPU that is not
there, the call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgwgpu.so")

OK, ERR_INVALID, ERR_CUDA, ERR_NOT_SPD, ERR_RUNTIME, ERR_RANGE, ERR_TIMEOUT, ERR_REJECTED = range(8)

_lock = threading.Lock()
_lib = None


class GwgpuError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[gwgpu error {code}] {message}")
        self.code = code


class Telegram(ctypes.Structure):
    PRINT = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p)
    PROGRESS = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_char_p,
                                ctypes.c_char_p)
    PERCENT = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_double, ctypes.c_char_p, ctypes.c_char_p)
    STOP = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p)
    _fields_ = [("user", ctypes.c_void_p), ("print", PRINT), ("progress", PROGRESS),
                ("progress_percent", PERCENT), ("stop", STOP)]


class Stats(ctypes.Structure):
    _fields_ = [("criterion_evals", ctypes.c_int), ("contract_launches", ctypes.c_int),
                ("contract_ms", ctypes.c_double), ("contract_flops", ctypes.c_double),
                ("contract_bytes", ctypes.c_double), ("select_launches", ctypes.c_int),
                ("select_ms", ctypes.c_double), ("kernel_launches", ctypes.c_longlong),
                ("contract_tiles", ctypes.c_longlong), ("contract_phase_cycles", ctypes.c_double * 12),
                ("d2c_fills", ctypes.c_int), ("d2c_fill_ms", ctypes.c_double)]


class Request(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("p", ctypes.c_int), ("coords", ctypes.POINTER(ctypes.c_double)),
                ("x", ctypes.POINTER(ctypes.c_double)), ("y", ctypes.POINTER(ctypes.c_double)),
                ("geographic", ctypes.c_int), ("kind", ctypes.c_int), ("adaptive", ctypes.c_int),
                ("kernel", ctypes.c_int), ("criterion", ctypes.c_int), ("bandwidth", ctypes.c_double),
                ("precision", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("slot", ctypes.c_int), ("evaluations", ctypes.c_int),
                ("bandwidth", ctypes.c_double), ("aicc", ctypes.c_double), ("rss", ctypes.c_double),
                ("shat", ctypes.c_double * 2), ("submit_ms", ctypes.c_double), ("start_ms", ctypes.c_double),
                ("end_ms", ctypes.c_double), ("error", ctypes.c_char * 160)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong), ("failed", ctypes.c_longlong),
                ("rejected", ctypes.c_longlong), ("running", ctypes.c_longlong), ("queued", ctypes.c_longlong),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("first_start_ms", ctypes.c_double), ("last_end_ms", ctypes.c_double),
                ("local_fits", ctypes.c_double), ("reserved_bytes", ctypes.c_double),
                ("peak_reserved_bytes", ctypes.c_double), ("max_concurrent", ctypes.c_int)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("problems", ctypes.c_int), ("segments", ctypes.c_int), ("flush_tiles", ctypes.c_int),
                ("order", ctypes.c_int), ("solve_rows", ctypes.c_int), ("select_ctas", ctypes.c_int),
                ("tuned", ctypes.c_int), ("tuned_ms", ctypes.c_double), ("last_ms", ctypes.c_double),
                ("graph", ctypes.c_int), ("launches_per_evaluate", ctypes.c_int), ("contract_ctas", ctypes.c_int),
                ("rows_total", ctypes.c_double)]


# (name, restype, argtypes) of every function declared in include/gwgpu.h
_vp, _ip, _dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
_i, _d, _sz = ctypes.c_int, ctypes.c_double, ctypes.c_size_t
SIGNATURES = [
    ("gwgpu_version", _i, []),
    ("gwgpu_last_error", ctypes.c_char_p, []),
    ("gwgpu_device_count", _i, [_ip]),
    ("gwgpu_gwr_create", _i, [ctypes.POINTER(_vp)]),
    ("gwgpu_gwr_destroy", None, [_vp]),
    ("gwgpu_gwr_set_coords", _i, [_vp, _i, _dp]),
    ("gwgpu_gwr_set_dependent_variable", _i, [_vp, _i, _dp]),
    ("gwgpu_gwr_set_independent_variables", _i, [_vp, _i, _i, _dp]),
    ("gwgpu_gwr_set_spatial_weight", _i, [_vp, _d, _i, _i, _i]),
    ("gwgpu_gwr_set_is_autoselect_bandwidth", _i, [_vp, _i]),
    ("gwgpu_gwr_set_bandwidth_selection_criterion", _i, [_vp, _i]),
    ("gwgpu_gwr_set_golden_upper_bounds", _i, [_vp, _d]),
    ("gwgpu_gwr_set_golden_lower_bounds", _i, [_vp, _d]),
    ("gwgpu_gwr_set_has_hat_matrix", _i, [_vp, _i]),
    ("gwgpu_gwr_set_has_intercept", _i, [_vp, _i]),
    ("gwgpu_gwr_set_is_autoselect_indep_vars", _i, [_vp, _i]),
    ("gwgpu_gwr_set_indep_var_selection_threshold", _i, [_vp, _d]),
    ("gwgpu_gwr_set_parallel_type", _i, [_vp, _i]),
    ("gwgpu_gwr_set_omp_thread_num", _i, [_vp, _i]),
    ("gwgpu_gwr_set_gpu_id", _i, [_vp, _i]),
    ("gwgpu_gwr_set_group_size", _i, [_vp, _sz]),
    ("gwgpu_gwr_set_precision", _i, [_vp, _i]),
    ("gwgpu_gwr_set_telegram", _i, [_vp, ctypes.POINTER(Telegram)]),
    ("gwgpu_gwr_fit", _i, [_vp]),
    ("gwgpu_gwr_predict", _i, [_vp, _i, _dp, _dp]),
    ("gwgpu_gwr_status", _i, [_vp]),
    ("gwgpu_gwr_shape", _i, [_vp, _ip, _ip, _ip]),
    ("gwgpu_gwr_betas", _i, [_vp, _dp]),
    ("gwgpu_gwr_betas_se", _i, [_vp, _dp]),
    ("gwgpu_gwr_shat", _i, [_vp, _dp]),
    ("gwgpu_gwr_qdiag", _i, [_vp, _dp]),
    ("gwgpu_gwr_s", _i, [_vp, _dp]),
    ("gwgpu_gwr_diagnostic", _i, [_vp, _dp]),
    ("gwgpu_gwr_bandwidth", _i, [_vp, _dp]),
    ("gwgpu_gwr_bandwidth_criterion_list", _i, [_vp, _ip, _dp, _dp]),
    ("gwgpu_gwr_selected_vars", _i, [_vp, _ip, _ip]),
    ("gwgpu_gwr_var_criterion_list", _i, [_vp, _ip, _ip, _ip, _ip, _dp]),
    ("gwgpu_csv_read", _i, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
    ("gwgpu_table_shape", _i, [_vp, _ip, _ip]),
    ("gwgpu_table_column_name", ctypes.c_char_p, [_vp, _i]),
    ("gwgpu_table_columns", _i, [_vp, _i, ctypes.POINTER(ctypes.c_char_p), _dp]),
    ("gwgpu_table_destroy", None, [_vp]),
    ("gwgpu_mgwr_create", _i, [ctypes.POINTER(_vp)]),
    ("gwgpu_mgwr_destroy", None, [_vp]),
    ("gwgpu_mgwr_set_coords", _i, [_vp, _i, _dp]),
    ("gwgpu_mgwr_set_dependent_variable", _i, [_vp, _i, _dp]),
    ("gwgpu_mgwr_set_independent_variables", _i, [_vp, _i, _i, _dp]),
    ("gwgpu_mgwr_set_spatial_weights", _i, [_vp, _i, _dp, _ip, _ip, _i]),
    ("gwgpu_mgwr_set_bandwidth_initilize", _i, [_vp, _i, _ip]),
    ("gwgpu_mgwr_set_bandwidth_selection_approach", _i, [_vp, _i, _ip]),
    ("gwgpu_mgwr_set_preditor_centered", _i, [_vp, _i, _ip]),
    ("gwgpu_mgwr_set_bandwidth_select_threshold", _i, [_vp, _i, _dp]),
    ("gwgpu_mgwr_set_bandwidth_select_retry_times", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_max_iteration", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_criterion_type", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_criterion_threshold", _i, [_vp, _d]),
    ("gwgpu_mgwr_set_adaptive_lower", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_golden_upper_bounds", _i, [_vp, _d]),
    ("gwgpu_mgwr_set_golden_lower_bounds", _i, [_vp, _d]),
    ("gwgpu_mgwr_set_has_hat_matrix", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_has_intercept", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_parallel_type", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_gpu_id", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_precision", _i, [_vp, _i]),
    ("gwgpu_mgwr_set_telegram", _i, [_vp, ctypes.POINTER(Telegram)]),
    ("gwgpu_mgwr_fit", _i, [_vp]),
    ("gwgpu_mgwr_status", _i, [_vp]),
    ("gwgpu_mgwr_betas", _i, [_vp, _dp]),
    ("gwgpu_mgwr_betas_se", _i, [_vp, _dp]),
    ("gwgpu_mgwr_betas_tv", _i, [_vp, _dp]),
    ("gwgpu_mgwr_bandwidths", _i, [_vp, _dp]),
    ("gwgpu_mgwr_diagnostic", _i, [_vp, _dp]),
    ("gwgpu_mgwr_info", _i, [_vp, _dp, _ip]),
    ("gwgpu_mgwr_counters", _i, [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), _dp]),
    ("gwgpu_engine_create", _i, [_i, ctypes.POINTER(_vp)]),
    ("gwgpu_engine_destroy", None, [_vp]),
    ("gwgpu_engine_set_data", _i, [_vp, _i, _i, _dp, _dp, _dp, _i]),
    ("gwgpu_engine_set_precision", _i, [_vp, _i]),
    ("gwgpu_engine_set_flush_tiles", _i, [_vp, _i]),
    ("gwgpu_engine_set_tc_wait_limit", _i, [_vp, ctypes.c_uint]),
    ("gwgpu_engine_set_refinement", _i, [_vp, _i, _i]),
    ("gwgpu_engine_criterion", _i, [_vp, _d, _i, _i, _i, _dp]),
    ("gwgpu_engine_global_criterion", _i, [_vp, _i, _ip, _dp]),
    ("gwgpu_engine_fit", _i, [_vp, _d, _i, _i, _i, _dp, _dp, _dp, _dp, _dp]),
    ("gwgpu_engine_max_distance", _i, [_vp, _dp]),
    ("gwgpu_engine_golden", _i, [_vp, _i, _i, _i, _d, _d, _dp, _ip, _dp, _dp, _i]),
    ("gwgpu_engine_clear_cache", _i, [_vp]),
    ("gwgpu_engine_set_distance_cache", _i, [_vp, ctypes.c_longlong]),
    ("gwgpu_engine_release_distance_cache", _i, [_vp]),
    ("gwgpu_engine_distance_cache_active", _i, [_vp, _ip]),
    ("gwgpu_engine_predict", _i, [_vp, _i, _dp, _d, _i, _i, _dp]),
    ("gwgpu_engine_event_record", _i, [_vp, _i]),
    ("gwgpu_engine_event_elapsed", _i, [_vp, _i, _i, ctypes.POINTER(ctypes.c_float)]),
    ("gwgpu_engine_thresholds", _i, [_vp, _d, _i, _dp]),
    ("gwgpu_engine_enable_stats", _i, [_vp, _i]),
    ("gwgpu_engine_get_stats", _i, [_vp, ctypes.POINTER(Stats)]),
    ("gwgpu_engine_reset_stats", _i, [_vp]),
    ("gwgpu_criterion_noalloc", _i, [_i, _i, _i, _i, _d, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("gwgpu_server_create", _i, [_i, _d, _i, ctypes.POINTER(_vp)]),
    ("gwgpu_server_destroy", _i, [_vp]),
    ("gwgpu_server_submit", _i, [_vp, ctypes.POINTER(Request), _dp, ctypes.POINTER(ctypes.c_longlong)]),
    ("gwgpu_server_wait", _i, [_vp, ctypes.c_longlong, _d, ctypes.POINTER(Result)]),
    ("gwgpu_server_poll", _i, [_vp, ctypes.c_longlong, _ip]),
    ("gwgpu_server_get_stats", _i, [_vp, ctypes.POINTER(ServerStats)]),
    ("gwgpu_server_estimate", _d, [_vp, ctypes.POINTER(Request)]),
    ("gwgpu_estimate_bytes", _d, [_i, _i, _i, _i, _i]),
    ("gwgpu_admit_slot", _i, [_d, _i, _dp, _ip, _d]),
    ("gwgpu_batch_create", _i, [_i, ctypes.POINTER(_vp)]),
    ("gwgpu_batch_destroy", _i, [_vp]),
    ("gwgpu_batch_set_problems", _i, [_vp, _i, _ip, _ip, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), _ip, _i]),
    ("gwgpu_batch_set_candidates", _i, [_vp, _ip, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), _i, _i, _i]),
    ("gwgpu_batch_evaluate", _i, [_vp, _i, _dp]),
    ("gwgpu_batch_autotune", _i, [_vp, _i]),
    ("gwgpu_batch_set_tuning", _i, [_vp, _i, _i, _i, _i]),
    ("gwgpu_batch_get_info", _i, [_vp, ctypes.POINTER(BatchInfo)]),
    ("gwgpu_engine_tc_selftest", _i, [_vp, _i, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                      ctypes.POINTER(ctypes.c_float)]),
]

# The drop-in factories of include/IGWRBasicGpuTask.h.
TASK_SIGNATURES = [
    ("GWRBasicGpuTaskFit_Create", _vp, [_i, _i, _i]),
    ("GWRBasicGpuTaskPredict_Create", _vp, [_i, _i, _i, _i]),
    ("GWRBasicGpuTask_Del", None, [_vp]),
    ("GWRBasicGpuTask_SetData", _i, [_vp, _dp, _dp, _dp]),
    ("GWRBasicGpuTask_SetPredictLocations", _i, [_vp, _dp]),
    ("GWRBasicGpuTask_GetBetas", _i, [_vp, _dp]),
    ("GWRBasicGpuTask_GetBetasSE", _i, [_vp, _dp]),
]


def lib():
    """Load libgwgpu.so, building it first when it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                from . import build
                build.build()
            L = ctypes.CDLL(LIB_PATH)
            for name, res, args in SIGNATURES + TASK_SIGNATURES:
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(rc: int):
    if rc != OK:
        raise GwgpuError(rc, lib().gwgpu_last_error().decode(errors="replace"))
    return rc


def dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
