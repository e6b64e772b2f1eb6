"""ctypes binding of the C ABI declared in include/clode_gb300.h.

The library is loaded from the package's in-tree build directory
(``clode_gb300/_build/libclode_gb300.so``; ``python -m clode_gb300.build``
makes it).  There is no fallback: importing this module without the library
raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import library_path

CLODE_OK = 0
ERROR_NAMES = {
    1: "invalid argument", 2: "CUDA error", 3: "program build error", 4: "program not built",
    5: "no CUDA device", 6: "out of memory", 7: "invalid state", 8: "internal error",
}

# enum values of include/clode_gb300.h
SIM_BASE, SIM_FEATURES, SIM_TRAJECTORY = 0, 1, 2
ARRAY_X0, ARRAY_XF, ARRAY_DT, ARRAY_TF, ARRAY_PARS, ARRAY_TSPAN = 0, 1, 2, 3, 4, 5
ARRAY_F, ARRAY_T, ARRAY_X, ARRAY_DX, ARRAY_AUX = 6, 7, 8, 9, 10
ARRAY_EVENT_T, ARRAY_EVENT_X, ARRAY_EVENT_DX, ARRAY_EVENT_AUX = 11, 12, 13, 14
STRING_PROGRAM, STRING_FEATURE_NAMES, STRING_AVAILABLE_STEPPERS = 0, 1, 2
STRING_AVAILABLE_OBSERVERS, STRING_OBSERVER_NAME, STRING_STEPPER = 3, 4, 5
STRING_STATUS_REPORT, STRING_BUILD_LOG = 6, 7
STAT_STEPS, STAT_REJECTED, STAT_RHS_EVALS, STAT_EVENTS, STAT_COUNT = 0, 1, 2, 3, 8


class ClodeError(RuntimeError):
    """A failed C-ABI call; ``code`` is the CLODE_ERR_* value."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{message} [{ERROR_NAMES.get(code, code)}]")
        self.code = code


class CProblem(C.Structure):
    _fields_ = [("rhs_source", C.c_char_p), ("rhs_name", C.c_char_p), ("n_var", C.c_int), ("n_par", C.c_int),
                ("n_aux", C.c_int), ("n_wiener", C.c_int), ("var_names", C.c_char_p), ("par_names", C.c_char_p),
                ("aux_names", C.c_char_p)]


class CSolverParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("dtmax", C.c_double), ("abstol", C.c_double), ("reltol", C.c_double),
                ("max_steps", C.c_uint), ("max_store", C.c_uint), ("nout", C.c_uint)]


class CObserverParams(C.Structure):
    _fields_ = [("e_var_ix", C.c_uint), ("f_var_ix", C.c_uint), ("max_event_count", C.c_uint),
                ("max_event_timestamps", C.c_uint), ("min_x_amp", C.c_double), ("min_imi", C.c_double),
                ("nhood_radius", C.c_double), ("x_up_thresh", C.c_double), ("x_down_thresh", C.c_double),
                ("dx_up_thresh", C.c_double), ("dx_down_thresh", C.c_double), ("eps_dx", C.c_double)]


class CDeviceInfo(C.Structure):
    _fields_ = [("name", C.c_char * 256), ("vendor", C.c_char * 64), ("version", C.c_char * 64),
                ("ordinal", C.c_int), ("compute_units", C.c_int), ("cc_major", C.c_int), ("cc_minor", C.c_int),
                ("max_clock_mhz", C.c_int), ("max_work_group_size", C.c_int), ("double_support", C.c_int),
                ("device_memory_size", C.c_ulonglong), ("max_memory_alloc_size", C.c_ulonglong)]


class CSizes(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("n_pts", "n_var", "n_par", "n_aux", "n_wiener", "n_features",
                                             "max_store", "t_elements", "x_elements", "aux_elements",
                                             "n_store_var", "n_store_aux", "event_rows")]


LOG_SINK = C.CFUNCTYPE(None, C.c_int, C.c_char_p)

_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_SIZE = C.c_size_t

# name -> (restype, argtypes); every symbol declared in include/clode_gb300.h
SIGNATURES = {
    "clode_last_error": (C.c_char_p, []),
    "clode_version": (C.c_int, []),
    "clode_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "clode_device_query": (C.c_int, [C.c_int, C.POINTER(CDeviceInfo)]),
    "clode_log_set_level": (C.c_int, [C.c_int]),
    "clode_log_get_level": (C.c_int, []),
    "clode_log_set_pattern": (C.c_int, [C.c_char_p]),
    "clode_log_set_sink": (C.c_int, [LOG_SINK]),
    "clode_log_message": (C.c_int, [C.c_int, C.c_char_p]),
    "clode_set_cache_dir": (C.c_int, [C.c_char_p]),
    "clode_sim_create": (C.c_int, [C.c_int, C.POINTER(CProblem), C.c_char_p, C.c_char_p,
                                   C.POINTER(CObserverParams), C.c_int, C.c_int, C.POINTER(_P)]),
    "clode_sim_destroy": (C.c_int, [_P]),
    "clode_sim_set_problem_info": (C.c_int, [_P, C.POINTER(CProblem)]),
    "clode_sim_set_stepper": (C.c_int, [_P, C.c_char_p]),
    "clode_sim_set_precision": (C.c_int, [_P, C.c_int]),
    "clode_sim_set_device": (C.c_int, [_P, C.c_int]),
    "clode_sim_set_observer": (C.c_int, [_P, C.c_char_p]),
    "clode_sim_build": (C.c_int, [_P]),
    "clode_sim_set_problem_data": (C.c_int, [_P, _DP, _SIZE, _DP, _SIZE]),
    "clode_sim_set_x0": (C.c_int, [_P, _DP, _SIZE]),
    "clode_sim_set_pars": (C.c_int, [_P, _DP, _SIZE]),
    "clode_sim_set_tspan": (C.c_int, [_P, _DP]),
    "clode_sim_set_solver_params": (C.c_int, [_P, C.POINTER(CSolverParams)]),
    "clode_sim_get_solver_params": (C.c_int, [_P, C.POINTER(CSolverParams)]),
    "clode_sim_set_observer_params": (C.c_int, [_P, C.POINTER(CObserverParams)]),
    "clode_sim_get_observer_params": (C.c_int, [_P, C.POINTER(CObserverParams)]),
    "clode_sim_seed_rng": (C.c_int, [_P, C.c_int, C.c_int]),
    "clode_sim_transient": (C.c_int, [_P]),
    "clode_sim_initialize_observer": (C.c_int, [_P]),
    "clode_sim_features": (C.c_int, [_P, C.c_int]),
    "clode_sim_is_observer_initialized": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "clode_sim_trajectory": (C.c_int, [_P]),
    "clode_sim_shift_tspan": (C.c_int, [_P]),
    "clode_sim_shift_x0": (C.c_int, [_P]),
    "clode_sim_get_sizes": (C.c_int, [_P, C.POINTER(CSizes)]),
    "clode_sim_get": (C.c_int, [_P, C.c_int, _DP, _SIZE, C.POINTER(_SIZE)]),
    "clode_sim_get_n_stored": (C.c_int, [_P, C.POINTER(C.c_int), _SIZE, C.POINTER(_SIZE)]),
    "clode_sim_get_string": (C.c_int, [_P, C.c_int, C.c_char_p, _SIZE, C.POINTER(_SIZE)]),
    "clode_sim_set_tspan_per_member": (C.c_int, [_P, _DP, _SIZE]),
    "clode_sim_get_status": (C.c_int, [_P, C.POINTER(C.c_int), _SIZE, C.POINTER(_SIZE)]),
    "clode_sim_features_store": (C.c_int, [_P, C.c_int, C.c_uint]),
    "clode_sim_get_n_events": (C.c_int, [_P, C.POINTER(C.c_int), _SIZE, C.POINTER(_SIZE)]),
    "clode_sim_set_store_variables": (C.c_int, [_P, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.c_int]),
    "clode_sim_get_events_by_member": (C.c_int, [_P, C.c_longlong, C.c_longlong, C.c_longlong, _DP, _DP, _DP, _DP,
                                                 C.POINTER(C.c_int)]),
    "clode_sim_get_trajectory_by_member": (C.c_int, [_P, C.c_longlong, C.c_longlong, C.c_longlong, _DP, _DP, _DP,
                                                     _DP, C.POINTER(C.c_int)]),
    "clode_sim_get_rng_state": (C.c_int, [_P, C.POINTER(C.c_ulonglong), _SIZE, C.POINTER(_SIZE)]),
    "clode_sim_set_rng_state": (C.c_int, [_P, C.POINTER(C.c_ulonglong), _SIZE]),
    "clode_sim_get_stats": (C.c_int, [_P, C.POINTER(C.c_ulonglong)]),
    "clode_sim_last_kernel_ms": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "clode_sim_set_option": (C.c_int, [_P, C.c_char_p, C.c_double]),
    "clode_sim_get_option": (C.c_int, [_P, C.c_char_p, C.POINTER(C.c_double)]),
    "clode_sim_kernel_info": (C.c_int, [_P, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "clode_launch_count": (C.c_ulonglong, []),
    "clode_rng_jump": (C.c_int, [C.c_ulonglong, C.c_ulonglong, C.c_ulonglong, C.POINTER(C.c_ulonglong),
                                 C.POINTER(C.c_ulonglong)]),
    "clode_sim_features_noalloc": (C.c_int, [_P, C.c_longlong, _P, _P, _P, C.POINTER(C.c_ulonglong), _P, _P, _P,
                                             _P, C.POINTER(C.c_int), _P]),
    "clode_sim_autotune": (C.c_int, [_P, C.c_longlong, C.POINTER(C.c_double)]),
    "clode_sim_chain": (C.c_int, [_P, C.POINTER(C.c_int), C.c_int, C.c_int]),
    "clode_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(_P)]),
    "clode_mlp_destroy": (C.c_int, [_P]),
    "clode_mlp_param_count": (C.c_int, [_P, C.POINTER(_SIZE)]),
    "clode_mlp_get_params": (C.c_int, [_P, C.POINTER(C.c_float), _SIZE]),
    "clode_mlp_set_params": (C.c_int, [_P, C.POINTER(C.c_float), _SIZE]),
    "clode_mlp_gradients": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int,
                                      C.POINTER(C.c_float), _SIZE, C.POINTER(C.c_float)]),
    "clode_mlp_train": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_longlong, C.c_int, C.c_int,
                                  C.c_float, C.c_ulonglong, C.POINTER(C.c_float)]),
    "clode_mlp_predict": (C.c_int, [_P, C.POINTER(C.c_float), C.c_longlong, C.POINTER(C.c_float),
                                    C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "clode_mlp_predict_grid": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                          C.POINTER(C.c_float)]),
    "clode_mlp_screen": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(C.c_int)]),
    "clode_mlp_timings": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
}


def _load() -> C.CDLL:
    path = os.environ.get("CLODE_GB300_LIBRARY") or library_path()
    if not os.path.exists(path):
        raise ImportError(f"native library not built: {path} (run `python -m clode_gb300.build`)")
    lib = C.CDLL(path, mode=C.RTLD_GLOBAL)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(rc: int) -> None:
    if rc != CLODE_OK:
        raise ClodeError(rc, lib.clode_last_error().decode(errors="replace"))


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def as_f64(values) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(values, dtype=np.float64).ravel())
