"""ctypes binding of the C ABI in include/heomgb.h.

The shared library is built in-tree (libheom_gb300/_lib/libheomgb.so).  There
is no CPU fallback: if the library is missing or cannot be loaded, every entry
point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

OK = 0
STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "STATE", 3: "CUDA", 4: "ALLOC", 5: "UNSUPPORTED", 6: "NUMERIC",
          7: "CAPACITY"}

c_int_p = ctypes.POINTER(ctypes.c_int)
c_ll_p = ctypes.POINTER(ctypes.c_longlong)
c_double_p = ctypes.POINTER(ctypes.c_double)
CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_double, ctypes.c_void_p)
HRCHY_FILTER = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                ctypes.c_void_p)


class Kwargs(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("atol", ctypes.c_double), ("rtol", ctypes.c_double),
                ("has_dt", ctypes.c_int), ("has_atol", ctypes.c_int), ("has_rtol", ctypes.c_int)]


class HeomError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"heomgb error {STATUS.get(status, status)}: {message}")
        self.status = status


# name -> (restype, argtypes)
SIGNATURES = {
    "heomgb_last_error": (ctypes.c_char_p, []),
    "heomgb_version": (ctypes.c_char_p, []),
    "heomgb_abi_version": (ctypes.c_int, []),
    "heomgb_launch_count": (ctypes.c_longlong, []),
    "heomgb_qme_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "heomgb_qme_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "heomgb_qme_set_hamiltonian": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "heomgb_qme_alloc_noises": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "heomgb_qme_set_noise": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p]),
    "heomgb_qme_set_precision": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "heomgb_qme_set_normalization": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "heomgb_qme_set_order": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "heomgb_qme_set_hrchy_filter": (ctypes.c_int, [ctypes.c_void_p, HRCHY_FILTER, ctypes.c_void_p]),
    "heomgb_qme_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "heomgb_qme_get_precision": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_double_p, c_double_p]),
    "heomgb_qme_set_param": (ctypes.c_int, [ctypes.c_void_p]),
    "heomgb_qme_get_n_hrchy": (ctypes.c_int, [ctypes.c_void_p, c_int_p]),
    "heomgb_qme_get_n_dim": (ctypes.c_int, [ctypes.c_void_p, c_int_p]),
    "heomgb_qme_main_size": (ctypes.c_int, [ctypes.c_void_p, c_ll_p]),
    "heomgb_qme_get_hrchy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "heomgb_qme_calc_diff": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "heomgb_qme_calc_diff_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p, ctypes.c_void_p]),
    "heomgb_solver_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "heomgb_solver_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "heomgb_qme_solver_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "heomgb_qme_solver_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "heomgb_batch_solver_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                  ctypes.POINTER(ctypes.c_void_p)]),
    "heomgb_qme_solver_main_size": (ctypes.c_int, [ctypes.c_void_p, c_ll_p]),
    "heomgb_qme_solver_tuning": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "heomgb_qme_solver_tensor_cores": (ctypes.c_int, [ctypes.c_void_p, c_int_p]),
    "heomgb_qme_solver_site_kernel": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p]),
    "heomgb_qme_solver_resident": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p]),
    "heomgb_qme_solver_local": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p]),
    "heomgb_qme_solver_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                               CALLBACK, ctypes.c_void_p, ctypes.POINTER(Kwargs)]),
    "heomgb_qme_solver_solve_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.c_int, CALLBACK, ctypes.c_void_p,
                                                      ctypes.POINTER(Kwargs)]),
    "heomgb_qme_solver_stats": (ctypes.c_int, [ctypes.c_void_p, c_ll_p, c_ll_p, c_ll_p, c_double_p]),
    "heomgb_qme_solver_timing": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_ll_p]),
    "heomgb_probe_fma_peaks": (ctypes.c_int, [c_double_p, c_double_p]),
    "heomgb_mlp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "heomgb_mlp_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "heomgb_mlp_sizes": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_ll_p]),
    "heomgb_mlp_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "heomgb_mlp_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "heomgb_mlp_set_loss": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "heomgb_mlp_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "heomgb_mlp_gradients": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "heomgb_mlp_train_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_float, ctypes.POINTER(ctypes.c_float)]),
    "heomgb_qme_set_terminator": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "heomgb_hrchy_build_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, c_int_p, ctypes.c_void_p]),
    "heomgb_errnrm1_scratch": (ctypes.c_size_t, [ctypes.c_longlong]),
    "heomgb_errnrm1_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                             ctypes.c_double, ctypes.c_longlong, ctypes.c_void_p, c_double_p,
                                             ctypes.c_void_p]),
}

_LIB = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it first if it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise FileNotFoundError(f"CUDA library {path} is missing; run libheom_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        msg = load().heomgb_last_error()
        raise HeomError(status, msg.decode() if msg else "")


def launch_count() -> int:
    return int(load().heomgb_launch_count())


def probe_fma_peaks():
    """(FP64, FP32) FMA throughput of the current GPU in TFLOP/s."""
    a, b = ctypes.c_double(), ctypes.c_double()
    check(load().heomgb_probe_fma_peaks(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value
