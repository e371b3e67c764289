"""ctypes binding of libfwiflow_gb300.so (the C ABI of include/fwiflow_gb300.h).

The library is built in-tree by fwiflow.jl_gb300/build.py. There is no CPU
fallback: if the library is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libfwiflow_gb300.so")

STATUS = {
    0: "OK", 1: "ERR_ARG", 2: "ERR_PARAM", 3: "ERR_COURANT", 4: "ERR_CUDA", 5: "ERR_OOM", 6: "ERR_IO",
    7: "ERR_TIMEOUT", 8: "ERR_UNSUPPORTED",
}


class FwiError(RuntimeError):
    """A C-ABI call returned a non-zero fwigb_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None

_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int)
_V = ctypes.c_void_p

SIGNATURES = {
    "fwigb_create": ([ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_V)], ctypes.c_int),
    "fwigb_destroy": ([_V], ctypes.c_int),
    "fwigb_last_error": ([_V], ctypes.c_char_p),
    "fwigb_last_global_error": ([], ctypes.c_char_p),
    "fwigb_misfit": ([_V, _D, _D, _D, _D, ctypes.c_int, _I, ctypes.c_int, _D], ctypes.c_int),
    "fwigb_misfit_grad": ([_V, _D, _D, _D, _D, ctypes.c_int, _I, ctypes.c_int, _D, _D, _D, _D, _D], ctypes.c_int),
    "fwigb_obs": ([_V, _D, _D, _D, _D, ctypes.c_int, _I, ctypes.c_int, _F, ctypes.c_int], ctypes.c_int),
    "fwigb_misfit_grad_obs": ([_V, _D, _D, _D, _D, ctypes.c_int, _I, ctypes.c_int, _F, _D, _D, _D, _D, _D],
                              ctypes.c_int),
    "fwigb_geometry": ([_V, _I, _I, _I, _I, _I], ctypes.c_int),
    "fwigb_shot_nrec": ([_V, ctypes.c_int, _I], ctypes.c_int),
    "fwigb_shot_info": ([_V, ctypes.c_int, _I, _I, _I, _I], ctypes.c_int),
    "fwigb_cufd": ([_D, _D, _D, _D, _D, _D, _D, _D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int, _I,
                    ctypes.c_char_p], ctypes.c_int),
    "fwigb_set_model": ([_V, _D, _D, _D], ctypes.c_int),
    "fwigb_stage_shots": ([_V, _D, ctypes.c_int, _I, ctypes.c_int, ctypes.c_int, _F], ctypes.c_int),
    "fwigb_run": ([_V, ctypes.c_int], ctypes.c_int),
    "fwigb_fetch": ([_V, _D, _D, _D, _D, _D, _F], ctypes.c_int),
    "fwigb_synchronize": ([_V], ctypes.c_int),
    "fwigb_stream": ([_V], _V),
    "fwigb_last_launch_count": ([_V], ctypes.c_longlong),
    "fwigb_set_kernel_timing": ([_V, ctypes.c_int], ctypes.c_int),
    "fwigb_tile_config": ([_V, _I], ctypes.c_int),
    "fwigb_tile_rows": ([_V, _I], ctypes.c_int),
    "fwigb_tile_registers": ([_V, _I], ctypes.c_int),
    "fwigb_set_tile_registers": ([_V, _I], ctypes.c_int),
    "fwigb_set_tile_rows": ([_V, _I], ctypes.c_int),
    "fwigb_set_graphs": ([_V, ctypes.c_int], ctypes.c_int),
    "fwigb_sweep_time": ([_V, ctypes.c_int, ctypes.c_int, _D], ctypes.c_int),
    "fwigb_set_batching": ([_V, ctypes.c_int, ctypes.c_ulonglong], ctypes.c_int),
    "fwigb_last_group_count": ([_V], ctypes.c_int),
    "fwigb_set_illumination": ([_V, ctypes.c_int], ctypes.c_int),
    "fwigb_misfit_gathers_noalloc": ([_V, _V, _V, ctypes.c_int, ctypes.c_int, ctypes.c_float, _D, _V], ctypes.c_int),
    "fwigb_noalloc_last_error": ([], ctypes.c_char_p),
    "fwigb_test_inject_wait_timeout": ([_V, ctypes.c_int], ctypes.c_int),
    "fwigb_fetch_illumination": ([_V, _D], ctypes.c_int),
    "fwigb_cnn_conv3x3": ([_V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _V, _V, _V, _V,
                           _V, _V, _V], ctypes.c_int),
    "fwigb_cnn_tile_count": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "fwigb_cnn_conv3x3_tc": ([_V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _V, _V, _V, _V, _V, _V,
                              _V], ctypes.c_int),
    "fwigb_cnn_pack_weights_tc": ([_V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _V,
                                   _V], ctypes.c_int),
    "fwigb_cnn_wgrad_partials": ([_V, _V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _V, _V],
                                 ctypes.c_int),
    "fwigb_cnn_reduce_partials": ([_V, ctypes.c_int, ctypes.c_int, _V, _V], ctypes.c_int),
    "fwigb_cnn_bias_partials": ([_V, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, _V, _V], ctypes.c_int),
    "fwigb_cnn_adam": ([_V, _V, _V, _V, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                        ctypes.c_float, ctypes.c_int, _V], ctypes.c_int),
    "fwigb_cnn_pack_weights": ([_V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _V, _V],
                               ctypes.c_int),
    "fwigb_cnn_mse_grad": ([_V, _V, _V, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_float, _V, _V, _V],
                           ctypes.c_int),
    "fwigb_set_tile_config": ([_V, _I], ctypes.c_int),
    "fwigb_kernel_times": ([_V, _D, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
}


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the library (once). Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with fwiflow.jl_gb300/build.py (no CPU fallback exists)")
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_D) if a is not None else None


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_F) if a is not None else None


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_I) if a is not None else None


def check(rc: int, ctx=None) -> None:
    if rc != 0:
        lib = load()
        msg = lib.fwigb_last_error(ctx) if ctx else lib.fwigb_last_global_error()
        raise FwiError(rc, (msg or b"").decode(errors="replace"))
