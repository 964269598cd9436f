"""Loader of libdtsgb.so, the CUDA product library (C ABI in include/dtsgb.h).

There is no fallback: if the library is missing or fails to load, importing
the package raises, so a GPU run can never silently compute on the CPU.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libdtsgb.so"
HEADER = PKG.parent / "include" / "dtsgb.h"

DTSGB_OK = 0
DTSGB_ERR_INVALID_ARGUMENT = 1
DTSGB_ERR_INVALID_DIMS = 2
DTSGB_ERR_UNSUPPORTED = 3
DTSGB_ERR_CUDA = 4
DTSGB_ERR_OUT_OF_MEMORY = 5
DTSGB_ERR_TOO_SMALL = 6
DTSGB_WARN_GRID_TOO_LARGE = 100


class DtsgbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"dtsgb status {status}: {msg}")
        self.status = status


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = ctypes.CDLL(str(LIB_PATH))
        _declare(lib)
        _lib = lib
    return _lib


def declared_symbols() -> list[str]:
    """Names of every entry point include/dtsgb.h declares."""
    text = HEADER.read_text()
    return re.findall(r"DTSGB_API\s+[^;(]*?\b(dtsgb_\w+)\s*\(", text)


class FilterParams(ctypes.Structure):
    _fields_ = [("sigma_x", ctypes.c_float), ("sigma_y", ctypes.c_float),
                ("sigma_r", ctypes.c_float)]


class ConfParams(ctypes.Structure):
    _fields_ = [("sigma_x", ctypes.c_float), ("sigma_y", ctypes.c_float),
                ("sigma_r", ctypes.c_float), ("sigmas", ctypes.c_float * 2)]


class OptimizeParams(ctypes.Structure):
    _fields_ = [("num_iterations", ctypes.c_int), ("loss", ctypes.c_int),
                ("lambda_", ctypes.c_float), ("sigma_z", ctypes.c_float),
                ("step_size", ctypes.c_float),
                ("photo_consis_lambda", ctypes.c_float),
                ("DT_lambda", ctypes.c_float)]


class HfbsParams(ctypes.Structure):
    _fields_ = [("sigma_x", ctypes.c_float), ("sigma_y", ctypes.c_float),
                ("sigma_l", ctypes.c_float), ("lambda_", ctypes.c_float),
                ("alpha", ctypes.c_float), ("beta", ctypes.c_float),
                ("bistoch_iter_max", ctypes.c_int),
                ("optim_iter_max", ctypes.c_int),
                ("neg_exp_beta", ctypes.c_float), ("grid_x", ctypes.c_int),
                ("grid_y", ctypes.c_int), ("grid_l", ctypes.c_int)]


def _declare(lib: ctypes.CDLL) -> None:
    vp, i, f, u = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint
    ll = ctypes.c_longlong
    pvp = ctypes.POINTER(ctypes.c_void_p)
    P = ctypes.POINTER
    sig = {
        "dtsgb_last_error": ([], ctypes.c_char_p),
        "dtsgb_version": ([], i),
        "dtsgb_dts_create": ([i, i, u, pvp], i),
        "dtsgb_dts_destroy": ([vp], i),
        "dtsgb_dts_set_stream": ([vp, vp], i),
        "dtsgb_dts_set_image_dim": ([vp, i, i], i),
        "dtsgb_dts_init_frame": ([vp, i, vp, vp, vp], i),
        "dtsgb_dts_init_frame_device": ([vp, i, vp, vp, vp], i),
        "dtsgb_dts_upload_targets": ([vp, vp, vp], i),
        "dtsgb_dts_upload_targets_device": ([vp, vp, vp], i),
        "dtsgb_dts_compute_differential": ([vp, P(FilterParams)], i),
        "dtsgb_dts_integrate": ([vp], i),
        "dtsgb_dts_filter": ([vp, P(FilterParams), vp, vp, i], i),
        "dtsgb_dts_compute_confidence": ([vp, P(ConfParams), i], i),
        "dtsgb_dts_optimize": ([vp, P(OptimizeParams), f], i),
        "dtsgb_dts_download": ([vp, i, vp], i),
        "dtsgb_dts_download_device": ([vp, i, vp], i),
        "dtsgb_dts_clear_all": ([vp], i),
        "dtsgb_dts_debug_bounds": ([vp, i, f, vp, vp], i),
        "dtsgb_debug_color_convert": ([i, vp, vp, ll], i),
        "dtsgb_hfbs_create": ([i, i, i, i, i, u, pvp], i),
        "dtsgb_hfbs_destroy": ([vp], i),
        "dtsgb_hfbs_set_stream": ([vp, vp], i),
        "dtsgb_hfbs_set_image_dim": ([vp, i, i], i),
        "dtsgb_hfbs_init_frame": ([vp, i, vp, vp, vp], i),
        "dtsgb_hfbs_init_frame_device": ([vp, i, vp, vp, vp], i),
        "dtsgb_hfbs_upload_targets": ([vp, vp, vp], i),
        "dtsgb_hfbs_upload_targets_device": ([vp, vp, vp], i),
        "dtsgb_hfbs_set_filter_params": ([vp, P(HfbsParams)], i),
        "dtsgb_hfbs_clear_all": ([vp], i),
        "dtsgb_hfbs_optimize": ([vp], i),
        "dtsgb_hfbs_download": ([vp, i, vp], i),
        "dtsgb_hfbs_download_device": ([vp, i, vp], i),
        "dtsgb_hfbs_grid_dims": ([vp, P(i), P(i), P(i)], i),
        "dtsgb_dts_synchronize": ([vp], i),
        "dtsgb_hfbs_synchronize": ([vp], i),
        "dtsgb_hfbs_debug_grid": ([vp, i, vp], i),
        "dtsgb_hfbs_enable_grad": ([vp, i, i], i),
        "dtsgb_hfbs_grad_info": ([vp, ctypes.POINTER(i), ctypes.POINTER(i)], i),
        "dtsgb_hfbs_backward": ([vp, vp, vp, vp], i),
        "dtsgb_hfbs_backward_device": ([vp, vp, vp, vp], i),
        "dtsgb_wait_timeouts": ([P(ctypes.c_ulonglong)], i),
        "dtsgb_profile_enable": ([i], i),
        "dtsgb_profile_reset": ([], i),
        "dtsgb_profile_read": ([i, P(i), P(ctypes.c_double)], i),
        "dtsgb_batch_create": ([i, P(i), P(i), u, pvp], i),
        "dtsgb_batch_destroy": ([vp], i),
        "dtsgb_batch_set_stream": ([vp, vp], i),
        "dtsgb_batch_use_graphs": ([vp, i], i),
        "dtsgb_batch_upload": ([vp, i, pvp, pvp, pvp], i),
        "dtsgb_batch_upload_device": ([vp, i, pvp, pvp, pvp], i),
        "dtsgb_batch_upload_targets": ([vp, pvp, pvp], i),
        "dtsgb_batch_upload_targets_device": ([vp, pvp, pvp], i),
        "dtsgb_batch_solve_dts": ([vp, P(FilterParams), P(OptimizeParams), f], i),
        "dtsgb_batch_solve_hfbs": ([vp, P(HfbsParams)], i),
        "dtsgb_batch_download": ([vp, i, pvp], i),
        "dtsgb_batch_download_device": ([vp, i, pvp], i),
        "dtsgb_batch_debug_plane": ([vp, i, i, vp, ll], i),
        "dtsgb_batch_set_tuning": ([vp, i, ll], i),
        "dtsgb_batch_get_tuning": ([vp, i, P(ll)], i),
        "dtsgb_batch_autotune": ([vp, P(FilterParams), P(OptimizeParams), f,
                                  P(HfbsParams), i], i),
        "dtsgb_batch_autotune_cached": ([vp, P(FilterParams), P(OptimizeParams), f,
                                         P(HfbsParams), i, ctypes.c_char_p, P(i)], i),
        "dtsgb_pipeline_create": ([i, P(i), P(i), u, i, pvp], i),
        "dtsgb_pipeline_destroy": ([vp], i),
        "dtsgb_pipeline_chunks": ([vp], i),
        "dtsgb_pipeline_batch": ([vp, i, pvp], i),
        "dtsgb_pipeline_run": ([vp, i, pvp, pvp, pvp, P(FilterParams), P(OptimizeParams), f,
                                P(HfbsParams), pvp, pvp], i),
        "dtsgb_pipeline_run_grad": ([vp, i, pvp, pvp, pvp, P(FilterParams), P(OptimizeParams),
                                     pvp, pvp, pvp, pvp], i),
        "dtsgb_batch_enable_grad": ([vp, i, i], i),
        "dtsgb_png_unfilter": ([vp, i, i, i, vp], i),
        "dtsgb_batch_grad_info": ([vp, P(i), P(i)], i),
        "dtsgb_batch_dts_backward": ([vp, pvp, pvp, pvp], i),
        "dtsgb_batch_dts_backward_device": ([vp, pvp, pvp, pvp], i),
        "dtsgb_batch_hfbs_backward": ([vp, pvp, pvp, pvp], i),
        "dtsgb_batch_hfbs_backward_device": ([vp, pvp, pvp, pvp], i),
        "dtsgb_batch_hfbs_grad_info": ([vp, ctypes.POINTER(i), ctypes.POINTER(i)], i),
        "dtsgb_dts_solve_noalloc": ([i, i, i, vp, vp, vp, P(FilterParams),
                                     P(OptimizeParams), f, vp, vp], i),
        "dtsgb_soft_create": ([i, P(i), P(i), pvp], i),
        "dtsgb_soft_destroy": ([vp], i),
        "dtsgb_soft_set_stream": ([vp, vp], i),
        "dtsgb_soft_edge_weights": ([vp, i, pvp, P(FilterParams), pvp, pvp], i),
        "dtsgb_soft_solve": ([vp, pvp, pvp, pvp, pvp, P(OptimizeParams), f, pvp], i),
        "dtsgb_soft_backward": ([vp, pvp, pvp, pvp, pvp, pvp], i),
        "dtsgb_dts_init_right_frame": ([vp, f, i, vp], i),
        "dtsgb_dts_init_right_frame_device": ([vp, f, i, vp], i),
        "dtsgb_dts_process_right_frame": ([vp], i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = res


def wait_timeouts() -> int:
    """Thread blocks that gave up waiting for an asynchronous tile copy since
    the library was loaded (dtsgb_wait_timeouts); 0 on a healthy run."""
    n = ctypes.c_ulonglong()
    check(load().dtsgb_wait_timeouts(ctypes.byref(n)))
    return n.value


def check(status: int, allow_warning: bool = False) -> int:
    if status == DTSGB_OK:
        return status
    if allow_warning and status >= 100:
        return status
    msg = load().dtsgb_last_error()
    raise DtsgbError(status, msg.decode() if msg else "")
