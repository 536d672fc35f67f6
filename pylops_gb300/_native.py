"""ctypes binding of ``libpylops_gb300.so`` (C ABI in ``include/kirchhoff_gb300.h``).

The library is the only compute path of this package: if it is missing or
fails to load, importing an operator raises instead of falling back to any
host implementation.
"""

import ctypes
import os
import threading

import numpy as np

from . import _build

KGB_OK = 0
KGB_ERR_VALUE = 1
KGB_ERR_NOT_IMPLEMENTED = 2
KGB_ERR_CUDA = 3
KGB_ERR_MEMORY = 4
KGB_ERR_STATE = 5

_EXC = {
    KGB_ERR_VALUE: ValueError,
    KGB_ERR_NOT_IMPLEMENTED: NotImplementedError,
    KGB_ERR_CUDA: RuntimeError,
    KGB_ERR_MEMORY: MemoryError,
    KGB_ERR_STATE: RuntimeError,
}

_lib = None
_lock = threading.Lock()

c_int = ctypes.c_int
c_i64 = ctypes.c_int64
c_float = ctypes.c_float
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p
c_dp = ctypes.POINTER(ctypes.c_double)
c_ip = ctypes.POINTER(ctypes.c_int)
c_i64p = ctypes.POINTER(ctypes.c_int64)

_SIGNATURES = {
    "kgb_version": ([], c_int),
    "kgb_last_error": ([], ctypes.c_char_p),
    "kgb_kirchhoff_create": ([ctypes.POINTER(c_vp), c_int, c_int, c_int, c_i64, c_int, c_dbl, c_int, c_dp, c_int, c_int], c_int),
    "kgb_kirchhoff_destroy": ([c_vp], c_int),
    "kgb_kirchhoff_set_traveltimes": ([c_vp, c_dp, c_dp], c_int),
    "kgb_kirchhoff_set_traveltime_table": ([c_vp, c_dp], c_int),
    "kgb_kirchhoff_set_weight_precision": ([c_vp, c_int], c_int),
    "kgb_kirchhoff_set_dynamic": ([c_vp, c_dp, c_dp, c_dp, c_dp, c_dp, c_dp, c_dp, c_dp, c_i64p, c_i64p], c_int),
    "kgb_kirchhoff_build_tables": ([c_vp, c_int, c_int, c_dp, c_int, c_dp, c_int, c_dp, c_int, c_dp, c_dp, c_dp,
                                    ctypes.c_int64, c_dp, c_dp, c_dp, c_i64p, c_i64p, c_dp], c_int),
    "kgb_kirchhoff_get_table": ([c_vp, c_int, c_dp], c_int),
    "kgb_kirchhoff_forward": ([c_vp, c_vp, c_vp, c_vp], c_int),
    "kgb_kirchhoff_adjoint": ([c_vp, c_vp, c_vp, c_vp], c_int),
    "kgb_kirchhoff_forward_static": ([c_vp, c_vp, c_vp, c_vp], c_int),
    "kgb_kirchhoff_forward_host": ([c_vp, c_vp, c_vp], c_int),
    "kgb_kirchhoff_adjoint_host": ([c_vp, c_vp, c_vp], c_int),
    "kgb_kirchhoff_spread": ([c_vp, c_vp, c_vp, c_vp], c_int),
    "kgb_kirchhoff_gather": ([c_vp, c_vp, c_vp, c_vp], c_int),
    "kgb_kirchhoff_wavelet": ([c_vp, c_vp, c_vp, c_int, c_vp], c_int),
    "kgb_kirchhoff_info": ([c_vp, c_i64p], c_int),
    "kgb_kirchhoff_set_variant": ([c_vp, c_int], c_int),
    "kgb_kirchhoff_set_adjoint_variant": ([c_vp, c_int], c_int),
    "kgb_dot_f64": ([c_vp, c_vp, c_i64, c_vp, c_vp], c_int),
    "kgb_solver_create": ([ctypes.POINTER(c_vp), c_vp, c_int], c_int),
    "kgb_solver_destroy": ([c_vp], c_int),
    "kgb_nsconv2d_apply": ([c_vp, c_vp, c_vp] + [c_int] * 6 + [c_dbl] * 4 + [c_int, c_vp], c_int),
    "kgb_lincomb_f32": ([c_vp, c_vp, c_dbl, c_vp, c_vp, c_int, c_i64, c_vp], c_int),
    "kgb_solver_set_diagonal": ([c_vp, c_vp], c_int),
    "kgb_solver_setup": ([c_vp, c_vp, c_vp, c_dp, c_int, c_vp], c_int),
    "kgb_solver_run": ([c_vp, c_int, c_int, c_vp], c_int),
    "kgb_solver_result": ([c_vp, c_vp, c_dp, c_dp, c_int, c_vp], c_int),
    "kgb_batch_create": ([ctypes.POINTER(c_vp), ctypes.POINTER(c_vp), c_int], c_int),
    "kgb_batch_destroy": ([c_vp], c_int),
    "kgb_batch_sizes": ([c_vp, c_i64p], c_int),
    "kgb_batch_set_tile": ([c_vp, c_int], c_int),
    "kgb_batch_set_gather": ([c_vp, c_int, c_int], c_int),
    "kgb_batch_forward": ([c_vp, c_vp, c_vp, c_vp], c_int),
    "kgb_batch_adjoint": ([c_vp, c_vp, c_vp, c_vp], c_int),
    "kgb_batch_cgls": ([c_vp, c_vp, c_vp, c_int, c_dbl, c_dbl, c_int, c_dp, c_ip, c_dp, c_vp], c_int),
    "kgb_gemm_bf16_tn": ([c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int, c_int, c_int, c_vp, c_int, c_vp, c_vp], c_int),
    "kgb_gemm_bf16_tn_splitk": ([c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_vp, c_i64,
                                 c_vp, c_vp], c_int),
    "kgb_conv3x3_bf16": ([c_vp, c_vp, c_vp] + [c_int] * 6 + [c_vp, c_int, c_vp, c_vp], c_int),
    "kgb_conv3x3_wgrad_bf16": ([c_vp, c_vp, c_vp] + [c_int] * 6 + [c_vp, c_i64, c_vp, c_vp], c_int),
    "kgb_conv3x3_s2_dgrad_bf16": ([c_vp, c_vp, c_vp] + [c_int] * 5 + [c_vp, c_vp], c_int),
    "kgb_unet_unfold": ([c_vp, c_vp] + [c_int] * 10 + [c_vp], c_int),
    "kgb_unet_unfold_t": ([c_vp, c_vp] + [c_int] * 6 + [c_vp], c_int),
    "kgb_unet_transpose": ([c_vp, c_vp, c_i64, c_int, c_i64, c_i64, c_int, c_vp], c_int),
    "kgb_unet_weights": ([c_vp, c_vp, c_vp] + [c_int] * 5 + [c_vp], c_int),
    "kgb_unet_weights_implicit": ([c_vp, c_vp, c_vp, c_int, c_int, c_int, c_vp], c_int),
    "kgb_unet_relu_grad": ([c_vp, c_vp, c_vp, c_i64, c_int, c_vp], c_int),
    "kgb_unet_rowsum": ([c_vp, c_vp, c_int, c_i64, c_vp, c_vp], c_int),
    "kgb_unet_upsample": ([c_vp, c_vp] + [c_int] * 7 + [c_vp], c_int),
    "kgb_unet_channels": ([c_vp, c_vp, c_i64, c_int, c_int, c_int, c_int, c_int, c_vp], c_int),
    "kgb_unet_to_bf16": ([c_vp, c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    "kgb_unet_image_rms": ([c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    "kgb_unet_row_transpose": ([c_vp, c_vp] + [c_int] * 5 + [c_vp], c_int),
    "kgb_unet_colsum": ([c_vp, c_vp, c_vp, c_i64, c_int, c_vp, c_vp], c_int),
    "kgb_unet_head_forward": ([c_vp, c_vp, c_vp, c_vp, c_i64, c_int, c_vp], c_int),
    "kgb_unet_head_dx": ([c_vp, c_vp, c_vp, c_i64, c_int, c_vp], c_int),
    "kgb_unet_conv3x3_c1": ([c_vp, c_vp, c_vp, c_vp] + [c_int] * 6 + [c_vp], c_int),
    "kgb_unet_conv3x3_c1_wgrad": ([c_vp, c_vp, c_vp] + [c_int] * 5 + [c_vp, c_vp], c_int),
    "kgb_unet_mse": ([c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp], c_int),
    "kgb_unet_adam": ([c_vp, c_vp, c_vp, c_vp, c_i64, c_float, c_float, c_float, c_float, c_int, c_vp], c_int),
    "kgb_eikonal_tables": ([c_int, c_ip, c_dp, c_dp, c_int, c_ip, c_dp, c_dp, c_int, c_int], c_int),
}


def exported_symbols():
    """Names of every C entry point the binding declares."""
    return sorted(_SIGNATURES)


def lib(build_if_missing: bool = True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if build_if_missing and (not os.path.exists(path) or _build._stale()):
            _build.build()
        if not os.path.exists(path):
            raise ImportError(
                f"pylops_gb300 CUDA library not found at {path}; build it with "
                "`python -c 'import pylops_gb300._build as b; b.build()'`"
            )
        L = ctypes.CDLL(path)
        for name, (args, res) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(rc: int):
    if rc != KGB_OK:
        msg = lib().kgb_last_error().decode(errors="replace")
        raise _EXC.get(rc, RuntimeError)(msg)


def dptr(a: np.ndarray):
    """float64 host pointer of a C-contiguous array."""
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(c_dp)


def i64ptr(a: np.ndarray):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(c_i64p)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(c_ip)


def vptr(a) -> int:
    """Raw address of a numpy array or a torch tensor."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()
