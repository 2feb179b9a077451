"""ctypes binding of the native library (``include/sbgpu.h``).

The library is built in-tree by ``stablebear_gb300.build`` into
``stablebear_gb300/_lib/libsbgpu.so``.  There is no CPU fallback: if the
library is missing, every compute entry raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libsbgpu.so")

SBG_OK = 0
SBG_ERR_OUT_OF_MEMORY = -4
SBG_ERR_CANCELLED = -5
ALLOC_UNLIMITED = (1 << 64) - 1  # SBG_ALLOC_UNLIMITED: no limit on the library's device allocations
STATUS_NAMES = {
    -1: "SBG_ERR_INVALID_ARGUMENT",
    -2: "SBG_ERR_INVALID_INPUT",
    -3: "SBG_ERR_CUDA",
    -4: "SBG_ERR_OUT_OF_MEMORY",
    -5: "SBG_ERR_CANCELLED",
    -6: "SBG_ERR_NO_DEVICE",
    -7: "SBG_ERR_TIMEOUT",
    -8: "SBG_ERR_INTERNAL",
    -9: "SBG_ERR_LOGIC",
}

F32, F64 = 0, 1
I32, I64 = 2, 3  # integer PCFs (sbg_iterate_rectangles)
OP_L1, OP_LP, OP_L2_INNER = 0, 1, 2
SKIP_NONE, SKIP_LOWER_NODIAG, SKIP_LOWER = 0, 1, 2
FLAG_ASYMMETRIC, FLAG_DIAGONAL, FLAG_NEGATIVE = 1, 2, 4  # sbg_dense_to_condensed_device
BATCH_GRAPH, BATCH_CALLER_ORDER, BATCH_TUNE_WINDOW = 1, 2, 4  # sbg_batch_create flags

# Every symbol include/sbgpu.h declares, with (restype, argtypes).
_P = ctypes.c_void_p
_U64 = ctypes.c_uint64
_I = ctypes.c_int
_D = ctypes.c_double
SIGNATURES = {
    "sbg_api_version": (_I, []),
    "sbg_last_error": (ctypes.c_char_p, []),
    "sbg_build_type": (ctypes.c_char_p, []),
    "sbg_get_ngpus": (_I, [ctypes.POINTER(_I)]),
    "sbg_set_force_cpu": (_I, [_I]),
    "sbg_get_force_cpu": (_I, []),
    "sbg_set_cuda_threshold": (_I, [_U64]),
    "sbg_get_cuda_threshold": (_U64, []),
    "sbg_set_block_dim": (_I, [ctypes.c_uint, ctypes.c_uint]),
    "sbg_set_min_block_side": (_I, [_U64]),
    "sbg_limit_gpus": (_I, [_I]),
    "sbg_limit_cpus": (_I, [_I]),
    "sbg_set_device_verbose": (_I, [_I]),
    "sbg_get_device_verbose": (_I, []),
    "sbg_set_tuning": (_I, [_I, _I, _I, _I, _U64]),
    "sbg_set_output_mode": (_I, [_I]),
    "sbg_set_window_cap": (_I, [_I]),
    "sbg_get_window_cap": (_I, []),
    "sbg_host_memory_access": (_I, [ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "sbg_create_integrate_task": (_I, [_I, _I, _D, _I, _P, _P, _U64, _P, ctypes.POINTER(_P)]),
    "sbg_create_cdist_task": (_I, [_I, _I, _D, _P, _P, _U64, _P, _P, _U64, _P, ctypes.POINTER(_P)]),
    "sbg_task_start": (_I, [_P]),
    "sbg_task_wait_for": (_I, [_P, ctypes.c_int64, ctypes.POINTER(_I)]),
    "sbg_task_wait": (_I, [_P]),
    "sbg_task_request_stop": (_I, [_P]),
    "sbg_task_stop_requested": (_I, [_P]),
    "sbg_task_progress": (_I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "sbg_task_step_text": (_I, [_P, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]),
    "sbg_task_destroy": (None, [_P]),
    "sbg_pairwise_host": (_I, [_I, _I, _D, _I, _P, _P, _U64, _P, _P, _U64, _P, _I]),
    "sbg_pairwise_device": (_I, [_I, _I, _D, _I, _P, _P, _U64, _P, _P, _U64, _P, _P, ctypes.c_uint32, _P, _U64,
                                 _U64, _U64, _P]),
    "sbg_pairwise_device_noalloc": (_I, [_I, _I, _D, _I, _P, _P, _U64, _U64, _P, _P, _U64, _U64, _P, _P,
                                         ctypes.c_uint32, _P, _U64, _U64, _U64, _P]),
    "sbg_pairwise_backward_device": (_I, [_I, _I, _D, _I, _P, _P, _U64, _U64, ctypes.c_uint32, _P, _P, _P, _P]),
    "sbg_batch_create": (_I, [_I, _I, _D, _I, _P, _U64, _I, ctypes.POINTER(_P)]),
    "sbg_batch_launch": (_I, [_P, _P]),
    "sbg_batch_autotune": (_I, [_P, _P, ctypes.POINTER(_D)]),
    "sbg_batch_info": (_I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "sbg_batch_shared_split": (_I, [_P, ctypes.POINTER(ctypes.c_uint32)]),
    "sbg_batch_destroy": (None, [_P]),
    "sbg_output_count": (_U64, [_I, _U64, _U64]),
    "sbg_kernel_launches": (_U64, []),
    "sbg_autotune_device": (_I, [_I, _I, _D, _I, _P, _P, _U64, _P, _P, _U64, ctypes.c_uint32, _P, _P,
                                 ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_D)]),
    "sbg_tuning_cache_lookup": (_I, [_I, _I, _D, _I, _U64, ctypes.c_uint32, ctypes.POINTER(_I), ctypes.POINTER(_I),
                                     ctypes.POINTER(_I)]),
    "sbg_tuning_cache_store": (_I, [_I, _I, _D, _I, _U64, ctypes.c_uint32, _I, _I]),
    "sbg_tuning_cache_clear": (_I, []),
    "sbg_set_alloc_limit": (_I, [_U64]),
    "sbg_device_allocations": (_U64, []),
    "sbg_device_bytes_held": (_U64, []),
    "sbg_block_device": (_I, [_I, _I, _D, _I, _P, _P, _P, _P, _U64, _U64, _U64, _U64, ctypes.c_uint32, _P, _P]),
    "sbg_length_order_device": (_I, [_P, _U64, _P, _P]),
    "sbg_measure_peak": (_I, [_I, ctypes.POINTER(_D)]),
    "sbg_enumerate_items": (_U64, [_I, _U64, _U64, _U64, _U64, ctypes.c_uint32, _P, _U64]),
    "sbg_condensed_to_dense_device": (_I, [_I, _I, _U64, _P, _P, _U64, _U64, _U64, _P]),
    "sbg_dense_to_condensed_device": (_I, [_I, _I, _U64, _P, _U64, _P, _P, _P]),
    "sbg_dense_fold_to_condensed_device": (_I, [_I, _I, _U64, _P, _U64, _P, _P]),
    "sbg_lp_norm_device": (_I, [_I, _D, _P, _P, _U64, _P, _P]),
    "sbg_lp_norm_host": (_I, [_I, _D, _P, _P, _U64, _P]),
    "sbg_iterate_rectangles": (_I, [_I, _P, _U64, _P, _U64, _D, _D, _P, _U64, _P]),
    "sbg_barcode_pcf_capacity": (_U64, [_I, _U64, _U64]),
    "sbg_barcodes_to_pcfs_device": (_I, [_I, _I, _P, _P, _U64, _U64, _P, _U64, _P, _P]),
    "sbg_barcodes_to_pcfs_host": (_I, [_I, _I, _P, _P, _U64, _P, _U64, _P]),
}

_lib = None
_lock = threading.Lock()


class NativeError(RuntimeError):
    """A failing C-ABI call: ``status`` is the sbg_status code."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def lib():
    """Load (once) and return the native library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"stablebear_gb300 native library not found at {LIB_PATH}; build it with "
                "`python -m stablebear_gb300.build` (needs nvcc).  There is no CPU fallback.")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def last_error() -> str:
    msg = lib().sbg_last_error()
    return msg.decode("utf-8", "replace") if msg else ""


def check(status: int) -> None:
    """Raise the Python exception matching a C-ABI status.

    Mirrors how the reference's pybind layer surfaces C++ exceptions:
    invalid_argument -> ValueError, logic_error -> RuntimeError, CUDA errors
    (runtime_error from CHK_CUDA) -> RuntimeError, allocation -> MemoryError.
    """
    if status == SBG_OK:
        return
    msg = last_error() or STATUS_NAMES.get(status, str(status))
    if status in (-1, -2):
        raise ValueError(msg)
    if status == -4:
        raise MemoryError(msg)
    if status == -5:
        raise InterruptedError(msg)
    raise NativeError(status, msg)


def ptr(a) -> ctypes.c_void_p:
    """Address of a numpy array's data (None for empty arrays)."""
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data) if a.size else ctypes.c_void_p(a.ctypes.data or 0)
