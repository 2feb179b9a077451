"""Process-wide settings (``stablebear/system.py:4-122`` over
``src/python/pymodule.cpp:136-159``).

This library has exactly one execution path, the GPU.  ``force_cpu`` and
``set_cuda_threshold`` are kept so existing code runs unchanged; their values
are stored and reported back but select nothing.
"""
from __future__ import annotations

import ctypes

from . import _native as nat


def force_cpu(on: bool):
    """Accepted for compatibility; computations still run on the GPU."""
    nat.check(nat.lib().sbg_set_force_cpu(1 if on else 0))


def set_block_size(x: int, y: int):
    """Accepted for compatibility (the kernels choose their own launch shape)."""
    nat.check(nat.lib().sbg_set_block_dim(int(x), int(y)))


def limit_cpus(n: int):
    nat.check(nat.lib().sbg_limit_cpus(int(n)))


def limit_gpus(n: int):
    nat.check(nat.lib().sbg_limit_gpus(int(n)))


def set_cuda_threshold(n: int):
    """Accepted for compatibility; there is no CPU path to fall back to."""
    nat.check(nat.lib().sbg_set_cuda_threshold(int(n)))


def get_cuda_threshold() -> int:
    return int(nat.lib().sbg_get_cuda_threshold())


def set_device_verbose(on: bool):
    """When on, each pairwise call prints that it runs on the CUDA device."""
    nat.check(nat.lib().sbg_set_device_verbose(1 if on else 0))


def set_min_block_side(n: int):
    """Accepted for compatibility (work items are sized by the engine)."""
    nat.check(nat.lib().sbg_set_min_block_side(int(n)))


def set_tuning(warps: int = 0, row_chunk: int = 0, variant: int = 0, order: int = 0, band_bytes: int = 0):
    """Engine knobs (0 = automatic): warps per CTA, rows per work item / 32,
    kernel variant (1 shared-memory, 2 global-memory, 3 shared-memory two-load
    walk, 4 hybrid, 5 shared-memory with row times and values apart, 6
    time-windowed shared memory; the float32 measurement variants 7, one
    unified shared-memory load per step from a row replicated 16 times, and
    8, merge path with one pair per warp, which the planner never picks),
    PCF order (1 as given, 2 sorted by breakpoint count), output bytes per
    pipeline band."""
    nat.check(nat.lib().sbg_set_tuning(int(warps), int(row_chunk), int(variant), int(order), int(band_bytes)))


def set_window_cap(cap: int = 0):
    """Time-windowed variant: the most elements of one PCF inside a time
    window (0 = the most that fit in shared memory)."""
    nat.check(nat.lib().sbg_set_window_cap(int(cap)))


def get_window_cap() -> int:
    return int(nat.lib().sbg_get_window_cap())


def build_type() -> str:
    return nat.lib().sbg_build_type().decode()


def get_ngpus() -> int:
    n = ctypes.c_int(0)
    nat.check(nat.lib().sbg_get_ngpus(ctypes.byref(n)))
    return n.value
