"""Roofline denominators for the pair kernels.

The pair kernels are a merge, not a contraction: neither HBM nor tensor
cores bound them.  The FP32 (and FP64) denominators are live measurements of
FMA lane-operations per second on the same device (``sbg_measure_peak``),
next to the nominal 152 SMs x 128 lanes x clock.
"""
from __future__ import annotations

import ctypes

from . import _native as nat


def fp32_peak(device: int = 0) -> dict:
    v = ctypes.c_double(0.0)
    nat.check(nat.lib().sbg_measure_peak(0, ctypes.byref(v)))
    return {"value": v.value / 1e12, "unit": "T lane-op/s",
            "source": "measured: FFMA loop kernel (8 independent chains/thread), same device, same run"}


def fp64_peak(device: int = 0) -> dict:
    v = ctypes.c_double(0.0)
    nat.check(nat.lib().sbg_measure_peak(1, ctypes.byref(v)))
    return {"value": v.value / 1e12, "unit": "T lane-op/s",
            "source": "measured: DFMA loop kernel (8 independent chains/thread), same device, same run"}
