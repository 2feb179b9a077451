"""Roofline denominators and counters for the pair kernels.

The pair kernels are a merge, not a contraction: they are bound by the SM
issue rate (FP32 lanes), not by HBM or tensor cores.  The denominator is a
live measurement of FFMA lane-operations per second on the same device
(``sbg_measure_peak``), next to the nominal 152 SMs x 128 lanes x clock.
"""
from __future__ import annotations

import ctypes
import json
import os

from . import _native as nat

_PROFILES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "profiles")


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


def traffic_per_launch(kernel: str, n: int):
    """DRAM bytes (read + write) per launch from the committed ncu summary
    ``profiles/traffic.json``, scaled from the captured case by output pairs
    (the traffic is dominated by the condensed output stream); None if the
    kernel has no capture yet."""
    path = os.path.join(_PROFILES, "traffic.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
    except (OSError, ValueError):
        return None
    e = d.get(kernel)
    if not e:
        return None
    pairs = n * (n - 1) // 2
    return float(e["bytes"]) * pairs / float(e["pairs"])
