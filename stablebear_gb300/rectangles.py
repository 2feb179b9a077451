"""``iterate_rectangles``: the rectangles of one pair of PCFs, as
stablebear/functional/pcf.py:306-374 returns them, computed on the device by
``sbg_iterate_rectangles`` (csrc/rectangles.cu)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as nat
from .pcf import Pcf

_CODES = {np.dtype(np.float32): nat.F32, np.dtype(np.float64): nat.F64,
          np.dtype(np.int32): nat.I32, np.dtype(np.int64): nat.I64}


class Rectangle:
    """An interval [left, right) on which both PCFs are constant, with their
    values there."""

    __slots__ = ("left", "right", "f_value", "g_value")

    def __init__(self, left, right, f_value, g_value):
        self.left = left
        self.right = right
        self.f_value = f_value
        self.g_value = g_value

    def __eq__(self, other):
        if isinstance(other, Rectangle):
            return (self.left == other.left and self.right == other.right
                    and self.f_value == other.f_value and self.g_value == other.g_value)
        if isinstance(other, tuple) and len(other) == 4:
            return (self.left, self.right, self.f_value, self.g_value) == other
        return NotImplemented

    def __repr__(self):
        return (f"Rectangle(left={self.left}, right={self.right}, "
                f"f_value={self.f_value}, g_value={self.g_value})")


def iterate_rectangles(f: Pcf, g: Pcf, a=0.0, b=float("inf")):
    """The rectangles formed by two PCFs on [a, b), in time order (a list of
    Rectangle): starting from each PCF's last breakpoint at or before a, the
    side whose next breakpoint comes first moves on (both on a tie), and the
    last rectangle runs to b.  TypeError for non-PCF arguments or PCFs of
    different types, as in the reference."""
    if not isinstance(f, Pcf) or not isinstance(g, Pcf):
        raise TypeError("Both f and g must be Pcf objects.")
    fp, gp = f._pts, g._pts
    if fp.dtype != gp.dtype:
        raise TypeError("f and g must have the same dtype.")
    code = _CODES.get(fp.dtype)
    if code is None:
        raise TypeError("iterate_rectangles is not supported for this PCF type.")
    fp = np.ascontiguousarray(fp)
    gp = np.ascontiguousarray(gp)
    cap = len(fp) + len(gp)
    out = np.empty((max(cap, 1), 4), dtype=fp.dtype)
    count = ctypes.c_uint64(0)
    nat.check(nat.lib().sbg_iterate_rectangles(code, nat.ptr(fp), len(fp), nat.ptr(gp), len(gp), float(a), float(b),
                                               nat.ptr(out), cap, ctypes.byref(count)))
    n = int(count.value)
    vt = fp.dtype.type
    return [Rectangle(vt(l), vt(r), vt(fv), vt(gv)) for l, r, fv, gv in out[:n]]
