"""``lp_norm``: the Lp norm of every PCF of an array, on the GPU.

Same name, arguments, result shape and errors as ``stablebear/norms.py:10-62``;
``Norms_f32_f32`` / ``Norms_f64_f64`` mirror the pybind classes of
``src/python/functional/py_norms.cpp:16-56`` (static ``lpnorm_l1`` /
``lpnorm_lp`` returning ``(task, result)``).  The reference computes norms on
the CPU; here ``sbg_lp_norm_host`` runs one warp per PCF on the device.
"""
from __future__ import annotations

import numpy as np

from . import _native as nat
from .pcf import PcfArray, _resolve_pcf_inputs, pcf32, pcf64
from .task import EmptyTask, _run_task


class _NormsBackend:
    _np = np.float32
    _code = nat.F32

    @classmethod
    def _norm(cls, X: PcfArray, p: float):
        pts, off = X.csr()
        n = len(off) - 1
        out = np.zeros(tuple(X.shape), dtype=cls._np)
        if n:
            nat.check(nat.lib().sbg_lp_norm_host(cls._code, float(p), nat.ptr(pts), nat.ptr(off), n,
                                                 nat.ptr(out)))
        return EmptyTask(), out

    @classmethod
    def lpnorm_l1(cls, X: PcfArray):
        return cls._norm(X, 1.0)

    @classmethod
    def lpnorm_lp(cls, X: PcfArray, p: float):
        return cls._norm(X, p)


class Norms_f32_f32(_NormsBackend):
    _np = np.float32
    _code = nat.F32


class Norms_f64_f64(_NormsBackend):
    _np = np.float64
    _code = nat.F64


_NORMS_BACKEND_MAP = {pcf32: Norms_f32_f32, pcf64: Norms_f64_f64}


def lp_norm(fs, p=1, verbose=False) -> np.ndarray:
    r"""The :math:`L_p` norm :math:`(\int_0^\infty |f(t)|^p dt)^{1/p}` of each
    PCF in ``fs``; an array of the same shape as ``fs``."""
    if p < 1:
        raise ValueError("p must be >= 1.")
    (X,) = _resolve_pcf_inputs(fs)
    backend = _NORMS_BACKEND_MAP.get(X.dtype)
    if backend is None:
        raise TypeError(f"lp_norm is not supported for PCF type {X.dtype}")
    if p == 1:
        task, out = backend.lpnorm_l1(X)
    else:
        task, out = backend.lpnorm_lp(X, float(p))
    _run_task(lambda: task, verbose=verbose)
    return out
