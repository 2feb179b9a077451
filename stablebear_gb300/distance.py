"""The pairwise API: ``pdist``, ``cdist``, ``l2_kernel``, ``lp_distance``.

Same names, arguments, return types and errors as ``stablebear/distance.py``
and ``stablebear/inner_product.py``; the per-dtype backend classes
``Distance_f32_f32`` / ``Distance_f64_f64`` / ``InnerProduct_f32_f32`` /
``InnerProduct_f64_f64`` mirror the pybind classes of
``src/python/functional/py_distance.cpp:225-250`` and
``py_inner_product.cpp:71-90``: static methods returning ``(task, result)``.
Those classes are the compiled pybind11 module ``_sb_gb300`` where it was
built (``_binding.py``), else the ctypes classes below, over the same C ABI.

Every computation runs on the GPU through the native library; there is no
CPU path (``force_cpu`` is accepted and ignored, see ``system.py``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _binding
from . import _native as nat
from .matrices import DistanceMatrix, SymmetricMatrix
from .pcf import Pcf, PcfArray, _has_matching_types, _resolve_pcf_inputs, pcf32, pcf64
from .task import EmptyTask, StoppableTask, _run_task


def _device_verbose(msg: str):
    if nat.lib().sbg_get_device_verbose():
        print(msg)


def _create_integrate(dtype_code, op, p, skip, pts, off, n, out):
    h = ctypes.c_void_p()
    nat.check(nat.lib().sbg_create_integrate_task(dtype_code, op, float(p), skip, nat.ptr(pts), nat.ptr(off), n,
                                                  nat.ptr(out), ctypes.byref(h)))
    return StoppableTask(h, keepalive=(out,)).start()


def _create_cdist(dtype_code, op, p, xp, xo, nx, yp, yo, ny, out):
    h = ctypes.c_void_p()
    nat.check(nat.lib().sbg_create_cdist_task(dtype_code, op, float(p), nat.ptr(xp), nat.ptr(xo), nx, nat.ptr(yp),
                                              nat.ptr(yo), ny, nat.ptr(out), ctypes.byref(h)))
    return StoppableTask(h, keepalive=(out,)).start()


class _DistanceBackend:
    _np = np.float32
    _code = nat.F32

    @classmethod
    def _pdist(cls, X: PcfArray, op, p):
        pts, off = X.csr()
        n = len(off) - 1
        dm = DistanceMatrix(n, dtype=cls._np)
        if n < 2:
            return EmptyTask(), dm
        _device_verbose("Integral computation on CUDA device(s)")
        task = _create_integrate(cls._code, op, p, nat.SKIP_LOWER_NODIAG, pts, off, n, dm.data)
        return task, dm

    @classmethod
    def pdist_l1(cls, X: PcfArray):
        return cls._pdist(X, nat.OP_L1, 1.0)

    @classmethod
    def pdist_lp(cls, X: PcfArray, p: float):
        return cls._pdist(X, nat.OP_LP, p)

    @classmethod
    def _cdist(cls, X: PcfArray, Y: PcfArray, op, p):
        xp, xo = X.csr()
        yp, yo = Y.csr()
        nx, ny = len(xo) - 1, len(yo) - 1
        out = np.zeros(tuple(X.shape) + tuple(Y.shape), dtype=cls._np)
        if nx == 0 or ny == 0:
            return EmptyTask(), out
        _device_verbose("Cross-distance computation on CUDA device(s)")
        task = _create_cdist(cls._code, op, p, xp, xo, nx, yp, yo, ny, out)
        return task, out

    @classmethod
    def cdist_l1(cls, X, Y):
        return cls._cdist(X, Y, nat.OP_L1, 1.0)

    @classmethod
    def cdist_lp(cls, X, Y, p: float):
        return cls._cdist(X, Y, nat.OP_LP, p)

    @classmethod
    def _pair(cls, f: Pcf, g: Pcf, op, p):
        out = np.zeros(1, dtype=cls._np)
        fo = np.array([0, f.size], dtype=np.uint64)
        go = np.array([0, g.size], dtype=np.uint64)
        fp = np.ascontiguousarray(f._pts, dtype=cls._np)
        gp = np.ascontiguousarray(g._pts, dtype=cls._np)
        nat.check(nat.lib().sbg_pairwise_host(cls._code, op, float(p), nat.SKIP_NONE, nat.ptr(fp), nat.ptr(fo), 1,
                                              nat.ptr(gp), nat.ptr(go), 1, nat.ptr(out), 1))
        return out[0]

    @classmethod
    def lp_distance_l1(cls, f: Pcf, g: Pcf):
        return cls._pair(f, g, nat.OP_L1, 1.0)

    @classmethod
    def lp_distance_lp(cls, f: Pcf, g: Pcf, p: float):
        return cls._pair(f, g, nat.OP_LP, p)


class Distance_f32_f32(_DistanceBackend):
    _np = np.float32
    _code = nat.F32


class Distance_f64_f64(_DistanceBackend):
    _np = np.float64
    _code = nat.F64


class _InnerProductBackend:
    _np = np.float32
    _code = nat.F32

    @classmethod
    def l2(cls, X: PcfArray):
        pts, off = X.csr()
        n = len(off) - 1
        sm = SymmetricMatrix(n, dtype=cls._np)
        if n == 0:
            return EmptyTask(), sm
        _device_verbose("Kernel computation on CUDA device(s)")
        task = _create_integrate(cls._code, nat.OP_L2_INNER, 1.0, nat.SKIP_LOWER, pts, off, n, sm.data)
        return task, sm


class InnerProduct_f32_f32(_InnerProductBackend):
    _np = np.float32
    _code = nat.F32


class InnerProduct_f64_f64(_InnerProductBackend):
    _np = np.float64
    _code = nat.F64


# The same four classes over ctypes (defined above) and, where it was built,
# compiled over pybind11 (_sb_gb300): the public names are the compiled ones
# when present, the ctypes ones otherwise.
CTYPES_BACKENDS = {"Distance_f32_f32": Distance_f32_f32, "Distance_f64_f64": Distance_f64_f64,
                   "InnerProduct_f32_f32": InnerProduct_f32_f32, "InnerProduct_f64_f64": InnerProduct_f64_f64}
_compiled = _binding.compiled()
if _compiled is not None:
    Distance_f32_f32 = _compiled.Distance_f32_f32
    Distance_f64_f64 = _compiled.Distance_f64_f64
    InnerProduct_f32_f32 = _compiled.InnerProduct_f32_f32
    InnerProduct_f64_f64 = _compiled.InnerProduct_f64_f64

_DISTANCE_BACKEND_MAP = {pcf32: Distance_f32_f32, pcf64: Distance_f64_f64}
_INNER_PRODUCT_BACKEND_MAP = {pcf32: InnerProduct_f32_f32, pcf64: InnerProduct_f64_f64}
_VTYPE_TO_DISTANCE_BACKEND = {np.float32: Distance_f32_f32, np.float64: Distance_f64_f64}


def _backend(mapping, X: PcfArray):
    b = mapping.get(X.dtype)
    if b is None:
        raise TypeError(f"this operation is not supported for PCF type {X.dtype}")
    return b


def lp_distance(f: Pcf, g: Pcf, p=1) -> float:
    r"""The :math:`L_p` distance :math:`(\int_0^\infty |f - g|^p dt)^{1/p}`
    between two PCFs (``stablebear/distance.py:17-64``)."""
    if p < 1:
        raise ValueError("p must be >= 1.")
    if not isinstance(f, Pcf) or not isinstance(g, Pcf):
        raise TypeError("Both f and g must be Pcf objects.")
    if not _has_matching_types(f, g):
        raise TypeError("f and g must have the same dtype.")
    backend = _VTYPE_TO_DISTANCE_BACKEND.get(f.vtype)
    if backend is None:
        raise TypeError(f"lp_distance is not supported for this PCF type (vtype={f.vtype}).")
    if p == 1:
        return float(backend.lp_distance_l1(f, g))
    return float(backend.lp_distance_lp(f, g, float(p)))


def pdist(fs, p=1, verbose=False) -> DistanceMatrix:
    r"""Pairwise :math:`L_p` distance matrix of a 1-D array of PCFs
    (``stablebear/distance.py:67-111``)."""
    if p < 1:
        raise ValueError("p must be >= 1.")
    (X,) = _resolve_pcf_inputs(fs)
    if len(X.shape) != 1:
        raise ValueError("1d tensor expected.")
    backend = _backend(_DISTANCE_BACKEND_MAP, X)
    if p == 1:
        task, dm = backend.pdist_l1(X)
    else:
        task, dm = backend.pdist_lp(X, float(p))
    _run_task(lambda: task, verbose=verbose)
    return dm


def cdist(X, Y, p=1, verbose=False) -> np.ndarray:
    r"""Pairwise :math:`L_p` distances between two arrays of PCFs; result of
    shape ``(*X.shape, *Y.shape)`` (``stablebear/distance.py:114-154``)."""
    if p < 1:
        raise ValueError("p must be >= 1.")
    Xt, Yt = _resolve_pcf_inputs(X, Y)
    backend = _backend(_DISTANCE_BACKEND_MAP, Xt)
    if p == 1:
        task, out = backend.cdist_l1(Xt, Yt)
    else:
        task, out = backend.cdist_lp(Xt, Yt, float(p))
    _run_task(lambda: task, verbose=verbose)
    return out


def l2_kernel(fs, verbose=False) -> SymmetricMatrix:
    r"""Pairwise :math:`L_2` kernel (Gram) matrix of a 1-D array of PCFs
    (``stablebear/inner_product.py:13-50``)."""
    (X,) = _resolve_pcf_inputs(fs)
    if len(X.shape) != 1:
        raise ValueError("1d tensor expected.")
    backend = _backend(_INNER_PRODUCT_BACKEND_MAP, X)
    task, sm = backend.l2(X)
    _run_task(lambda: task, verbose=verbose)
    return sm
