"""PCF values and arrays of PCFs — the input side of the pairwise path.

``Pcf`` follows ``stablebear/functional/pcf.py`` and its validation in
``src/python/pypcf_support.hpp:35-92``: an ``(n, 2)`` array of ``(t, v)``
breakpoints in non-decreasing time order starting at ``t = 0``.  The function
takes value ``v_k`` on ``[t_k, t_{k+1})`` and ``v_{n-1}`` from ``t_{n-1}`` on.

``PcfArray`` is the 1-D (or N-D) container the pairwise functions take.  It
stores the PCFs as the reference's flattened CSR (``points`` ``(M, 2)`` plus
``offsets`` ``(N + 1)``, ``include/sbear/cuda/offset_data_manager.hpp:42-68``),
which is also the layout the native library consumes, so a large array goes to
the GPU without per-PCF copies.  The reference's general N-d tensor algebra is
not part of this package.
"""
from __future__ import annotations

from typing import Iterable, Sequence

import numpy as np


class _PcfDtype:
    def __init__(self, name, np_dtype):
        self.__name__ = name
        self.name = name
        self.np_dtype = np.dtype(np_dtype)

    def __repr__(self):
        return self.name


pcf32 = _PcfDtype("pcf32", np.float32)
pcf64 = _PcfDtype("pcf64", np.float64)
pcf32i = _PcfDtype("pcf32i", np.int32)
pcf64i = _PcfDtype("pcf64i", np.int64)
float32 = np.float32
float64 = np.float64

_BY_NP = {np.dtype(np.float32): pcf32, np.dtype(np.float64): pcf64,
          np.dtype(np.int32): pcf32i, np.dtype(np.int64): pcf64i}


def _as_pcf_dtype(dtype):
    if dtype is None:
        return None
    if isinstance(dtype, _PcfDtype):
        return dtype
    try:
        return _BY_NP[np.dtype(dtype)]
    except (TypeError, KeyError):
        raise TypeError(f"unsupported PCF dtype {dtype!r}") from None


def _validate_points(pts: np.ndarray) -> None:
    """Checks of src/python/pypcf_support.hpp:52-89."""
    if pts.ndim != 2 or pts.shape[1] != 2:
        raise RuntimeError(f"Input array should be Nx2 (supplied shape is {pts.shape}).")
    if pts.shape[0] == 0:
        raise ValueError("A PCF needs at least one breakpoint.")
    t = pts[:, 0]
    if np.issubdtype(pts.dtype, np.floating) and not np.all(np.isfinite(t)):
        raise ValueError("Breakpoint times must be finite.")
    if np.any(t[1:] < t[:-1]):
        raise ValueError("Breakpoints must be given in non-decreasing time order.")
    if t[0] != 0:
        raise ValueError(f"The first breakpoint must have time t=0 (got t={float(t[0])}).")


class Pcf:
    """A piecewise constant function given by its ``(t, v)`` breakpoints."""

    __slots__ = ("_pts",)

    def __init__(self, data=None, dtype=None):
        dt = _as_pcf_dtype(dtype)
        if data is None:
            arr = np.zeros((1, 2), dtype=dt.np_dtype if dt else np.float32)
        elif isinstance(data, Pcf):
            arr = data._pts.astype(dt.np_dtype if dt else data._pts.dtype, copy=True)
        else:
            arr = np.array(data)
            if dt is not None:
                arr = arr.astype(dt.np_dtype)
            elif arr.dtype not in _BY_NP:
                arr = arr.astype(np.float64 if np.issubdtype(arr.dtype, np.floating) or arr.dtype == object
                                 else np.int64)
            arr = np.ascontiguousarray(arr)
        _validate_points(arr)
        self._pts = arr

    @classmethod
    def _trusted(cls, pts: np.ndarray) -> "Pcf":
        obj = cls.__new__(cls)
        obj._pts = pts
        return obj

    @property
    def dtype(self):
        return _BY_NP[self._pts.dtype]

    @property
    def vtype(self):
        return self._pts.dtype.type

    @property
    def size(self) -> int:
        return int(self._pts.shape[0])

    def to_numpy(self) -> np.ndarray:
        return self._pts.copy()

    def __array__(self, dtype=None, copy=None):
        return self._pts.astype(dtype) if dtype is not None else self._pts.copy()

    def astype(self, dtype) -> "Pcf":
        return Pcf(self._pts, dtype=dtype)

    def __call__(self, t):
        """Evaluate at times ``t`` (value of the last breakpoint <= t)."""
        t = np.asarray(t)
        idx = np.searchsorted(self._pts[:, 0], t, side="right") - 1
        idx = np.clip(idx, 0, None)
        return self._pts[idx, 1]

    def __len__(self):
        return self.size

    def __eq__(self, other):
        return isinstance(other, Pcf) and self._pts.dtype == other._pts.dtype and np.array_equal(self._pts, other._pts)

    def __repr__(self):
        body = ", ".join(f"f({t}) = {v}" for t, v in self._pts[:8])
        more = ", ..." if self.size > 8 else ""
        return f"Pcf<{self.dtype}>({body}{more})"


def _has_matching_types(f: Pcf, g: Pcf) -> bool:
    return f._pts.dtype == g._pts.dtype


class PcfArray:
    """An array (any shape) of PCFs of one dtype, stored as a flat CSR."""

    def __init__(self, pcfs: Iterable[Pcf] | None = None, dtype=None, shape=None):
        dt = _as_pcf_dtype(dtype)
        items = list(pcfs) if pcfs is not None else []
        for f in items:
            if not isinstance(f, Pcf):
                raise TypeError(f"PcfArray elements must be Pcf objects, got {type(f).__name__}")
        if dt is None:
            dt = items[0].dtype if items else pcf32
        for f in items:
            if f.dtype is not dt and f._pts.dtype != dt.np_dtype:
                raise TypeError("all PCFs must have the same dtype")
        lens = np.fromiter((f.size for f in items), dtype=np.uint64, count=len(items))
        offsets = np.zeros(len(items) + 1, dtype=np.uint64)
        np.cumsum(lens, out=offsets[1:])
        pts = (np.concatenate([f._pts for f in items]).astype(dt.np_dtype, copy=False)
               if items else np.zeros((0, 2), dtype=dt.np_dtype))
        self._init_csr(pts, offsets, dt, tuple(shape) if shape is not None else (len(items),))

    def _init_csr(self, pts, offsets, dt, shape, index=None):
        self._pts = pts
        self._off = offsets
        self._dtype = dt
        n = len(offsets) - 1
        if index is None:
            if int(np.prod(shape, dtype=np.int64)) != n:
                raise ValueError(f"shape {shape} does not match {n} PCFs")
            index = np.arange(n, dtype=np.int64).reshape(shape)
        self._index = index
        self._edits = {}

    @classmethod
    def from_csr(cls, points, offsets, shape=None, validate=True) -> "PcfArray":
        """Wrap an ``(M, 2)`` points array and ``N + 1`` offsets (no copy when
        already contiguous float32/float64 / uint64)."""
        pts = np.ascontiguousarray(points)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        if pts.ndim != 2 or pts.shape[1] != 2:
            raise ValueError("points must be an (M, 2) array")
        if len(off) == 0 or off[0] != 0 or int(off[-1]) != pts.shape[0] or np.any(off[1:] < off[:-1]):
            raise ValueError("offsets must be non-decreasing from 0 to len(points)")
        dt = _as_pcf_dtype(pts.dtype)
        obj = cls.__new__(cls)
        n = len(off) - 1
        obj._init_csr(pts, off, dt, tuple(shape) if shape is not None else (n,))
        if validate:
            obj._validate()
        return obj

    def _validate(self):
        pts, off = self._pts, self._off
        lens = np.diff(off.astype(np.int64))
        if np.any(lens <= 0):
            raise ValueError("A PCF needs at least one breakpoint.")
        if len(lens) == 0:
            return
        t = pts[:, 0]
        if np.issubdtype(pts.dtype, np.floating) and not np.all(np.isfinite(t)):
            raise ValueError("Breakpoint times must be finite.")
        starts = off[:-1].astype(np.int64)
        if np.any(t[starts] != 0):
            raise ValueError("The first breakpoint must have time t=0.")
        dec = t[1:] < t[:-1]
        if dec.size:
            dec[starts[1:] - 1] = False  # boundaries between PCFs
            if np.any(dec):
                raise ValueError("Breakpoints must be given in non-decreasing time order.")

    # --- array protocol --------------------------------------------------------

    @property
    def shape(self):
        return self._index.shape

    @property
    def ndim(self):
        return self._index.ndim

    @property
    def dtype(self):
        return self._dtype

    @property
    def size(self):
        return int(self._index.size)

    def __len__(self):
        if self._index.ndim == 0:
            raise TypeError("len() of a 0-d PcfArray")
        return self._index.shape[0]

    def _pcf_at(self, k: int) -> Pcf:
        if k in self._edits:
            return self._edits[k]
        a, b = int(self._off[k]), int(self._off[k + 1])
        return Pcf._trusted(self._pts[a:b])

    def __getitem__(self, key):
        sub = self._index[key]
        if np.ndim(sub) == 0:
            return self._pcf_at(int(sub))
        view = PcfArray.__new__(PcfArray)
        view._pts, view._off, view._dtype = self._pts, self._off, self._dtype
        view._index = np.asarray(sub)
        view._edits = self._edits
        return view

    def __setitem__(self, key, value):
        sub = self._index[key]
        if np.ndim(sub) != 0:
            raise NotImplementedError("only single-element assignment is supported")
        if not isinstance(value, Pcf):
            raise TypeError(f"expected a Pcf, got {type(value).__name__}")
        if value._pts.dtype != self._dtype.np_dtype:
            raise TypeError(f"cannot assign a {value.dtype} PCF into a {self._dtype} array")
        self._edits[int(sub)] = value

    def __iter__(self):
        for k in range(len(self)):
            yield self[k]

    def __repr__(self):
        return f"PcfArray<{self._dtype}>(shape={self.shape})"

    # --- flat CSR in iteration order -----------------------------------------

    def csr(self):
        """``(points, offsets)`` of the PCFs in C order of ``self.shape``."""
        flat = self._index.reshape(-1)
        n_all = len(self._off) - 1
        if not self._edits and flat.size == n_all and np.array_equal(flat, np.arange(n_all)):
            return self._pts, self._off
        pieces = [self._pcf_at(int(k))._pts for k in flat]
        offsets = np.zeros(len(pieces) + 1, dtype=np.uint64)
        if pieces:
            np.cumsum([p.shape[0] for p in pieces], out=offsets[1:])
            pts = np.ascontiguousarray(np.concatenate(pieces).astype(self._dtype.np_dtype, copy=False))
        else:
            pts = np.zeros((0, 2), dtype=self._dtype.np_dtype)
        return pts, offsets


def zeros(shape, dtype=pcf32) -> PcfArray:
    """An array of zero PCFs (each ``[(0, 0)]``), as ``stablebear.zeros``."""
    dt = _as_pcf_dtype(dtype)
    if isinstance(shape, int):
        shape = (shape,)
    n = int(np.prod(shape, dtype=np.int64)) if len(shape) else 1
    pts = np.zeros((n, 2), dtype=dt.np_dtype)
    off = np.arange(n + 1, dtype=np.uint64)
    arr = PcfArray.__new__(PcfArray)
    arr._init_csr(pts, off, dt, tuple(shape))
    return arr


def _resolve_pcf_inputs(*items):
    """Turn PcfArray / list-of-Pcf / single Pcf inputs into PcfArrays of one
    dtype (stablebear/base_tensor.py:485-505)."""
    out = []
    for it in items:
        if isinstance(it, PcfArray):
            out.append(it)
        elif isinstance(it, Pcf):
            out.append(PcfArray([it]))
        elif isinstance(it, (list, tuple)):
            out.append(PcfArray(it) if len(it) else PcfArray([], dtype=pcf32))
        else:
            raise TypeError(f"expected a PcfArray, a Pcf or a list of Pcf, got {type(it).__name__}")
    if len({a.dtype.np_dtype for a in out}) > 1:
        raise TypeError("All inputs must have the same dtype.")
    return out
