"""Barcodes and their PCF summaries, computed on the GPU.

``barcode_to_stable_rank`` and ``barcode_to_betti_curve`` have the names,
arguments and results of ``stablebear/persistence/barcode_summary.py:42-95``:
a single ``Barcode`` gives a ``Pcf``, an array of barcodes gives a
``PcfArray`` of the same shape.  The reference converts barcode by barcode on
the CPU; here one call converts the whole array (``sbg_barcodes_to_pcfs_host``,
one CTA per barcode).  ``barcodes_to_pcfs_device`` keeps everything on the
device, so persistence summaries feed ``autograd.l2_kernel`` / ``pdist``
without a host round trip.

A ``Barcode`` holds an ``(n, 2)`` float32 or float64 array of
``(birth, death)`` rows; an infinite bar has death ``inf`` or the dtype's
maximum (``include/sbear/persistence/barcode.hpp:18-21``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as nat
from .pcf import PcfArray

STABLE_RANK, BETTI_CURVE = 0, 1


class Barcode:
    """A persistence barcode: ``(birth, death)`` pairs."""

    def __init__(self, bc):
        if isinstance(bc, Barcode):
            self._bars = bc._bars
            return
        if not isinstance(bc, np.ndarray) or bc.dtype not in (np.float32, np.float64):
            raise TypeError(f"Barcode cannot be constructed with object of type {type(bc)}")
        bars = np.ascontiguousarray(bc)
        if bars.size == 0:
            bars = bars.reshape(0, 2)
        if bars.ndim != 2 or bars.shape[1] != 2:
            raise ValueError("a barcode is an (n, 2) array of (birth, death) pairs")
        self._bars = bars

    @property
    def dtype(self):
        return self._bars.dtype

    def __len__(self):
        return self._bars.shape[0]

    def to_numpy(self) -> np.ndarray:
        return self._bars.copy()

    def __array__(self, dtype=None, copy=None):
        return self._bars if dtype is None else self._bars.astype(dtype, copy=False)

    def __repr__(self):
        return f"Barcode({len(self)} bars, dtype={self._bars.dtype})"


def _collect(bc):
    """(list of Barcodes in C order, shape or None for a single barcode)."""
    if isinstance(bc, Barcode):
        return [bc], None
    if isinstance(bc, np.ndarray) and bc.dtype != object:
        return [Barcode(bc)], None
    arr = np.empty(len(bc), dtype=object) if not isinstance(bc, np.ndarray) else bc
    if not isinstance(bc, np.ndarray):
        for i, b in enumerate(bc):
            arr[i] = b
    items = [b if isinstance(b, Barcode) else Barcode(b) for b in arr.reshape(-1)]
    return items, arr.shape


def _csr(items):
    dts = {b.dtype for b in items}
    if len(dts) > 1:
        raise TypeError("All barcodes must have the same dtype.")
    dt = dts.pop() if dts else np.dtype(np.float32)
    offs = np.zeros(len(items) + 1, dtype=np.uint64)
    np.cumsum([len(b) for b in items], out=offs[1:])
    bars = (np.ascontiguousarray(np.concatenate([b._bars for b in items]).astype(dt, copy=False))
            if items else np.zeros((0, 2), dt))
    return bars, offs, dt


def _convert(bc, kind):
    items, shape = _collect(bc)
    bars, boff, dt = _csr(items)
    n = len(items)
    code = nat.F32 if dt == np.float32 else nat.F64
    cap = nat.lib().sbg_barcode_pcf_capacity(kind, n, int(boff[-1]))
    pts = np.zeros((max(cap, 1), 2), dtype=dt)
    off = np.zeros(n + 1, dtype=np.uint64)
    if n:
        nat.check(nat.lib().sbg_barcodes_to_pcfs_host(kind, code, nat.ptr(bars), nat.ptr(boff), n, nat.ptr(pts), cap,
                                                      nat.ptr(off)))
    pts = pts[: int(off[-1])]
    out = PcfArray.from_csr(pts, off, shape=shape if shape is not None else (n,), validate=False)
    if shape is None:
        return out._pcf_at(0)
    return out


def barcode_to_stable_rank(bc, verbose=False):
    r"""Stable rank of each barcode: the PCF counting, for each :math:`t \geq 0`,
    the bars whose length (death minus birth) is greater than :math:`t`."""
    return _convert(bc, STABLE_RANK)


def barcode_to_betti_curve(bc, verbose=False):
    r"""Betti curve of each barcode: the PCF counting, for each :math:`t`, the
    bars alive at :math:`t` (birth :math:`\leq t <` death)."""
    return _convert(bc, BETTI_CURVE)


def barcodes_to_pcfs_device(bars, bar_offsets, kind="stable_rank", stream=None):
    """Device-resident conversion: ``bars`` an ``(M, 2)`` CUDA tensor of
    ``(birth, death)`` rows and ``bar_offsets`` an ``int64`` CUDA tensor of
    ``n + 1`` offsets.  Returns ``(points, offsets)`` CUDA tensors: the PCFs'
    points occupy ``points[:offsets[-1]]`` (the tensor is sized for the upper
    bound, so nothing is read back to the host)."""
    import torch
    k = {"stable_rank": STABLE_RANK, "betti_curve": BETTI_CURVE}.get(kind, kind)
    if k not in (STABLE_RANK, BETTI_CURVE):
        raise ValueError("kind must be 'stable_rank' or 'betti_curve'")
    if not bars.is_cuda or not bar_offsets.is_cuda:
        raise ValueError("bars and bar_offsets must be CUDA tensors")
    if bars.dtype not in (torch.float32, torch.float64):
        raise TypeError("bars must be float32 or float64")
    bars = bars.contiguous()
    boff = bar_offsets.contiguous()
    n = boff.numel() - 1
    cap = nat.lib().sbg_barcode_pcf_capacity(k, n, bars.shape[0])
    pts = torch.empty((max(cap, 1), 2), dtype=bars.dtype, device=bars.device)
    off = torch.empty(n + 1, dtype=torch.int64, device=bars.device)
    s = stream if stream is not None else torch.cuda.current_stream(bars.device)
    code = nat.F32 if bars.dtype == torch.float32 else nat.F64
    nat.check(nat.lib().sbg_barcodes_to_pcfs_device(k, code, bars.data_ptr(), boff.data_ptr(), n, bars.shape[0],
                                                    pts.data_ptr(), cap, off.data_ptr(),
                                                    ctypes.c_void_p(s.cuda_stream)))
    return pts, off
