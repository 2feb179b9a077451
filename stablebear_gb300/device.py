"""Device-resident results: condensed <-> dense on the GPU.

A pairwise result computed on the device (``autograd.pdist``,
``autograd.l2_kernel``, ``sbg_pairwise_device``) stays in HBM in the
reference's condensed order.  These functions expand it to a dense matrix, or
condense a dense device matrix, without a host round trip; the reference does
both with serial host loops over all n^2 entries
(``src/python/py_distance_matrix.hpp:37-73``,
``src/python/py_symmetric_matrix.hpp:62-81``).

``kind`` is ``"distance"`` (DistanceMatrix storage: ``n(n-1)/2`` values, zero
diagonal) or ``"symmetric"`` (SymmetricMatrix storage: ``n(n+1)/2`` values);
the classes themselves are accepted too.
"""
from __future__ import annotations

import ctypes

from . import _native as nat
from .matrices import DistanceMatrix, SymmetricMatrix


def _kind(kind) -> int:
    if kind in ("distance", DistanceMatrix):
        return nat.SKIP_LOWER_NODIAG
    if kind in ("symmetric", SymmetricMatrix):
        return nat.SKIP_LOWER
    raise ValueError("kind must be 'distance' or 'symmetric'")


def _dtype_code(t) -> int:
    import torch
    if t.dtype == torch.float32:
        return nat.F32
    if t.dtype == torch.float64:
        return nat.F64
    raise TypeError(f"Unsupported dtype {t.dtype}; use float32 or float64")


def _stream(t):
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def condensed_to_dense(storage, n: int, kind="distance", row_begin: int = 0, row_end: int | None = None,
                       out=None):
    """Rows ``[row_begin, row_end)`` of the dense ``n x n`` matrix whose
    condensed storage is the CUDA tensor ``storage``; returns a
    ``(row_end - row_begin, n)`` tensor (``out`` if given, which may have a
    row stride larger than ``n``)."""
    import torch
    skip = _kind(kind)
    if not storage.is_cuda:
        raise ValueError("storage must be a CUDA tensor")
    storage = storage.contiguous()
    n = int(n)
    want = nat.lib().sbg_output_count(skip, n, n)
    if storage.numel() != want:
        raise ValueError(f"storage holds {storage.numel()} values; a {n} x {n} matrix of this kind needs {want}")
    row_end = n if row_end is None else min(int(row_end), n)
    row_begin = int(row_begin)
    if row_begin < 0 or row_begin > row_end:
        raise ValueError("need 0 <= row_begin <= row_end")
    rows = row_end - row_begin
    if out is None:
        out = torch.empty((rows, n), dtype=storage.dtype, device=storage.device)
    else:
        if out.dtype != storage.dtype or out.device != storage.device:
            raise ValueError("out must match storage's dtype and device")
        if out.dim() != 2 or out.shape[0] != rows or out.shape[1] != n or out.stride(1) != 1:
            raise ValueError(f"out must be a ({rows}, {n}) tensor with unit column stride")
    ld = out.stride(0) if rows > 1 else max(n, 1)
    with torch.cuda.device(storage.device):
        nat.check(nat.lib().sbg_condensed_to_dense_device(_dtype_code(storage), skip, n, storage.data_ptr(),
                                                          out.data_ptr(), ld, row_begin, row_end, _stream(storage)))
    return out


def dense_to_condensed(dense, kind="distance", check: bool = True):
    """Condensed storage of the square CUDA matrix ``dense``.  With
    ``check``, raises ``ValueError`` with the reference's message when the
    matrix is not symmetric, or (distance) has a non-zero diagonal or a
    negative entry; the flags are read back, which synchronises the stream."""
    import torch
    skip = _kind(kind)
    if not dense.is_cuda:
        raise ValueError("dense must be a CUDA tensor")
    if dense.dim() != 2:
        raise ValueError("Expected a 2-D array")
    if dense.shape[0] != dense.shape[1]:
        raise ValueError("Expected a square array")
    if dense.stride(1) != 1:
        dense = dense.contiguous()
    n = dense.shape[0]
    out = torch.empty(nat.lib().sbg_output_count(skip, n, n), dtype=dense.dtype, device=dense.device)
    flags = torch.zeros(1, dtype=torch.int32, device=dense.device)
    ld = dense.stride(0) if n > 1 else max(n, 1)
    with torch.cuda.device(dense.device):
        nat.check(nat.lib().sbg_dense_to_condensed_device(_dtype_code(dense), skip, n, dense.data_ptr(), ld,
                                                          out.data_ptr(), flags.data_ptr(), _stream(dense)))
    if check:
        f = int(flags.item())
        if f & nat.FLAG_DIAGONAL:
            raise ValueError("Diagonal entries must be zero")
        if f & nat.FLAG_NEGATIVE:
            raise ValueError("Entries must be nonnegative")
        if f & nat.FLAG_ASYMMETRIC:
            raise ValueError("Matrix must be symmetric")
    return out
