"""Batched pairwise integration: many independent PCF arrays of uneven size
computed by one persistent launch (``sbg_batch_*`` in ``include/sbgpu.h``).

The reference computes one problem per task
(``include/sbear/cuda/pcf_block_op.cuh:127-203``); a batch plans all of them
once — PCFs of each problem visited in order of breakpoint count, problems
ordered by estimated merge work, largest first — and then launches them
together, optionally as a replayed CUDA graph.  Device memory is owned by
torch tensors (plumbing only; the computation is the native kernel).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as nat
from .matrices import DistanceMatrix, SymmetricMatrix
from .pcf import PcfArray, _resolve_pcf_inputs


class _Problem(ctypes.Structure):
    _fields_ = [("points", ctypes.c_void_p), ("offsets", ctypes.c_void_p), ("host_offsets", ctypes.c_void_p),
                ("n", ctypes.c_uint64), ("out", ctypes.c_void_p)]


_OPS = {"l1": (nat.OP_L1, nat.SKIP_LOWER_NODIAG), "lp": (nat.OP_LP, nat.SKIP_LOWER_NODIAG),
        "l2_kernel": (nat.OP_L2_INNER, nat.SKIP_LOWER)}


class PairwiseBatch:
    """A planned batch of pdist (``op="l1"`` / ``"lp"``) or L2 kernel
    (``op="l2_kernel"``) problems.

    ``problems``: a list of ``(points, offsets)`` CSR pairs (numpy, host).
    ``run()`` computes all problems on the current CUDA stream and returns
    the device outputs (torch tensors in condensed order).
    ``tune_window=True`` lets ``autotune()`` also move the time-windowed
    kernel's window cap (the split of shared memory between the column
    block and the row buffers); window ends then move, so sums may change in
    their last bits.  Without it no tuned setting changes a result.
    """

    def __init__(self, problems, op="l1", p=1.0, graph=True, caller_order=False, device=None, tune_window=False):
        import torch
        if op not in _OPS:
            raise ValueError(f"op must be one of {sorted(_OPS)}")
        opc, skip = _OPS[op]
        if op == "lp" and p < 1:
            raise ValueError("p must be >= 1.")
        if op == "lp" and p == 1:
            opc = nat.OP_L1
        self.op, self.p, self.skip = op, float(p), skip
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        dts = {np.dtype(pts.dtype) for pts, _ in problems}
        if len(dts) > 1:
            raise TypeError("All problems must have the same dtype.")
        self.np_dtype = dts.pop() if dts else np.dtype(np.float32)
        self.code = nat.F32 if self.np_dtype == np.float32 else nat.F64
        tdt = torch.float32 if self.code == nat.F32 else torch.float64
        self._keep = []
        self.outputs = []
        self.sizes = []
        arr = (_Problem * max(1, len(problems)))()
        for k, (pts, off) in enumerate(problems):
            pts = np.ascontiguousarray(pts)
            off = np.ascontiguousarray(off, dtype=np.uint64)
            n = len(off) - 1
            dp = torch.from_numpy(pts).to(self.device)
            do = torch.from_numpy(off.astype(np.int64)).to(self.device)
            count = int(nat.lib().sbg_output_count(skip, n, n))
            out = torch.empty(max(1, count), dtype=tdt, device=self.device)
            self._keep += [dp, do, off]
            self.outputs.append(out[:count])
            self.sizes.append(n)
            arr[k] = _Problem(dp.data_ptr(), do.data_ptr(), off.ctypes.data, n, out.data_ptr())
        h = ctypes.c_void_p()
        flags = ((nat.BATCH_GRAPH if graph else 0) | (nat.BATCH_CALLER_ORDER if caller_order else 0)
                 | (nat.BATCH_TUNE_WINDOW if tune_window else 0))
        nat.check(nat.lib().sbg_batch_create(self.code, opc, self.p, skip, ctypes.cast(arr, ctypes.c_void_p),
                                             len(problems), flags, ctypes.byref(h)))
        self._h = h

    def _stream(self):
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def run(self):
        nat.check(nat.lib().sbg_batch_launch(self._h, self._stream()))
        return self.outputs

    def autotune(self) -> float:
        ms = ctypes.c_double(0.0)
        nat.check(nat.lib().sbg_batch_autotune(self._h, self._stream(), ctypes.byref(ms)))
        return ms.value

    def info(self) -> dict:
        items, pairs = ctypes.c_uint64(), ctypes.c_uint64()
        warps, rows = ctypes.c_int(), ctypes.c_int()
        nat.check(nat.lib().sbg_batch_info(self._h, ctypes.byref(items), ctypes.byref(pairs), ctypes.byref(warps),
                                           ctypes.byref(rows)))
        split = ctypes.c_uint32()
        nat.check(nat.lib().sbg_batch_shared_split(self._h, ctypes.byref(split)))
        return {"items": items.value, "pairs": pairs.value, "warps": warps.value, "rows_per_item": rows.value,
                "column_elements": split.value}

    def matrices(self):
        """The results as host ``DistanceMatrix`` / ``SymmetricMatrix``."""
        cls = SymmetricMatrix if self.skip == nat.SKIP_LOWER else DistanceMatrix
        return [cls._wrap(n, o.cpu().numpy()) for n, o in zip(self.sizes, self.outputs)]

    def close(self):
        if getattr(self, "_h", None):
            nat.lib().sbg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _problems(arrays):
    probs = []
    for a in arrays:
        (X,) = _resolve_pcf_inputs(a)
        if len(X.shape) != 1:
            raise ValueError("1d tensor expected.")
        probs.append(X.csr())
    return probs


def pdist_batched(arrays, p=1, graph=False):
    """``pdist`` of every 1-D PCF array in ``arrays`` in one launch."""
    if p < 1:
        raise ValueError("p must be >= 1.")
    b = PairwiseBatch(_problems(arrays), op="l1" if p == 1 else "lp", p=p, graph=graph)
    try:
        b.run()
        return b.matrices()
    finally:
        b.close()


def l2_kernel_batched(arrays, graph=False):
    """``l2_kernel`` of every 1-D PCF array in ``arrays`` in one launch."""
    b = PairwiseBatch(_problems(arrays), op="l2_kernel", graph=graph)
    try:
        b.run()
        return b.matrices()
    finally:
        b.close()
