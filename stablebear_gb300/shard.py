"""One pairwise problem split over several GPUs, one process per GPU.

The path shards by row bands with no collective on the data path, as the
reference splits its tiles over GPUs with one worker per device
(``include/sbear/cuda/cuda_block_executor.cuh:128-151``):

* ``row_bands`` cuts the rows into one contiguous band per rank, each a whole
  number of 1024-PCF order windows (so every band runs in the length order)
  and holding about the same number of output elements;
* ``compute_band`` runs this rank's band through the stream-ordered device
  entry into a band-sized buffer: the band's results are exactly the
  contiguous output range ``band_output_range`` names;
* ``gather_to_rank0`` collects the bands on rank 0 (the only collective, after
  the computation, and only when the caller wants one matrix in one place).
"""
from __future__ import annotations

import ctypes

from . import _native as nat

WINDOW = 1024  # the device entry's processing-order window (rows per band are multiples of it)


def output_start(skip_mode: int, row: int, n_cols: int) -> int:
    """First output element of ``row`` (DistanceMatrix, SymmetricMatrix or dense order)."""
    if skip_mode == nat.SKIP_LOWER_NODIAG:
        return row * (row - 1) // 2 if row else 0
    if skip_mode == nat.SKIP_LOWER:
        return row * (row + 1) // 2
    return row * n_cols


def band_output_range(skip_mode: int, n: int, row_begin: int, row_end: int, n_cols: int | None = None):
    """``(lo, hi)``: the output elements a band of rows owns."""
    nc = n if n_cols is None else n_cols
    return output_start(skip_mode, row_begin, nc), output_start(skip_mode, row_end, nc)


def row_bands(n: int, world_size: int, skip_mode: int = nat.SKIP_LOWER_NODIAG, n_cols: int | None = None,
              align: int = WINDOW):
    """``world_size`` contiguous ``(row_begin, row_end)`` bands covering ``[0, n)``:
    boundaries are multiples of ``align`` and split the output elements about
    evenly (later rows of a triangle own more pairs).  Bands may be empty
    when there are fewer windows than ranks."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    nc = n if n_cols is None else n_cols
    total = output_start(skip_mode, n, nc)
    cuts = [0]
    for k in range(1, world_size):
        target = total * k / world_size
        lo, hi = cuts[-1], n
        while lo < hi:  # smallest row with output_start >= target
            mid = (lo + hi) // 2
            if output_start(skip_mode, mid, nc) >= target:
                hi = mid
            else:
                lo = mid + 1
        r = min(n, (lo + align // 2) // align * align)  # nearest window boundary
        cuts.append(max(cuts[-1], r))
    cuts.append(n)
    return [(cuts[k], cuts[k + 1]) for k in range(world_size)]


def compute_band(points, offsets, row_begin: int, row_end: int, op: int = nat.OP_L1, p: float = 1.0,
                 skip_mode: int = nat.SKIP_LOWER_NODIAG, max_points: int = 0):
    """This rank's band on its current CUDA device: ``(lo, values)`` with
    ``values`` the band's contiguous output range starting at element ``lo``."""
    import torch
    n = offsets.numel() - 1
    lo, hi = band_output_range(skip_mode, n, row_begin, row_end)
    out = torch.empty(hi - lo, dtype=points.dtype, device=points.device)
    if hi > lo:
        code = nat.F32 if points.dtype == torch.float32 else nat.F64
        nat.check(nat.lib().sbg_pairwise_device(code, op, float(p), skip_mode, points.data_ptr(), offsets.data_ptr(),
                                                n, None, None, 0, None, None, int(max_points), out.data_ptr(), lo,
                                                row_begin, row_end,
                                                ctypes.c_void_p(torch.cuda.current_stream(points.device).cuda_stream)))
    return lo, out


def gather_to_rank0(lo: int, values, total: int, group=None):
    """Assemble every rank's ``(lo, values)`` band into one length-``total``
    tensor on rank 0 (``None`` elsewhere).  Works with any backend
    ``torch.distributed`` is initialised with (NCCL on GPUs, gloo on CPUs)."""
    import torch
    import torch.distributed as dist
    ws = dist.get_world_size(group)
    rank = dist.get_rank(group)
    meta = torch.tensor([lo, values.numel()], dtype=torch.int64, device=values.device)
    metas = [torch.zeros_like(meta) for _ in range(ws)]
    dist.all_gather(metas, meta, group=group)
    longest = max(int(m[1]) for m in metas)
    padded = torch.zeros(longest, dtype=values.dtype, device=values.device)
    padded[: values.numel()] = values
    parts = [torch.zeros_like(padded) for _ in range(ws)] if rank == 0 else None
    dist.gather(padded, parts, dst=0, group=group)
    if rank != 0:
        return None
    out = torch.empty(total, dtype=values.dtype, device=values.device)
    for m, part in zip(metas, parts):
        a, k = int(m[0]), int(m[1])
        out[a:a + k] = part[:k]
    return out
