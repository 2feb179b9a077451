"""Differentiable pairwise integrals: a ``torch.autograd.Function`` whose
forward is the pair kernel and whose backward is the hand-written backward
kernel (``sbg_pairwise_backward_device``).

The PCFs are a CUDA ``points`` tensor ``(M, 2)`` of ``(t, v)`` rows and an
``offsets`` tensor ``(N + 1,)`` (the reference's CSR).  The result is the
condensed matrix (``DistanceMatrix`` order for distances, ``SymmetricMatrix``
order for the kernel); ``condensed_to_dense`` expands it.  Gradients flow to
the values and to the breakpoint times (not to t = 0, and not at ties with a
breakpoint of the other PCF of a pair).  torch is plumbing here: device
memory and the autograd graph; both passes are native kernels.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as nat

_KINDS = {
    "l2_kernel": (nat.OP_L2_INNER, 1.0, nat.SKIP_LOWER),
    "l2": (nat.OP_LP, 2.0, nat.SKIP_LOWER_NODIAG),
    "l1": (nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG),
}


def _code(t):
    if t.dtype == torch.float32:
        return nat.F32
    if t.dtype == torch.float64:
        return nat.F64
    raise TypeError("points must be float32 or float64")


def _need_cuda(*tensors):
    for t in tensors:
        if not t.is_cuda:
            raise ValueError("the differentiable functions take CUDA tensors (the kernels read device memory)")


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


class PairwiseIntegral(torch.autograd.Function):
    @staticmethod
    def forward(ctx, points, offsets, kind, max_points):
        op, p, skip = _KINDS[kind]
        _need_cuda(points, offsets)
        points = points.contiguous()
        offsets = offsets.contiguous()
        n = offsets.numel() - 1
        count = int(nat.lib().sbg_output_count(skip, n, n))
        out = torch.empty(count, dtype=points.dtype, device=points.device)
        if count:
            nat.check(nat.lib().sbg_pairwise_device(_code(points), op, p, skip, points.data_ptr(), offsets.data_ptr(),
                                                    n, None, None, 0, None, None, int(max_points), out.data_ptr(), 0,
                                                    0, 0, _stream(points.device)))
        ctx.save_for_backward(points, offsets, out)
        ctx.kind = kind
        ctx.max_points = int(max_points)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        points, offsets, out = ctx.saved_tensors
        op, p, skip = _KINDS[ctx.kind]
        n = offsets.numel() - 1
        grad = torch.empty_like(points)
        go = grad_out.contiguous()
        nat.check(nat.lib().sbg_pairwise_backward_device(_code(points), op, p, skip, points.data_ptr(),
                                                         offsets.data_ptr(), n, points.shape[0], ctx.max_points,
                                                         go.data_ptr(), out.data_ptr(), grad.data_ptr(),
                                                         _stream(points.device)))
        return grad, None, None, None


def _max_points(offsets):
    return int((offsets[1:] - offsets[:-1]).max().item()) if offsets.numel() > 1 else 1


def l2_kernel(points, offsets, max_points=None):
    """Condensed L2 Gram matrix (SymmetricMatrix order), differentiable.
    ``max_points``: the largest PCF's breakpoint count, if the caller knows
    it (otherwise it is read from ``offsets``, which synchronises the
    stream); it must not be smaller than the true one."""
    mp = _max_points(offsets) if max_points is None else int(max_points)
    return PairwiseIntegral.apply(points, offsets, "l2_kernel", mp)


def pdist(points, offsets, p=2, max_points=None):
    """Condensed L1 or L2 distance matrix (DistanceMatrix order), differentiable;
    ``max_points`` as for ``l2_kernel``."""
    if p not in (1, 2):
        raise ValueError("gradients are implemented for p = 1 and p = 2")
    mp = _max_points(offsets) if max_points is None else int(max_points)
    return PairwiseIntegral.apply(points, offsets, "l1" if p == 1 else "l2", mp)


class _SymmetricExpand(torch.autograd.Function):
    """Condensed storage to the symmetric dense matrix on the device
    (``sbg_condensed_to_dense_device``); its gradient folds both mirror
    entries of dL/d(dense) back into the stored one
    (``sbg_dense_fold_to_condensed_device``)."""

    @staticmethod
    def forward(ctx, c, n, diagonal):
        skip = nat.SKIP_LOWER if diagonal else nat.SKIP_LOWER_NODIAG
        _need_cuda(c)
        n = int(n)
        c = c.contiguous()
        if c.numel() != int(nat.lib().sbg_output_count(skip, n, n)):
            raise ValueError(f"a condensed vector of {c.numel()} values is not a {n} x {n} matrix of this kind")
        dense = torch.empty((n, n), dtype=c.dtype, device=c.device)
        if n:
            nat.check(nat.lib().sbg_condensed_to_dense_device(_code(c), skip, n, c.data_ptr(), dense.data_ptr(), n, 0,
                                                              n, _stream(c.device)))
        ctx.n, ctx.skip = n, skip
        return dense

    @staticmethod
    def backward(ctx, grad_dense):
        g = grad_dense.contiguous()
        n = ctx.n
        gc = torch.empty(int(nat.lib().sbg_output_count(ctx.skip, n, n)), dtype=g.dtype, device=g.device)
        if n and gc.numel():
            nat.check(nat.lib().sbg_dense_fold_to_condensed_device(_code(g), ctx.skip, n, g.data_ptr(), n,
                                                                   gc.data_ptr(), _stream(g.device)))
        return gc, None, None


def condensed_to_dense(c, n, diagonal):
    """Expand a condensed vector to the symmetric n x n matrix (differentiable):
    ``diagonal`` True for SymmetricMatrix order (the L2 kernel), False for
    DistanceMatrix order (zero diagonal)."""
    return _SymmetricExpand.apply(c, n, diagonal)
