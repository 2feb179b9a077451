"""The differentiable functions hand device pointers to the kernels, so they
refuse host tensors before any native call (no GPU needed to check it)."""
import pytest


def test_autograd_functions_reject_host_tensors():
    import torch
    from stablebear_gb300 import autograd as ag
    pts = torch.zeros((4, 2))
    off = torch.tensor([0, 2, 4])
    with pytest.raises(ValueError, match="CUDA"):
        ag.l2_kernel(pts, off, max_points=2)
    with pytest.raises(ValueError, match="CUDA"):
        ag.pdist(pts, off, p=1, max_points=2)
    with pytest.raises(ValueError, match="CUDA"):
        ag.condensed_to_dense(torch.zeros(3), 3, False)
