"""compute_band on one GPU: the bands of row_bands, computed one after the
other, are the whole matrix bit for bit (each rank of a multi-GPU run
computes one of them)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3])
def test_bands_assemble_the_whole_matrix(world):
    import torch
    from stablebear_gb300 import _native as nat, shard, synthetic, autograd
    pts, off = synthetic.gaussian(3500, synthetic.uniform_lengths(1, 80), np.float32, seed=world)
    P = torch.from_numpy(pts).cuda()
    O = torch.from_numpy(off.astype(np.int64)).cuda()
    n = len(off) - 1
    lmax = int(np.diff(off.astype(np.int64)).max())
    whole = autograd.pdist(P, O, p=1)
    total = torch.empty_like(whole)
    for rb, re in shard.row_bands(n, world):
        lo, vals = shard.compute_band(P, O, rb, re, max_points=lmax)
        total[lo:lo + vals.numel()] = vals
    torch.cuda.synchronize()
    assert torch.equal(total, whole)
