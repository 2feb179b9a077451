"""Barcodes to stable ranks and Betti curves on the GPU against the oracle's
restatement of the reference's loops: the points must be identical (times are
copied or subtracted once, values are exact counts)."""
import numpy as np
import pytest

import stablebear_gb300 as sb
from stablebear_gb300 import persistence as pers
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _random_barcodes(n, max_bars, dt, seed, big=None):
    rng = np.random.default_rng(seed)
    bcs = []
    for i in range(n):
        m = int(rng.integers(0, max_bars + 1)) if big is None or i % 7 else big
        birth = rng.uniform(0, 4, m)
        life = rng.exponential(1.0, m)
        if i % 3 == 0:
            birth = np.round(birth * 4) / 4      # ties between bars
            life = np.round(life * 4) / 4        # zero-length bars and equal lifetimes
        death = birth + life
        inf = rng.random(m) < 0.05
        death[inf] = np.inf
        death[rng.random(m) < 0.02] = np.finfo(dt).max
        if i % 11 == 5 and m:
            birth[0] = 0.0                       # an event at t = 0
        bcs.append(np.column_stack([birth, death]).astype(dt))
    return bcs


def _oracle(bcs, kind):
    dt = bcs[0].dtype
    bars = np.concatenate(bcs).astype(dt) if bcs else np.zeros((0, 2), dt)
    off = np.zeros(len(bcs) + 1, np.uint64)
    np.cumsum([len(b) for b in bcs], out=off[1:])
    return orc.barcodes_to_pcfs(bars, off, kind)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("kind", [pers.STABLE_RANK, pers.BETTI_CURVE])
def test_random_barcodes_match_oracle(dt, kind):
    # barcodes longer than the shared-memory sort (4096 keys f32, 2048 f64)
    # take the global-memory path
    bcs = _random_barcodes(300, 60, dt, seed=kind * 10 + (dt == np.float64), big=2500)
    fn = pers.barcode_to_stable_rank if kind == pers.STABLE_RANK else pers.barcode_to_betti_curve
    got = fn(bcs)
    gp, go = got.csr()
    wp, wo = _oracle(bcs, kind)
    np.testing.assert_array_equal(go, wo)
    np.testing.assert_array_equal(gp, wp)


def test_single_barcodes_and_shapes():
    bc = pers.Barcode(np.array([[0.0, 1.0], [0.0, 3.0], [0.0, 2.0], [0.0, np.inf], [1.0, 3.0]]))
    sr = pers.barcode_to_stable_rank(bc)
    np.testing.assert_array_equal(np.asarray(sr), [[0, 5], [1, 4], [2, 2], [3, 1]])
    bt = pers.barcode_to_betti_curve(pers.Barcode(np.array([[0.0, 2.0], [1.0, 3.0], [0.5, 1.5]])))
    np.testing.assert_array_equal(np.asarray(bt), [[0, 1], [0.5, 2], [1, 3], [1.5, 2], [2, 1], [3, 0]])
    empty = pers.barcode_to_stable_rank(pers.Barcode(np.zeros((0, 2))))
    np.testing.assert_array_equal(np.asarray(empty), [[0, 0]])
    grid = np.empty((2, 3), dtype=object)
    for i in range(2):
        for j in range(3):
            grid[i, j] = pers.Barcode(np.array([[0.0, 1.0 + i + j], [0.5, 2.0]], np.float32))
    out = pers.barcode_to_betti_curve(grid)
    assert out.shape == (2, 3)
    for i in range(2):
        for j in range(3):
            np.testing.assert_array_equal(np.asarray(out[i, j]), np.asarray(pers.barcode_to_betti_curve(grid[i, j])))
    with pytest.raises(TypeError, match="same dtype"):
        pers.barcode_to_stable_rank([np.zeros((1, 2), np.float32), np.zeros((1, 2), np.float64)])


def test_device_chain_into_l2_kernel():
    """Stable ranks made on the device feed the differentiable kernel matrix
    directly; the result equals the host path on the same PCFs."""
    import torch
    from stablebear_gb300 import autograd
    bcs = _random_barcodes(120, 40, np.float32, seed=3)
    bcs = [b[np.isfinite(b[:, 1]) & (b[:, 1] < np.finfo(np.float32).max)] for b in bcs]  # finite tails
    bars = np.concatenate(bcs)
    off = np.zeros(len(bcs) + 1, np.int64)
    np.cumsum([len(b) for b in bcs], out=off[1:])
    pts, poff = pers.barcodes_to_pcfs_device(torch.from_numpy(bars).cuda(), torch.from_numpy(off).cuda())
    K = autograd.l2_kernel(pts[: int(poff[-1].item())], poff).cpu().numpy()
    srs = pers.barcode_to_stable_rank(bcs)
    want = sb.l2_kernel(srs).data
    np.testing.assert_allclose(K, want, rtol=1e-5, atol=1e-5 * np.abs(want).max())
