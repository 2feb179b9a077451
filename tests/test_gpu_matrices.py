"""condensed <-> dense on the GPU (sbg_condensed_to_dense_device,
sbg_dense_to_condensed_device) against the host containers: bitwise equal
values, row bands, strided outputs, and the reference's from_dense checks."""
import numpy as np
import pytest

import stablebear_gb300 as sb
from stablebear_gb300 import device as dev

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 31, 32, 33, 100, 257]


def _storage(n, kind, dt, seed):
    rng = np.random.default_rng(seed)
    cls = sb.DistanceMatrix if kind == "distance" else sb.SymmetricMatrix
    st = rng.uniform(0, 10, cls.storage_size(n)).astype(dt)
    return cls._wrap(n, st)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("kind", ["distance", "symmetric"])
def test_condensed_to_dense_matches_host(dt, kind):
    import torch
    for n in SIZES:
        m = _storage(n, kind, dt, n)
        got = dev.condensed_to_dense(torch.from_numpy(m.data).cuda(), n, kind).cpu().numpy()
        np.testing.assert_array_equal(got, m.to_dense())


@pytest.mark.parametrize("kind", ["distance", "symmetric"])
def test_row_bands_and_strided_out(kind):
    import torch
    n = 203
    m = _storage(n, kind, np.float32, 7)
    want = m.to_dense()
    st = torch.from_numpy(m.data).cuda()
    for rb, re in ((0, 0), (0, 1), (5, 6), (31, 97), (64, 128), (190, 203), (0, 203), (150, 999)):
        got = dev.condensed_to_dense(st, n, kind, rb, re).cpu().numpy()
        np.testing.assert_array_equal(got, want[rb:min(re, n)])
    big = torch.full((40, n + 13), -7.0, device="cuda")
    out = big[:, :n]
    dev.condensed_to_dense(st, n, kind, 100, 140, out=out)
    np.testing.assert_array_equal(out.cpu().numpy(), want[100:140])
    assert (big[:, n:] == -7.0).all()  # nothing written past the row


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("kind", ["distance", "symmetric"])
def test_dense_to_condensed_round_trip(dt, kind):
    import torch
    for n in SIZES:
        m = _storage(n, kind, dt, 100 + n)
        d = torch.from_numpy(m.to_dense()).cuda()
        got = dev.dense_to_condensed(d, kind).cpu().numpy()
        np.testing.assert_array_equal(got, m.data)


def test_dense_to_condensed_checks():
    import torch
    n = 70
    m = _storage(n, "distance", np.float64, 3)
    base = torch.from_numpy(m.to_dense()).cuda()
    d = base.clone()
    d[40, 3] += 1.0
    with pytest.raises(ValueError, match="Matrix must be symmetric"):
        dev.dense_to_condensed(d, "distance")
    with pytest.raises(ValueError, match="Matrix must be symmetric"):
        dev.dense_to_condensed(d, "symmetric")
    d = base.clone()
    d[65, 65] = 0.5
    with pytest.raises(ValueError, match="Diagonal entries must be zero"):
        dev.dense_to_condensed(d, "distance")
    dev.dense_to_condensed(d, "symmetric")  # a diagonal is fine for a SymmetricMatrix
    d = base.clone()
    d[10, 50] = d[50, 10] = -1.0
    with pytest.raises(ValueError, match="Entries must be nonnegative"):
        dev.dense_to_condensed(d, "distance")
    d = base.clone()
    d[1, 2] = float("nan")
    d[2, 1] = float("nan")
    with pytest.raises(ValueError, match="Matrix must be symmetric"):
        dev.dense_to_condensed(d, "distance")
    # unchecked: values come through regardless
    got = dev.dense_to_condensed(d, "distance", check=False)
    assert np.isnan(got[2 * 1 // 2 + 1].item())


def test_pdist_result_to_dense_on_device():
    """The autograd path's device-resident condensed result expands to the
    same dense matrix as the host DistanceMatrix of sb.pdist."""
    import torch
    from stablebear_gb300 import synthetic, autograd
    pts, off = synthetic.gaussian(150, synthetic.uniform_lengths(2, 60), np.float32, seed=4)
    X = sb.PcfArray.from_csr(pts, off)
    host = sb.pdist(X).to_dense()
    P = torch.from_numpy(pts).cuda()
    O = torch.from_numpy(off.astype(np.int64)).cuda()
    cond = autograd.pdist(P, O, p=1)
    got = dev.condensed_to_dense(cond.detach(), 150, "distance").cpu().numpy()
    # the host path may visit PCFs in length order, which regroups the
    # compensated sums: equal to f32 rounding, not bitwise
    np.testing.assert_allclose(got, host, rtol=1e-5, atol=0)
    assert (np.diag(got) == 0).all()


def test_argument_errors():
    import torch
    st = torch.zeros(10, device="cuda")
    with pytest.raises(ValueError, match="needs 15"):
        dev.condensed_to_dense(st, 5, "symmetric")
    with pytest.raises(ValueError, match="kind"):
        dev.condensed_to_dense(st, 5, "dense")
    with pytest.raises(ValueError, match="CUDA"):
        dev.condensed_to_dense(torch.zeros(10), 5)
    with pytest.raises(ValueError, match="square"):
        dev.dense_to_condensed(torch.zeros((3, 4), device="cuda"))
    with pytest.raises(TypeError):
        dev.condensed_to_dense(torch.zeros(10, dtype=torch.int32, device="cuda"), 5)
