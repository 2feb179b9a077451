"""The host entry's automatic band schedule against the device entry, bit for
bit, over the whole output.

Above 512 MB of output the host entry cuts the condensed matrix into bands of
whole 1024-PCF windows, taken from the last row down; the two lowest bands
are cut again into parts of about half the remaining output each, bands
alternate between two compute streams, and a band with few work items takes
fewer rows per item.  None of this may change a bit of a result: every pair's
arithmetic is the same as in the single device call.  N = 16,500 short PCFs
give 545 MB of output, just above the threshold, in a few milliseconds of
compute.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def native():
    from stablebear_gb300 import build
    build.build()


def _device_pdist(pts, off):
    import torch
    from stablebear_gb300 import _native as nat
    n = len(off) - 1
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    out = torch.full((n * (n - 1) // 2,), float("nan"), dtype=torch.float32, device="cuda")
    lmax = int(np.diff(off.astype(np.int64)).max())
    st = torch.cuda.current_stream().cuda_stream
    nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                            do.data_ptr(), n, None, None, 0, None, None, lmax, out.data_ptr(), 0, 0,
                                            0, ctypes.c_void_p(st)))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("row_chunk", [0, 3, 12])
def test_auto_bands_match_device_entry(capfd, row_chunk):
    """row_chunk: rows per work item / 32 fixed by the caller (0: the
    planner's); a band that takes fewer rows per item halves only an even
    chunk, so 3 stays 3 and 12 may become 6 or 3."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import _native as nat, synthetic
    n = 16500
    pts, off = synthetic.gaussian(n, synthetic.uniform_lengths(4, 24), np.float32, seed=21)
    assert n * (n - 1) // 2 * 4 > 512 << 20
    sb.set_tuning(row_chunk=row_chunk)
    try:
        want = _device_pdist(pts, off)
        nat.lib().sbg_set_device_verbose(1)
        try:
            got = sb.pdist(sb.PcfArray.from_csr(pts, off)).data
        finally:
            nat.lib().sbg_set_device_verbose(0)
    finally:
        sb.set_tuning()
    np.testing.assert_array_equal(got, want)
    # the phase report: one line per call, with a mark per band
    err = capfd.readouterr().err
    line = [ln for ln in err.splitlines() if ln.startswith("sbgpu host entry")]
    assert len(line) == 1
    bands = [tok for tok in line[0].split() if tok.startswith("band")]
    assert len(bands) > 4 and "synced" in line[0] and "freed" in line[0]


def test_auto_bands_cdist_match_device_entry():
    """The same schedule on a dense cross (cdist) output, whose rows all hold
    the same output: 12,000 x 12,000 float32 (576 MB)."""
    import torch
    import stablebear_gb300 as sb
    from stablebear_gb300 import _native as nat, synthetic
    nr = nc = 12000
    xp, xo = synthetic.gaussian(nr, synthetic.uniform_lengths(4, 20), np.float32, seed=31)
    yp, yo = synthetic.gaussian(nc, synthetic.uniform_lengths(4, 20), np.float32, seed=32)
    assert nr * nc * 4 > 512 << 20
    got = sb.cdist(sb.PcfArray.from_csr(xp, xo), sb.PcfArray.from_csr(yp, yo), p=1)
    lmax = int(max(np.diff(xo.astype(np.int64)).max(), np.diff(yo.astype(np.int64)).max()))
    dx, dxo = torch.from_numpy(xp).cuda(), torch.from_numpy(xo.astype(np.int64)).cuda()
    dy, dyo = torch.from_numpy(yp).cuda(), torch.from_numpy(yo.astype(np.int64)).cuda()
    out = torch.full((nr * nc,), float("nan"), dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_NONE, dx.data_ptr(), dxo.data_ptr(),
                                            nr, dy.data_ptr(), dyo.data_ptr(), nc, None, None, lmax,
                                            out.data_ptr(), 0, 0, 0, ctypes.c_void_p(st)))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(np.asarray(got).reshape(-1), out.cpu().numpy())
