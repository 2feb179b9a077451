"""lp_norm on the GPU (sbg_lp_norm_host / sbg_lp_norm_device) against the
reference's norms (golden fixture from its iterate_segments) and the oracle.
The GPU adds the segments of a PCF in 32 lane-strided partial sums, the
reference in order: f32 within 1e-5 relative, f64 within 1e-12."""
import ctypes
import os

import numpy as np
import pytest

import stablebear_gb300 as sb
from oracle import oracle as orc
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = {"f32": 1e-5, "f64": 1e-12}


def _rel(a, b):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)) if len(b) else 0.0


@pytest.mark.parametrize("tag", ["f32", "f64"])
@pytest.mark.parametrize("p", [1.0, 1.5, 2.0, 3.0])
def test_norms_match_reference_golden(tag, p):
    d = np.load(os.path.join(GOLDEN, "reference_norms.npz"))
    X = sb.PcfArray.from_csr(d[f"{tag}_points"], d[f"{tag}_offsets"])
    got = sb.lp_norm(X, p=p)
    assert got.dtype == d[f"{tag}_p{p}"].dtype
    assert _rel(got, d[f"{tag}_p{p}"]) <= TOL[tag]


def test_known_answers_and_shape():
    X = sb.zeros((2, 3), dtype=sb.pcf64)
    X[0, 0] = sb.Pcf(np.array([[0.0, 10.0], [2.0, 5.0], [4.0, 0.0]]))
    X[0, 1] = sb.Pcf(np.array([[0.0, 5.0], [3.0, 6.0], [5.0, 5.0], [8.0, 0.0]]))
    X[0, 2] = sb.Pcf(np.array([[0.0, 12.0], [3.0, 0.0]]))
    X[1, 0] = sb.Pcf(np.array([[0.0, 50.0], [0.5, 0.0]]))
    X[1, 1] = sb.Pcf(np.array([[0.0, 0.0]]))
    X[1, 2] = sb.Pcf(np.array([[0.0, 2.0], [3.0, 0.0]]))
    got = sb.lp_norm(X, p=1)
    assert got.shape == (2, 3)
    np.testing.assert_allclose(got, [[30, 42, 36], [25, 0, 6]], rtol=1e-12)
    for bad in (0.5, 0, -1):
        with pytest.raises(ValueError, match="p must be >= 1"):
            sb.lp_norm(X, p=bad)


@pytest.mark.parametrize("dt,tag", [(np.float32, "f32"), (np.float64, "f64")])
def test_random_long_pcfs_against_oracle(dt, tag):
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(3000, synthetic.uniform_lengths(1, 700), dt, seed=12)
    X = sb.PcfArray.from_csr(pts, off)
    for p in (1.0, 2.0, 2.5):
        assert _rel(sb.lp_norm(X, p=p), orc.lp_norm(pts, off, p)) <= TOL[tag]


def test_device_entry_on_caller_stream():
    import torch
    from stablebear_gb300 import _native as nat, synthetic
    pts, off = synthetic.gaussian(500, synthetic.uniform_lengths(1, 90), np.float32, seed=2)
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    out = torch.empty(500, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        nat.check(nat.lib().sbg_lp_norm_device(nat.F32, 1.0, dp.data_ptr(), do.data_ptr(), 500, out.data_ptr(),
                                               ctypes.c_void_p(s.cuda_stream)))
    s.synchronize()
    assert _rel(out.cpu().numpy(), orc.lp_norm(pts, off, 1.0)) <= 1e-5
