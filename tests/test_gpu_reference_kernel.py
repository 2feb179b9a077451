"""The reference's own CUDA block kernel, run on this GPU from a cubin of the
reference's headers (oracle/ref_gpu_kernel.cu, oracle/ref_gpu.cpp), against
the oracle and against this library.

This checks the harness that times the reference kernel for comparison: the
reference kernel drives one thread per pair over dense tiles from the
reference's scheduler, and its results agree with the reference's CPU
algorithm within the reference's own GPU-vs-CPU tolerance (float32 1e-5,
Lp 1e-4; test/test_block_integrate.cu:33,194).  Skipped where the cubin has
not been built (it needs the reference tree at build time).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    from stablebear_gb300 import build
    build.build()
    from oracle import oracle as orc
    ok = orc.ref_gpu_kernel_available()
    if ok is not True:
        pytest.skip(ok)
    import torch
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(1500, synthetic.uniform_lengths(1, 150), np.float32, seed=21)
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    torch.cuda.synchronize()
    return orc, pts, off, dp, do


def rel(got, want, floor=1e-30):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), floor)))


@pytest.mark.parametrize("op,p,tol", [("l1", 1.0, 1e-5), ("lp", 2.5, 1e-4)])
def test_reference_kernel_pdist(env, op, p, tol):
    import stablebear_gb300 as sb
    orc, pts, off, dp, do = env
    n = len(off) - 1
    out = np.full(n * (n - 1) // 2, np.nan, np.float32)
    # a small output budget: several tiles, including partial and diagonal ones
    ms, tiles = orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), n, op=op, p=p, host_out=out,
                                     max_output_elements=500_000)
    assert tiles > 1 and ms > 0
    assert not np.isnan(out).any()
    oop = orc.OP_L1 if op == "l1" else orc.OP_LP
    assert rel(out, orc.evaluate(pts, off, op=oop, p=p)) <= tol
    # this library's compensated sums against the double-double truth
    ours = sb.pdist(sb.PcfArray.from_csr(pts, off), p=p).data
    assert rel(ours, orc.evaluate(pts, off, op=oop, p=p, truth=True)) <= tol


@pytest.mark.parametrize("kernel", [False, True])
def test_reference_kernel_sampled_rows_equal_the_full_scatter(env, kernel):
    """The row-sampled copy-back (used beside the headline bench, where the
    full triangle is 20 GB) returns the same bits as the full host scatter."""
    orc, pts, off, dp, do = env
    n = len(off) - 1
    full = np.full(n * (n + 1) // 2 if kernel else n * (n - 1) // 2, np.nan, np.float32)
    orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), n, kernel=kernel, host_out=full,
                         max_output_elements=300_000)
    rows = np.array([0, 1, 2, 700, 701, 1499, 350, 1024], np.uint64)
    ms, tiles, vals, starts = orc.ref_gpu_triangle_rows(dp.data_ptr(), do.data_ptr(), n, rows, kernel=kernel,
                                                        max_output_elements=300_000)
    assert tiles > 1 and ms > 0
    per = 1 if kernel else 0
    for k, i in enumerate(int(r) for r in rows):
        lo = i * (i + 1) // 2 if kernel else i * (i - 1) // 2
        np.testing.assert_array_equal(vals[starts[k]:starts[k + 1]], full[lo:lo + i + per])


def test_reference_kernel_l2_kernel(env):
    import stablebear_gb300 as sb
    orc, pts, off, dp, do = env
    n = len(off) - 1
    out = np.full(n * (n + 1) // 2, np.nan, np.float32)
    ms, tiles = orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), n, kernel=True, host_out=out)
    assert tiles >= 1 and not np.isnan(out).any()
    want = orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL)
    assert rel(out, want, floor=1.0) <= 1e-5
    # the two naive float32 sums (the reference kernel's and this library's
    # compensated one) can differ by the naive sum's own error; this
    # library's is checked against the double-double truth
    ours = sb.l2_kernel(sb.PcfArray.from_csr(pts, off)).data
    truth = orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL, truth=True)
    assert rel(ours, truth, floor=1.0) <= 1e-5


def test_reference_kernel_f64(env):
    """Double precision (the stable-rank workload's type): the reference's own
    GPU-vs-CPU tolerance for double is 1e-10 (test/test_block_integrate.cu:43)."""
    import torch
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    orc = env[0]
    pts, off = synthetic.stable_rank(400, seed=3)
    n = len(off) - 1
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    out = np.full(n * (n + 1) // 2, np.nan, np.float64)
    orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), n, kernel=True, host_out=out, dtype=np.float64)
    want = orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL)
    assert rel(out, want, floor=1.0) <= 1e-10
    ours = sb.l2_kernel(sb.PcfArray.from_csr(pts, off)).data
    assert rel(ours, want, floor=1.0) <= 1e-12
