"""The device entry that allocates nothing (sbg_pairwise_device_noalloc).

It exists for callers that may not allocate device memory at the moment they
need a matrix (an application whose own allocator owns all device memory, a
component running inside someone else's graph capture, a plugin host that
only lends buffers).  The test calls it through the C ABI twice in a row and
checks each result against sbg_pairwise_device, the allocating entry point,
with the tolerance the other parity tests use (float32: 1e-5 relative; here
the two paths run the same kernel, so the results are in fact identical).
Both calls run with the library's device-allocation limit at zero, and the
test checks that the library's allocation counter and the device's free
memory do not move.  It also checks the clear rejection of a problem too
large for the fixed scratch (the hybrid kernel's packed copy of long PCFs).
This file is collected last so a failure here cannot hide others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    from stablebear_gb300 import build
    build.build()
    import torch
    from stablebear_gb300 import _native as nat
    assert torch.cuda.is_available()
    return torch, nat


def _device_csr(torch, pts, off):
    return torch.from_numpy(pts).cuda(), torch.from_numpy(off.astype(np.int64)).cuda()


def _run_pair(torch, nat, pts, off, skip, op, p):
    dp, do = _device_csr(torch, pts, off)
    n = len(off) - 1
    count = int(nat.lib().sbg_output_count(skip, n, n))
    lmax = int(np.diff(off.astype(np.int64)).max())
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    code = nat.F32 if pts.dtype == np.float32 else nat.F64
    tdt = torch.float32 if pts.dtype == np.float32 else torch.float64
    ref = torch.full((count,), float("nan"), dtype=tdt, device="cuda")
    nat.check(nat.lib().sbg_pairwise_device(code, op, p, skip, dp.data_ptr(), do.data_ptr(), n, None, None, 0,
                                            None, None, lmax, ref.data_ptr(), 0, 0, 0, st))
    outs = [torch.full((count,), float("nan"), dtype=tdt, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    # Both calls run with the library's allocation limit at 0, so any device
    # allocation through the library's allocator would fail the call; its
    # allocation counter must not move, and the device's free memory must be
    # the same before and after the second call (the first may still load
    # kernels, which the driver does lazily).
    lib = nat.lib()
    allocs = lib.sbg_device_allocations()
    lib.sbg_set_alloc_limit(0)
    try:
        for k, got in enumerate(outs):  # two calls in a row share the scratch
            if k == 1:
                torch.cuda.synchronize()
                free_before = torch.cuda.mem_get_info()[0]
            nat.check(lib.sbg_pairwise_device_noalloc(code, op, p, skip, dp.data_ptr(), do.data_ptr(), n,
                                                      int(off[-1]), None, None, 0, 0, None, None, lmax,
                                                      got.data_ptr(), 0, 0, 0, st))
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
    finally:
        lib.sbg_set_alloc_limit(nat.ALLOC_UNLIMITED)
    assert lib.sbg_device_allocations() == allocs
    assert free_after == free_before
    ref = ref.cpu().numpy().astype(np.float64)
    for got in outs:
        g = got.cpu().numpy().astype(np.float64)
        assert not np.isnan(g).any()
        rel = np.abs(g - ref) / np.maximum(np.abs(ref), 1.0 if op == nat.OP_L2_INNER else 1e-30)
        assert rel.max() <= TOL


def test_no_alloc_matches_allocating_entry(env):
    torch, nat = env
    from stablebear_gb300 import synthetic
    pts, off = synthetic.plain_l1(700, seed=31)
    _run_pair(torch, nat, pts, off, nat.SKIP_LOWER_NODIAG, nat.OP_L1, 1.0)
    _run_pair(torch, nat, pts, off, nat.SKIP_LOWER, nat.OP_L2_INNER, 1.0)


@pytest.mark.parametrize("variant", [0, 4])
def test_no_alloc_long_pcfs(env, variant):
    """PCFs too long for the plain shared-memory layout: the time-windowed
    kernel (the default) reads the breakpoints in place; the hybrid kernel
    (variant 4) puts its packed copy into the fixed scratch."""
    torch, nat = env
    from stablebear_gb300 import synthetic
    lens = np.array([3, 9000, 5, 1, 7000, 12] * 5)
    pts, off = synthetic.gaussian(len(lens), lens, np.float32, seed=5)
    nat.check(nat.lib().sbg_set_tuning(0, 0, variant, 0, 0))
    try:
        _run_pair(torch, nat, pts, off, nat.SKIP_LOWER_NODIAG, nat.OP_LP, 2.0)
    finally:
        nat.check(nat.lib().sbg_set_tuning(0, 0, 0, 0, 0))


def test_no_alloc_rejects_oversized_problem(env):
    torch, nat = env
    from stablebear_gb300 import synthetic
    lens = np.full(20, 40_000)  # 800k long breakpoints: more packed scratch than the fixed array holds
    pts, off = synthetic.gaussian(len(lens), lens, np.float32, seed=6)
    dp, do = _device_csr(torch, pts, off)
    out = torch.empty(190, dtype=torch.float32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # the hybrid kernel needs a packed copy of the breakpoints in the scratch
    nat.check(nat.lib().sbg_set_tuning(0, 0, 4, 0, 0))
    try:
        rc = nat.lib().sbg_pairwise_device_noalloc(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                                   do.data_ptr(), 20, int(off[-1]), None, None, 0, 0, None, None,
                                                   40_000, out.data_ptr(), 0, 0, 0, st)
        msg = nat.last_error()
    finally:
        nat.check(nat.lib().sbg_set_tuning(0, 0, 0, 0, 0))
    assert rc == -1
    assert "scratch" in msg and "limit" in msg
    # the time-windowed kernel (the default) reads the breakpoints in place
    ref = torch.empty(190, dtype=torch.float32, device="cuda")
    nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                            do.data_ptr(), 20, None, None, 0, None, None, 40_000, ref.data_ptr(),
                                            0, 0, 0, st))
    nat.check(nat.lib().sbg_pairwise_device_noalloc(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                                    do.data_ptr(), 20, int(off[-1]), None, None, 0, 0, None, None,
                                                    40_000, out.data_ptr(), 0, 0, 0, st))
    assert torch.equal(out, ref)
    assert nat.lib().sbg_pairwise_device_noalloc(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                                 do.data_ptr(), 20, int(off[-1]), None, None, 0, 0, None, None, 0,
                                                 out.data_ptr(), 0, 0, 0, st) == -1
    torch.cuda.synchronize()
