"""Single-problem launch-shape autotuning (sbg_autotune_device) and its cache.

The autotuner times (warps per CTA, rows per work item) shapes on the real
problem and caches the fastest under (element type, operation, skip mode,
shape bucket).  Neither knob changes a result bit (the time-windowed kernel
keeps the default plan's window cap under a cached shape), so the test
checks that a cached shape is found again and used, and that shapes pinned
in the cache give the same bits as the default plan, for the plain
shared-memory kernel and the time-windowed one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    from stablebear_gb300 import build
    build.build()
    import torch
    from stablebear_gb300 import _native as nat
    nat.check(nat.lib().sbg_tuning_cache_clear())
    yield torch, nat
    nat.check(nat.lib().sbg_tuning_cache_clear())
    nat.lib().sbg_set_tuning(0, 0, 0, 0, 0)


def _run(torch, nat, dp, do, n, lmax, out, op=0, p=1.0):
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    nat.check(nat.lib().sbg_pairwise_device(nat.F32, op, p, nat.SKIP_LOWER_NODIAG, dp.data_ptr(), do.data_ptr(), n,
                                            None, None, 0, None, None, lmax, out.data_ptr(), 0, 0, 0, st))
    torch.cuda.synchronize()
    return out.cpu().numpy().copy()


@pytest.mark.parametrize("kind", ["plain", "windowed"])
def test_autotune_caches_a_shape_and_keeps_every_bit(env, kind):
    torch, nat = env
    from stablebear_gb300 import synthetic
    lib = nat.lib()
    if kind == "plain":
        pts, off = synthetic.plain_l1(3000, seed=21)
    else:
        pts, off = synthetic.gaussian(1500, synthetic.uniform_lengths(8, 1024), np.float32, seed=22)
    n = len(off) - 1
    lmax = int(np.diff(off.astype(np.int64)).max())
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    out = torch.empty(n * (n - 1) // 2, device="cuda")
    default = _run(torch, nat, dp, do, n, lmax, out)

    hit = ctypes.c_int(-1)
    w, r = ctypes.c_int(0), ctypes.c_int(0)
    nat.check(lib.sbg_tuning_cache_lookup(nat.F32, 0, 1.0, nat.SKIP_LOWER_NODIAG, n, lmax, ctypes.byref(w),
                                          ctypes.byref(r), ctypes.byref(hit)))
    assert hit.value == 0
    ms = ctypes.c_double(0)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    nat.check(lib.sbg_autotune_device(nat.F32, 0, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(), do.data_ptr(), n,
                                      None, None, 0, lmax, out.data_ptr(), st, ctypes.byref(w), ctypes.byref(r),
                                      ctypes.byref(ms)))
    assert w.value in (16, 24, 32) and r.value % 32 == 0 and 32 <= r.value <= 1024 and ms.value > 0
    tuned_w, tuned_r = w.value, r.value
    # the cache holds the shape for this key (and for another problem of the same bucket)
    for nn in (n, n + 1):
        nat.check(lib.sbg_tuning_cache_lookup(nat.F32, 0, 1.0, nat.SKIP_LOWER_NODIAG, nn, lmax, ctypes.byref(w),
                                              ctypes.byref(r), ctypes.byref(hit)))
        assert hit.value == 1 and (w.value, r.value) == (tuned_w, tuned_r)
    # another operation is another key
    nat.check(lib.sbg_tuning_cache_lookup(nat.F32, 2, 1.0, nat.SKIP_LOWER, n, lmax, ctypes.byref(w),
                                          ctypes.byref(r), ctypes.byref(hit)))
    assert hit.value == 0
    # the default call now plans with the cached shape: same bits
    np.testing.assert_array_equal(_run(torch, nat, dp, do, n, lmax, out), default)
    # and so does every other shape pinned in the cache for this key
    for warps, rows in ((16, 32), (32, 64), (24, 128), (32, 1024)):
        nat.check(lib.sbg_tuning_cache_store(nat.F32, 0, 1.0, nat.SKIP_LOWER_NODIAG, n, lmax, warps, rows))
        np.testing.assert_array_equal(_run(torch, nat, dp, do, n, lmax, out), default)
    nat.check(lib.sbg_tuning_cache_clear())
    nat.check(lib.sbg_tuning_cache_lookup(nat.F32, 0, 1.0, nat.SKIP_LOWER_NODIAG, n, lmax, ctypes.byref(w),
                                          ctypes.byref(r), ctypes.byref(hit)))
    assert hit.value == 0
