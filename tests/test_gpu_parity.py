"""Parity of the CUDA path against the reference (golden fixtures made by the
reference's own code) and against the oracle on seeded inputs.

Tolerances (written here, used throughout):
  float32: relative 1e-5 (Lp with general p: 1e-4, the reference's own
           GPU-vs-CPU tolerance, test/test_block_integrate.cu:194,301);
  float64: relative 1e-12 (Lp with general p: 1e-10).
For the L2 kernel, whose terms cancel, the error is measured against
max(|ref|, 1) (values here are O(1)-O(100)).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f32": 1e-5, "f64": 1e-12}
TOL_LP = {"f32": 1e-4, "f64": 1e-10}


@pytest.fixture(scope="module", autouse=True)
def native():
    from stablebear_gb300 import build
    build.build()
    import stablebear_gb300 as sb
    assert sb.get_ngpus() >= 1, "no CUDA device"
    yield
    sb.set_tuning()


def rel_err(got, want, floor=1e-30):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    both_inf = np.isinf(got) & np.isinf(want) & (np.sign(got) == np.sign(want))
    d = np.abs(got - want)
    d[both_inf] = 0.0
    r = d / np.maximum(np.abs(want), floor)
    r[both_inf] = 0.0
    return float(np.max(r)) if r.size else 0.0


def arr(points, offsets):
    import stablebear_gb300 as sb
    return sb.PcfArray.from_csr(points, offsets)


def cross_native(pts, off, ypts, yoff, op, p):
    """cdist through the C ABI's cdist task (any op, incl. the cross kernel
    of create_cuda_block_cdist_l2_kernel_task)."""
    from stablebear_gb300 import _native as nat
    from stablebear_gb300.task import StoppableTask, _run_task
    nx, ny = len(off) - 1, len(yoff) - 1
    out = np.zeros(nx * ny, dtype=pts.dtype)
    h = ctypes.c_void_p()
    code = nat.F32 if pts.dtype == np.float32 else nat.F64
    nat.check(nat.lib().sbg_create_cdist_task(code, op, float(p), nat.ptr(pts), nat.ptr(off), nx, nat.ptr(ypts),
                                              nat.ptr(yoff), ny, nat.ptr(out), ctypes.byref(h)))
    t = StoppableTask(h, keepalive=(out,)).start()
    _run_task(lambda: t, verbose=False)
    return out


@pytest.mark.parametrize("case", ["ragged", "tails", "ties"])
def test_matches_reference_golden(golden_pairwise, tag, case):
    import stablebear_gb300 as sb
    g = golden_pairwise
    name = f"{case}_{tag}"
    pts, off = g[f"{name}__points"], g[f"{name}__offsets"]
    ypts, yoff = g[f"cols_{tag}__points"], g[f"cols_{tag}__offsets"]
    X = arr(pts, off)
    tol, tol_lp = TOL[tag], TOL_LP[tag]
    assert rel_err(sb.pdist(X).data, g[f"{name}__pdist_l1"]) <= tol
    assert rel_err(sb.pdist(X, p=2).data, g[f"{name}__pdist_l2"]) <= tol
    assert rel_err(sb.pdist(X, p=3).data, g[f"{name}__pdist_l3"]) <= tol_lp
    assert rel_err(sb.l2_kernel(X).data, g[f"{name}__kernel"], floor=1.0) <= tol
    Y = arr(ypts, yoff)
    assert rel_err(sb.cdist(X, Y).reshape(-1), g[f"{name}__cdist_l1"]) <= tol
    assert rel_err(sb.cdist(X, Y, p=1.5).reshape(-1), g[f"{name}__cdist_l15"]) <= tol_lp
    assert rel_err(cross_native(pts, off, ypts, yoff, 2, 1.0), g[f"{name}__cdist_l2k"], floor=1.0) <= tol


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_known_answers(dt):
    import stablebear_gb300 as sb
    pdt = sb.pcf32 if dt == np.float32 else sb.pcf64
    X = sb.zeros((2,), dtype=pdt)
    X[0] = sb.Pcf(np.array([[0.0, 10.0], [2.0, 5.0], [3.0, 0.0]], dtype=dt))
    X[1] = sb.Pcf(np.array([[0.0, 5.0], [6.0, 0.0]], dtype=dt))
    D = sb.pdist(X)
    assert D.size == 2 and D[0, 0] == 0.0 and D[0, 1] == pytest.approx(25.0) and D[1, 0] == D[0, 1]
    dense = D.to_dense()
    assert dense.shape == (2, 2) and dense[0, 1] == pytest.approx(25.0)

    X[0] = sb.Pcf(np.array([[0.0, 4.0], [1.0, 0.0]], dtype=dt))
    X[1] = sb.Pcf(np.array([[0.0, 1.0], [1.0, 0.0]], dtype=dt))
    assert sb.pdist(X, p=3)[0, 1] == pytest.approx(3.0)

    X[0] = sb.Pcf(np.array([[0.0, 4.0], [3.0, 0.0]], dtype=dt))
    X[1] = sb.Pcf(np.array([[0.0, 2.0], [3.0, 0.0]], dtype=dt))
    K = sb.l2_kernel(X)
    assert K[0, 0] == pytest.approx(48.0, rel=1e-5)
    assert K[0, 1] == pytest.approx(24.0, rel=1e-5)
    assert K[1, 1] == pytest.approx(12.0, rel=1e-5)
    one = sb.zeros((1,), dtype=pdt)
    one[0] = sb.Pcf(np.array([[0.0, 3.0], [2.0, 0.0]], dtype=dt))
    assert sb.l2_kernel(one)[0, 0] == pytest.approx(18.0, rel=1e-5)
    # test/test_l1_dist.cu:98-124: default PCFs are 0 apart, {(0,3),(1,0)} vs {(0,1),(2,0)} is 3
    assert sb.pdist(sb.zeros((2,), dtype=pdt))[0, 1] == 0.0
    f = sb.Pcf(np.array([[0, 3], [1, 0]], dtype=dt))
    g = sb.Pcf(np.array([[0, 1], [2, 0]], dtype=dt))
    assert sb.pdist([f, g])[0, 1] == pytest.approx(3.0, abs=1e-6)
    assert sb.lp_distance(f, g) == pytest.approx(3.0)
    assert sb.lp_distance(f, g, p=2) == pytest.approx(np.sqrt(4 + 1))


def test_lp_distance_closed_forms_on_gpu():
    import stablebear_gb300 as sb
    from tests.test_oracle import LP_CASES
    for dt in (np.float32, np.float64):
        for f, g, p, want in LP_CASES:
            got = sb.lp_distance(sb.Pcf(np.array(f, dtype=dt)), sb.Pcf(np.array(g, dtype=dt)), p=p)
            assert got == pytest.approx(want, rel=1e-6, abs=1e-6)


def test_empty_and_tiny_inputs():
    import stablebear_gb300 as sb
    D = sb.pdist(sb.zeros((0,)))
    assert isinstance(D, sb.DistanceMatrix) and D.size == 0
    D1 = sb.pdist(sb.zeros((1,)))
    assert D1.size == 1 and D1[0, 0] == 0.0
    K0 = sb.l2_kernel(sb.zeros((0,)))
    assert K0.size == 0
    assert sb.pdist([]).size == 0
    C = sb.cdist(sb.zeros((0,)), sb.zeros((3,)))
    assert C.shape == (0, 3)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n", [2, 31, 33, 97, 300])
def test_random_problems_against_oracle(dt, n):
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    from oracle import oracle as orc
    tag = "f32" if dt == np.float32 else "f64"
    pts, off = synthetic.gaussian(n, synthetic.uniform_lengths(1, 90), dt, seed=n)
    X = arr(pts, off)
    assert rel_err(sb.pdist(X).data, orc.evaluate(pts, off)) <= TOL[tag]
    assert rel_err(sb.pdist(X, p=2).data, orc.evaluate(pts, off, op=orc.OP_LP, p=2.0)) <= TOL[tag]
    assert rel_err(sb.pdist(X, p=2.5).data, orc.evaluate(pts, off, op=orc.OP_LP, p=2.5)) <= TOL_LP[tag]
    assert rel_err(sb.l2_kernel(X).data, orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL),
                   floor=1.0) <= TOL[tag]
    ypts, yoff = synthetic.gaussian(45, synthetic.uniform_lengths(1, 70), dt, seed=n + 1000)
    got = sb.cdist(X, arr(ypts, yoff))
    assert got.shape == (n, 45)
    want = orc.evaluate(pts, off, mode=orc.MODE_CROSS, col_points=ypts, col_offsets=yoff)
    assert rel_err(got.reshape(-1), want) <= TOL[tag]


def test_accuracy_against_fp64_truth_at_scale():
    """Poisson(256)+2 PCFs (the large pdist workload's shape), sampled rows
    against the double-double oracle: compensated FP32 stays within 1e-5."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    from oracle import oracle as orc
    pts, off = synthetic.large_l1(3000, seed=5)
    D = sb.pdist(arr(pts, off))
    rows = np.array([1, 2, 500, 1501, 2047, 2999], dtype=np.uint64)
    truth, starts = orc.evaluate_rows(pts, off, rows, truth=True)
    naive, _ = orc.evaluate_rows(pts, off, rows)
    got = np.concatenate([D.data[int(i) * (int(i) - 1) // 2: int(i) * (int(i) - 1) // 2 + int(i)] for i in rows])
    assert rel_err(got, truth) <= 1e-5
    assert rel_err(got, naive) <= 1e-5


def test_variants_orders_and_bands_agree():
    """Shared-memory vs global-memory kernel, caller vs length-sorted order,
    one band vs many: the same values (bitwise for the per-pair arithmetic
    that does not depend on orientation)."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(700, synthetic.uniform_lengths(1, 200), np.float32, seed=9)
    X = arr(pts, off)
    try:
        sb.set_tuning(variant=1, order=1)
        base = sb.pdist(X).data.copy()
        sb.set_tuning(variant=2, order=1)
        gm = sb.pdist(X).data.copy()
        sb.set_tuning(variant=1, order=1, band_bytes=64 << 10)
        banded = sb.pdist(X).data.copy()
        sb.set_tuning(variant=1, order=2)
        srt = sb.pdist(X).data.copy()
        sb.set_tuning(variant=1, order=1, warps=4, row_chunk=1)
        small = sb.pdist(X).data.copy()
        sb.set_tuning(variant=4, order=1)
        hyb = sb.pdist(X).data.copy()
        sb.set_tuning(variant=3, order=1)
        two = sb.pdist(X).data.copy()
        sb.set_tuning(variant=5, order=1)
        one = sb.pdist(X).data.copy()
    finally:
        sb.set_tuning()
    np.testing.assert_array_equal(hyb, base)
    np.testing.assert_array_equal(two, base)
    np.testing.assert_array_equal(one, base)
    np.testing.assert_array_equal(gm, base)
    np.testing.assert_array_equal(banded, base)
    np.testing.assert_array_equal(small, base)
    # zero-width rectangles add nothing, so neither the processing order nor
    # which PCF of a pair is the warp's row changes a bit of the result
    np.testing.assert_array_equal(srt, base)


def test_long_pcfs():
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    from oracle import oracle as orc
    lens = np.array([3, 5000, 7, 1, 4096, 12] * 6)
    pts, off = synthetic.gaussian(len(lens), lens, np.float32, seed=4)
    X = arr(pts, off)
    # 5000-rectangle sums: the naive FP32 reference itself drifts by more
    # than 1e-5 here, so the bound is against the FP64 oracle, and against
    # the reference within its own error plus 1e-5.
    for got, op, mode in ((sb.pdist(X).data, orc.OP_L1, orc.MODE_PDIST),
                          (sb.l2_kernel(X).data, orc.OP_L2, orc.MODE_KERNEL)):
        floor = 1.0 if op == orc.OP_L2 else 1e-30
        truth = orc.evaluate(pts, off, op=op, mode=mode, truth=True)
        naive = orc.evaluate(pts, off, op=op, mode=mode)
        assert rel_err(got, truth, floor) <= 1e-5
        assert rel_err(got, naive, floor) <= rel_err(naive, truth, floor) + 1e-5


def test_cdist_self_equals_pdist():
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    pts, off = synthetic.plain_l1(150, seed=8)
    X = arr(pts, off)
    C = sb.cdist(X, X)
    D = sb.pdist(X).to_dense()
    np.testing.assert_allclose(C, D, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(C, C.T, rtol=1e-5, atol=1e-6)


def test_device_entry_matches_host_entry():
    """sbg_pairwise_device on torch-owned device buffers equals the host
    pipeline bit for bit: the whole output (both visit the PCFs in the same
    length order), and two row bands in caller order against the host entry
    in caller order."""
    import torch
    import stablebear_gb300 as sb
    from stablebear_gb300 import _native as nat, synthetic
    pts, off = synthetic.plain_l1(800, seed=12)
    host = sb.pdist(arr(pts, off)).data
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    n = len(off) - 1
    out = torch.full((n * (n - 1) // 2,), float("nan"), dtype=torch.float32, device="cuda")
    lmax = int(np.diff(off.astype(np.int64)).max())
    st = torch.cuda.current_stream().cuda_stream
    nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                            do.data_ptr(), n, None, None, 0, None, None, lmax, out.data_ptr(), 0, 0,
                                            0, ctypes.c_void_p(st)))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), host)
    sb.set_tuning(order=1)
    try:
        host = sb.pdist(arr(pts, off)).data
    finally:
        sb.set_tuning()
    # two bands written into separate buffers (row_begin a multiple of 512)
    cut = 512
    lo = torch.empty(cut * (cut - 1) // 2, dtype=torch.float32, device="cuda")
    hi = torch.empty(n * (n - 1) // 2 - cut * (cut - 1) // 2, dtype=torch.float32, device="cuda")
    nat.check(nat.lib().sbg_set_tuning(0, 16, 0, 0, 0))
    try:
        nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                                do.data_ptr(), n, None, None, 0, None, None, lmax, lo.data_ptr(), 0,
                                                0, cut, ctypes.c_void_p(st)))
        nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                                do.data_ptr(), n, None, None, 0, None, None, 0, hi.data_ptr(),
                                                cut * (cut - 1) // 2, cut, n, ctypes.c_void_p(st)))
    finally:
        nat.check(nat.lib().sbg_set_tuning(0, 0, 0, 0, 0))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(np.concatenate([lo.cpu().numpy(), hi.cpu().numpy()]), host)


def test_task_progress_and_stop():
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    from stablebear_gb300.distance import Distance_f32_f32
    pts, off = synthetic.plain_l1(2000, seed=2)
    X = arr(pts, off)
    task, dm = Distance_f32_f32.pdist_l1(X)
    task.wait()
    assert task.work_completed() == task.work_total() == 2000 * 1999 // 2
    assert task.work_step_unit() == "integral"
    task.close()


def test_task_stop_cancels():
    """A stop requested right after start is honoured between bands: the
    worker returns SBG_ERR_CANCELLED (InterruptedError in Python), once, and
    the task reports less work completed than its total
    (include/sbear/task.hpp:21-31, rethrown once by wait_for at :84-96).
    With 256 KB bands the N = 6000 triangle (72 MB) has about 280 bands, each a
    kernel launch plus a synchronised copy, so the worker cannot finish them
    all before the stop request a few microseconds after start."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    from stablebear_gb300.distance import Distance_f32_f32
    pts, off = synthetic.plain_l1(6000, seed=2)
    X = arr(pts, off)
    sb.set_tuning(band_bytes=256 << 10)
    try:
        task, dm = Distance_f32_f32.pdist_l1(X)
        task.request_stop()
        with pytest.raises(InterruptedError, match="cancelled"):
            task.wait()
        assert task.stop_requested()
        assert 0 < task.work_completed() < task.work_total() == 6000 * 5999 // 2
        task.wait()  # the error surfaces once
        task.close()
        # the next task runs to completion and matches an uncancelled run
        task, dm = Distance_f32_f32.pdist_l1(X[:300])
        task.wait()
        task.close()
        np.testing.assert_array_equal(dm.data, sb.pdist(X[:300]).data)
    finally:
        sb.set_tuning()


def test_alloc_limit_injects_out_of_memory():
    """Host-side fault injection of the allocation failure (the reference's
    CHK_CUDA path, include/sbear/cuda/cuda_util.cuh:8-10): with a limit below
    what a call needs, the call fails with SBG_ERR_OUT_OF_MEMORY
    (MemoryError) before it touches device memory, on the device entry, the
    blocking host entry and a task (whose worker error surfaces from wait);
    with the limit lifted the same calls succeed."""
    import ctypes
    import torch
    import stablebear_gb300 as sb
    from stablebear_gb300 import _native as nat, synthetic
    from stablebear_gb300.distance import Distance_f32_f32
    lib = nat.lib()
    pts, off = synthetic.plain_l1(500, seed=9)
    n = 500
    want = sb.pdist(arr(pts, off)).data
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    out = torch.full((n * (n - 1) // 2,), -1.0, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def device_call():
        return lib.sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(), do.data_ptr(),
                                       n, None, None, 0, None, None, 0, out.data_ptr(), 0, 0, 0, st)

    held = lib.sbg_device_bytes_held()
    try:
        assert lib.sbg_set_alloc_limit(0) == 0
        allocs = lib.sbg_device_allocations()
        assert device_call() == nat.SBG_ERR_OUT_OF_MEMORY
        assert "sbg_set_alloc_limit" in nat.last_error()
        torch.cuda.synchronize()
        assert bool((out == -1.0).all())                      # nothing ran
        with pytest.raises(MemoryError, match="refused"):
            sb.pdist(arr(pts, off))                          # blocking host entry
        task, dm = Distance_f32_f32.pdist_l1(arr(pts, off))  # task: the worker's error, once
        with pytest.raises(MemoryError):
            task.wait()
        task.wait()
        task.close()
        assert lib.sbg_device_allocations() == allocs
        assert lib.sbg_device_bytes_held() == held
    finally:
        lib.sbg_set_alloc_limit(nat.ALLOC_UNLIMITED)
    assert device_call() == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), want)
    np.testing.assert_array_equal(sb.pdist(arr(pts, off)).data, want)
    assert lib.sbg_device_bytes_held() == held


def test_invalid_input_raises_value_error():
    import stablebear_gb300 as sb
    with pytest.raises(ValueError, match="p must be >= 1"):
        sb.pdist(sb.zeros((2,)), p=0.5)
    with pytest.raises(ValueError):
        sb.pdist(sb.zeros((10, 20)))
    sb.pdist(sb.zeros((10, 20))[:, 2])
    with pytest.raises(ValueError):
        sb.l2_kernel(sb.zeros((10, 20)))
    with pytest.raises(TypeError, match="same dtype"):
        sb.cdist(sb.PcfArray([sb.Pcf(np.array([[0.0, 1.0]], dtype=np.float32))]),
                 sb.PcfArray([sb.Pcf(np.array([[0.0, 1.0]], dtype=np.float64))]))
    with pytest.raises(TypeError):
        sb.lp_distance(sb.Pcf(np.array([[0, 1], [1, 0]], dtype=np.int32)), sb.Pcf(np.array([[0, 0]], dtype=np.int32)))


def _window_order(lens, w=1024):
    """Stable sort by length inside each window of w consecutive PCFs."""
    return np.concatenate([k + np.argsort(lens[k:k + w], kind="stable") for k in range(0, len(lens), w)])


def test_length_order_permutation():
    """sbg_length_order_device is the windowed stable sort by length, for
    sizes below one window, at whole windows, and with a padded last window
    of either parity."""
    import torch
    from stablebear_gb300 import _native as nat
    rng = np.random.default_rng(0)
    for n in (1, 2, 37, 1024, 1025, 2049, 3000, 20000, 100000):
        lens = rng.integers(1, 400, n)
        off = np.zeros(n + 1, np.int64)
        np.cumsum(lens, out=off[1:])
        do = torch.from_numpy(off).cuda()
        perm = torch.empty(n, dtype=torch.int32, device="cuda")
        nat.check(nat.lib().sbg_length_order_device(do.data_ptr(), n, perm.data_ptr(),
                                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        got = perm.cpu().numpy().view(np.uint32)
        np.testing.assert_array_equal(got, _window_order(lens))


def test_device_length_order_is_the_stable_length_sort():
    """The device entry's own processing order (computed on the GPU) gives
    the same bits as passing the windowed stable length sort as the
    permutation, for pdist, the kernel matrix and cdist."""
    import torch
    from stablebear_gb300 import _native as nat, synthetic
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n, lo, hi in ((3000, 1, 300), (37, 1, 9), (2049, 5, 6), (20000, 1, 40)):
        pts, off = synthetic.gaussian(n, synthetic.uniform_lengths(lo, hi), np.float32, seed=n)
        lens = np.diff(off.astype(np.int64))
        perm = torch.from_numpy(_window_order(lens).astype(np.uint32).view(np.int32)).cuda()
        dp = torch.from_numpy(pts).cuda()
        do = torch.from_numpy(off.astype(np.int64)).cuda()
        lmax = int(lens.max())
        for skip, op, p in ((nat.SKIP_LOWER_NODIAG, nat.OP_L1, 1.0), (nat.SKIP_LOWER, nat.OP_L2_INNER, 1.0)):
            cnt = nat.lib().sbg_output_count(skip, n, n)
            a = torch.empty(cnt, device="cuda")
            b = torch.empty(cnt, device="cuda")
            nat.check(nat.lib().sbg_pairwise_device(nat.F32, op, p, skip, dp.data_ptr(), do.data_ptr(), n, None, None,
                                                    0, None, None, lmax, a.data_ptr(), 0, 0, 0, st))
            nat.check(nat.lib().sbg_pairwise_device(nat.F32, op, p, skip, dp.data_ptr(), do.data_ptr(), n, None, None,
                                                    0, perm.data_ptr(), None, lmax, b.data_ptr(), 0, 0, 0, st))
            torch.cuda.synchronize()
            assert torch.equal(a, b)
        # cdist: rows and columns ordered separately
        m = max(2, n // 3)
        cp, co = pts[: int(off[m])], off[: m + 1]
        cperm = torch.from_numpy(_window_order(np.diff(co.astype(np.int64))).astype(np.uint32)
                                 .view(np.int32)).cuda()
        dcp = torch.from_numpy(np.ascontiguousarray(cp)).cuda()
        dco = torch.from_numpy(co.astype(np.int64)).cuda()
        a = torch.empty(n * m, device="cuda")
        b = torch.empty(n * m, device="cuda")
        nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_NONE, dp.data_ptr(), do.data_ptr(),
                                                n, dcp.data_ptr(), dco.data_ptr(), m, None, None, lmax, a.data_ptr(),
                                                0, 0, 0, st))
        nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_NONE, dp.data_ptr(), do.data_ptr(),
                                                n, dcp.data_ptr(), dco.data_ptr(), m, perm.data_ptr(),
                                                cperm.data_ptr(), lmax, b.data_ptr(), 0, 0, 0, st))
        torch.cuda.synchronize()
        assert torch.equal(a, b)


def test_kernel_launch_counter():
    """sbg_kernel_launches counts the kernels of a call: one pair kernel in
    caller order; the length order adds its sort kernels."""
    import torch
    import stablebear_gb300 as sb
    from stablebear_gb300 import _native as nat, synthetic
    lib = nat.lib()
    pts, off = synthetic.plain_l1(600, seed=2)
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    n = len(off) - 1
    out = torch.empty(n * (n - 1) // 2, device="cuda")
    lmax = int(np.diff(off.astype(np.int64)).max())
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call():
        before = lib.sbg_kernel_launches()
        nat.check(lib.sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                          do.data_ptr(), n, None, None, 0, None, None, lmax, out.data_ptr(), 0, 0, 0,
                                          st))
        return lib.sbg_kernel_launches() - before

    sb.set_tuning(order=1)
    try:
        assert call() == 1
    finally:
        sb.set_tuning()
    assert call() > 1


def test_bands_in_length_order_match_one_band():
    """The host pipeline in length order, cut into bands of whole order
    windows, gives the bits of one band, for pdist, the kernel matrix and
    cdist."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(2600, synthetic.uniform_lengths(1, 120), np.float32, seed=31)
    X = arr(pts, off)
    Y = arr(*synthetic.gaussian(700, synthetic.uniform_lengths(1, 90), np.float32, seed=32))
    one = (sb.pdist(X).data.copy(), sb.l2_kernel(X).data.copy(), sb.cdist(X, Y).copy())
    try:
        sb.set_tuning(band_bytes=256 << 10)
        many = (sb.pdist(X).data.copy(), sb.l2_kernel(X).data.copy(), sb.cdist(X, Y).copy())
    finally:
        sb.set_tuning()
    for a, b in zip(one, many):
        np.testing.assert_array_equal(a, b)


def test_device_bands_of_whole_windows_use_the_length_order():
    """Device-entry bands of whole 1024-PCF windows run in the length order
    and give the bits of the whole call, each band into its own buffer."""
    import torch
    from stablebear_gb300 import _native as nat, synthetic
    pts, off = synthetic.gaussian(2600, synthetic.uniform_lengths(1, 100), np.float32, seed=33)
    n = len(off) - 1
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    lmax = int(np.diff(off.astype(np.int64)).max())
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    total = n * (n - 1) // 2
    whole = torch.empty(total, device="cuda")
    nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                            do.data_ptr(), n, None, None, 0, None, None, lmax, whole.data_ptr(), 0, 0,
                                            0, st))
    parts = []
    for rb, re in ((0, 1024), (1024, 2048), (2048, n)):
        base = rb * (rb - 1) // 2
        buf = torch.full((re * (re - 1) // 2 - base,), float("nan"), device="cuda")
        nat.check(nat.lib().sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                                do.data_ptr(), n, None, None, 0, None, None, lmax, buf.data_ptr(),
                                                base, rb, re, st))
        parts.append(buf)
    torch.cuda.synchronize()
    assert torch.equal(torch.cat(parts), whole)


def test_infinite_values_at_shared_breakpoints():
    """A value of inf right after a breakpoint both PCFs share: the
    reference advances both sides there and returns inf; no zero-width
    rectangle may turn it into inf * 0 = NaN."""
    import stablebear_gb300 as sb
    from oracle import oracle as orc
    for dt in (np.float32, np.float64):
        pcfs = [[[0, 0], [1, np.inf], [2, 0]], [[0, 0], [1, 5], [3, 0]], [[0, 1], [1, 2], [2, 0]],
                [[0, -np.inf], [1, 0]], [[0, 0], [1, 0]]]
        pts = np.concatenate([np.array(p, dt) for p in pcfs])
        off = np.zeros(len(pcfs) + 1, np.uint64)
        np.cumsum([len(p) for p in pcfs], out=off[1:])
        X = arr(pts, off)
        for got, op, mode in ((sb.pdist(X).data, orc.OP_L1, orc.MODE_PDIST),
                              (sb.l2_kernel(X).data, orc.OP_L2, orc.MODE_KERNEL)):
            want = orc.evaluate(pts, off, op=op, mode=mode)
            np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
            np.testing.assert_array_equal(got[np.isinf(want)], want[np.isinf(want)])
