"""The time-windowed kernel (variant 6, the automatic choice for PCFs too long
for the plain shared-memory layout) against the oracle.

Window caps down to one element force every pair across many windows, with
window ends on duplicate and shared breakpoints.  Tolerances as in
test_gpu_parity.py: float32 relative 1e-5 (Lp with general p 1e-4), float64
1e-12 (Lp 1e-10); the L2 kernel against max(|ref|, 1).

A window's compensated sum is handed to the next window as one rounded
value, so with caps of a few elements (a window per rectangle or two) the
float32 sum is close to a naive one, whose error alone reaches 1e-5 here:
those cases compare with the double-double truth oracle at 3e-5, still far
below the share of a single rectangle (about 1e-2 of a sum).
"""
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
    yield
    sb.set_tuning()
    sb.set_window_cap(0)


@pytest.fixture
def windowed():
    import stablebear_gb300 as sb

    def use(cap, **kw):
        sb.set_tuning(variant=6, **kw)
        sb.set_window_cap(cap)

    yield use
    sb.set_tuning()
    sb.set_window_cap(0)


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


def check_all_ops(pts, off, tag, ypts=None, yoff=None, truth=False):
    """Every op and mode against the oracle: the reference's naive sum, or
    with truth=True the double-double one (float32 bound 3e-5 then)."""
    import stablebear_gb300 as sb
    from oracle import oracle as orc
    X = arr(pts, off)
    tol = dict(TOL, f32=3e-5) if truth else TOL
    tol_lp = dict(TOL_LP, f32=max(3e-5, TOL_LP["f32"])) if truth else TOL_LP
    assert rel_err(sb.pdist(X).data, orc.evaluate(pts, off, truth=truth)) <= tol[tag]
    assert rel_err(sb.pdist(X, p=2).data, orc.evaluate(pts, off, op=orc.OP_LP, p=2.0, truth=truth)) <= tol[tag]
    assert rel_err(sb.pdist(X, p=2.5).data, orc.evaluate(pts, off, op=orc.OP_LP, p=2.5, truth=truth)) <= tol_lp[tag]
    assert rel_err(sb.l2_kernel(X).data, orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL, truth=truth),
                   floor=1.0) <= tol[tag]
    if ypts is not None:
        got = sb.cdist(X, arr(ypts, yoff))
        want = orc.evaluate(pts, off, mode=orc.MODE_CROSS, col_points=ypts, col_offsets=yoff, truth=truth)
        assert rel_err(got.reshape(-1), want) <= tol[tag]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("cap", [1, 3, 8, 40])
def test_windows_match_oracle(windowed, dt, cap):
    from stablebear_gb300 import synthetic
    tag = "f32" if dt == np.float32 else "f64"
    pts, off = synthetic.gaussian(75, synthetic.uniform_lengths(1, 120), dt, seed=cap)
    ypts, yoff = synthetic.gaussian(37, synthetic.uniform_lengths(1, 90), dt, seed=cap + 500)
    windowed(cap)
    check_all_ops(pts, off, tag, ypts, yoff, truth=cap < 16)


def _with_duplicates(n, seed, dt):
    """PCFs on a shared coarse time grid (ties across PCFs) with repeated
    times (zero-width segments), including at t = 0."""
    rng = np.random.default_rng(seed)
    grid = (np.cumsum(rng.integers(0, 3, size=400)) * 0.125).astype(dt)  # steps of 0, 1/8 or 1/4
    pts, off = [], [0]
    for _ in range(n):
        L = int(rng.integers(1, 150))
        t = np.sort(rng.choice(grid, size=L, replace=True)).astype(dt)
        t[0] = 0
        v = rng.normal(size=L).astype(dt)
        v[-1] = 0  # a finite integral (a non-zero tail runs to the largest float)
        pts.append(np.stack([t, v], axis=1))
        off.append(off[-1] + L)
    return np.concatenate(pts).astype(dt), np.array(off, dtype=np.uint64)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("cap", [2, 5, 16])
def test_window_ends_on_duplicate_and_shared_breakpoints(windowed, dt, cap):
    tag = "f32" if dt == np.float32 else "f64"
    pts, off = _with_duplicates(64, seed=cap, dt=dt)
    ypts, yoff = _with_duplicates(33, seed=cap + 99, dt=dt)
    windowed(cap)
    check_all_ops(pts, off, tag, ypts, yoff, truth=True)


def test_one_window_equals_the_plain_kernel_bitwise(windowed):
    """PCFs that fit one window take the plain kernel's steps exactly."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(300, synthetic.uniform_lengths(2, 200), np.float32, seed=7)
    X = arr(pts, off)
    try:
        sb.set_tuning(variant=5)
        plain = sb.pdist(X).data.copy()
        kern = sb.l2_kernel(X).data.copy()
    finally:
        sb.set_tuning()
    windowed(256)
    np.testing.assert_array_equal(sb.pdist(X).data, plain)
    np.testing.assert_array_equal(sb.l2_kernel(X).data, kern)


def test_many_windows_with_small_items_and_few_warps(windowed):
    """One 32-row item per column group, 4 warps: the window walk with rows
    shared out dynamically, rows outside the triangle and ragged last groups."""
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(101, synthetic.uniform_lengths(1, 300), np.float32, seed=11)
    windowed(24, warps=4, row_chunk=1)
    check_all_ops(pts, off, "f32", truth=True)


def test_long_pcfs_take_the_windowed_path_by_default(windowed):
    """Lengths up to 7000: too long for the plain layout; the automatic plan
    gives the same bits as the windowed variant at its automatic cap."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    from oracle import oracle as orc
    lens = np.array([3, 7000, 60, 1, 4096, 900, 12, 2500] * 5)
    pts, off = synthetic.gaussian(len(lens), lens, np.float32, seed=4)
    X = arr(pts, off)
    auto = sb.pdist(X).data.copy()
    windowed(0)
    np.testing.assert_array_equal(sb.pdist(X).data, auto)
    truth = orc.evaluate(pts, off, truth=True)
    assert rel_err(auto, truth) <= 1e-5


def test_infinite_values_across_windows(windowed):
    """An infinite value over a stretch that window ends cut gives inf, never
    NaN (no zero-width rectangle multiplies it)."""
    import stablebear_gb300 as sb
    from oracle import oracle as orc
    t = np.arange(40, dtype=np.float32)
    v1 = np.zeros(40, np.float32)
    v1[10:20] = np.inf
    v2 = np.ones(40, np.float32)
    t2 = t + np.float32(0.5)
    t2[0] = 0
    pts = np.concatenate([np.stack([t, v1], 1), np.stack([t, v2], 1), np.stack([t2, v2], 1)])
    off = np.array([0, 40, 80, 120], dtype=np.uint64)
    windowed(3)
    got = sb.pdist(arr(pts, off)).data
    want = orc.evaluate(pts, off)
    assert not np.isnan(got).any()
    assert rel_err(got, want) <= 1e-5


def test_cap_too_large_for_shared_memory_is_an_error(windowed):
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(40, synthetic.uniform_lengths(1, 50), np.float32, seed=1)
    windowed(100000)
    with pytest.raises(Exception, match="shared memory"):
        sb.pdist(arr(pts, off))
