"""The float32 measurement variants of the pair kernel (sbg_set_tuning
variant 7: replicated row with one unified shared-memory load per step;
variant 8: merge path, one pair per warp) against the default kernel and the
oracle.

Variant 7 walks the same rectangles in the same Kahan blocks as the default
kernel (variant 5), so for finite values its results are equal bit for bit.
Variant 8 sums each lane's share of a pair and adds the 32 partial sums by
a shuffle tree: it is held to the contract's float32 bound against the
double-double truth (1e-5 relative; general p 1e-4; the L2 kernel against
max(|truth|, 1)).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def native():
    from stablebear_gb300 import build
    build.build()
    import stablebear_gb300 as sb
    yield
    sb.set_tuning()


def _with_variant(v, fn):
    import stablebear_gb300 as sb
    sb.set_tuning(variant=v)
    try:
        return fn()
    finally:
        sb.set_tuning()


def rel(got, want, floor=1e-30):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), floor)))


def test_variant7_equals_the_default_kernel_bit_for_bit():
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(700, synthetic.uniform_lengths(1, 60), np.float32, seed=41)
    X = sb.PcfArray.from_csr(pts, off)
    ypts, yoff = synthetic.gaussian(90, synthetic.uniform_lengths(1, 60), np.float32, seed=42)
    Y = sb.PcfArray.from_csr(ypts, yoff)
    cases = {"pdist L1": lambda: sb.pdist(X).data, "pdist L2": lambda: sb.pdist(X, p=2).data,
             "pdist L1.5": lambda: sb.pdist(X, p=1.5).data, "l2 kernel": lambda: sb.l2_kernel(X).data,
             "cdist L1": lambda: sb.cdist(X, Y)}
    for name, fn in cases.items():
        want = _with_variant(5, fn)
        got = _with_variant(7, fn)
        np.testing.assert_array_equal(got, want, err_msg=name)


def test_variant7_with_ties_and_zero_width_segments():
    """Shared and repeated breakpoints (ties between the two PCFs and within
    one): the tie rules of the walk, so still equal to the default."""
    import stablebear_gb300 as sb
    rng = np.random.default_rng(43)
    pcfs = []
    for _ in range(150):
        L = int(rng.integers(1, 40))
        t = np.concatenate([[0.0], np.cumsum(np.round(rng.exponential(1.0, L - 1) * 2) / 2)])
        v = rng.normal(size=L)
        v[-1] = 0.0
        pcfs.append(np.stack([t, v], 1))
    pts = np.concatenate(pcfs).astype(np.float32)
    off = np.zeros(len(pcfs) + 1, np.uint64)
    np.cumsum([len(p) for p in pcfs], out=off[1:])
    X = sb.PcfArray.from_csr(pts, off)
    for p in (1, 2):
        np.testing.assert_array_equal(_with_variant(7, lambda: sb.pdist(X, p=p).data),
                                      _with_variant(5, lambda: sb.pdist(X, p=p).data))


@pytest.mark.parametrize("lengths", [(1, 60), (100, 400)])
def test_variant8_against_truth(lengths):
    import stablebear_gb300 as sb
    from oracle import oracle as orc
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(400, synthetic.uniform_lengths(*lengths), np.float32, seed=44)
    X = sb.PcfArray.from_csr(pts, off)
    assert rel(_with_variant(8, lambda: sb.pdist(X).data), orc.evaluate(pts, off, truth=True)) <= 1e-5
    assert rel(_with_variant(8, lambda: sb.pdist(X, p=2).data),
               orc.evaluate(pts, off, op=orc.OP_LP, p=2.0, truth=True)) <= 1e-5
    assert rel(_with_variant(8, lambda: sb.pdist(X, p=1.5).data),
               orc.evaluate(pts, off, op=orc.OP_LP, p=1.5, truth=True)) <= 1e-4
    assert rel(_with_variant(8, lambda: sb.l2_kernel(X).data),
               orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL, truth=True), floor=1.0) <= 1e-5
    ypts, yoff = synthetic.gaussian(50, synthetic.uniform_lengths(*lengths), np.float32, seed=45)
    got = _with_variant(8, lambda: sb.cdist(X, sb.PcfArray.from_csr(ypts, yoff)).reshape(-1))
    want = orc.evaluate(pts, off, mode=orc.MODE_CROSS, col_points=ypts, col_offsets=yoff, truth=True)
    assert rel(got, want) <= 1e-5


def test_variants_reject_what_they_cannot_run():
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    p64, o64 = synthetic.gaussian(50, synthetic.uniform_lengths(1, 30), np.float64, seed=46)
    for v in (7, 8):
        with pytest.raises(ValueError, match="float32 only"):
            _with_variant(v, lambda: sb.pdist(sb.PcfArray.from_csr(p64, o64)))
    # a row replicated 16 times does not fit shared memory for long PCFs
    pl, ol = synthetic.gaussian(64, synthetic.uniform_lengths(2000, 2500), np.float32, seed=47)
    with pytest.raises(ValueError, match="do not fit"):
        _with_variant(7, lambda: sb.pdist(sb.PcfArray.from_csr(pl, ol)))
