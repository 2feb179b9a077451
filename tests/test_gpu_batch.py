"""Batched launches (many independent problems, one persistent kernel)
against the oracle and against the single-problem path.

Tolerances as in test_gpu_parity.py: float32 1e-5 relative (L2 kernel
against max(|ref|, 1)), float64 1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def native():
    from stablebear_gb300 import build
    build.build()


def rel_err(got, want, floor=1e-30):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    d = np.abs(got - want) / np.maximum(np.abs(want), floor)
    return float(d.max()) if d.size else 0.0


def _problems(seed, count, dt=np.float32, nmax=300, lmax=400):
    from stablebear_gb300 import synthetic
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(rng.integers(0, nmax))
        out.append(synthetic.betti(n, synthetic.uniform_lengths(1, lmax), dt, seed=seed * 1000 + k) if n else
                   (np.zeros((0, 2), dt), np.zeros(1, np.uint64)))
    return out


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("op", ["l1", "lp", "l2_kernel"])
def test_batch_matches_oracle(dt, op):
    from stablebear_gb300.batch import PairwiseBatch
    from oracle import oracle as orc
    probs = _problems(3, 17, dt)
    p = 2.0 if op == "lp" else 1.0
    b = PairwiseBatch(probs, op=op, p=p, graph=False)
    outs = [o.cpu().numpy() for o in b.run()]
    tol = 1e-5 if dt == np.float32 else 1e-12
    for (pts, off), got in zip(probs, outs):
        n = len(off) - 1
        if n == 0:
            assert got.size == 0
            continue
        if op == "l2_kernel":
            want = orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL)
            assert rel_err(got, want, floor=1.0) <= tol
        else:
            want = orc.evaluate(pts, off, op=orc.OP_L1 if op == "l1" else orc.OP_LP, p=p)
            assert rel_err(got, want) <= tol
    b.close()


def test_batch_graph_replay_and_autotune_are_stable():
    from stablebear_gb300.batch import PairwiseBatch
    import torch
    probs = _problems(5, 40)
    b = PairwiseBatch(probs, op="l1", graph=True)
    first = [o.clone() for o in b.run()]
    for o in b.outputs:
        o.fill_(float("nan"))
    second = b.run()
    for a, c in zip(first, second):
        assert torch.equal(a, c)
    ms = b.autotune()
    assert ms > 0
    third = b.run()
    torch.cuda.synchronize()
    for a, c in zip(first, third):
        assert torch.equal(a, c)
    info = b.info()
    assert info["pairs"] == sum((len(off) - 1) * (len(off) - 2) // 2 for _, off in probs if len(off) > 1)
    b.close()


@pytest.mark.parametrize("variant", [0, 4])
def test_batch_long_pcfs(variant):
    """PCFs far longer than a shared-memory slice: the time-windowed kernel
    (the default) walks them window by window; the hybrid kernel (variant 4)
    reads column groups too long for its block from global memory."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    from stablebear_gb300.batch import PairwiseBatch
    from oracle import oracle as orc
    lens = np.array([20, 6000, 40, 3, 7000, 15] * 7)
    pts, off = synthetic.gaussian(len(lens), lens, np.float32, seed=2)
    small = synthetic.plain_l1(90, seed=3)
    sb.set_tuning(variant=variant)
    try:
        b = PairwiseBatch([(pts, off), small], op="l1", graph=False)
    finally:
        sb.set_tuning()
    got = [o.cpu().numpy() for o in b.run()]
    truth = orc.evaluate(pts, off, truth=True)
    assert rel_err(got[0], truth) <= 1e-5
    assert rel_err(got[1], orc.evaluate(*small)) <= 1e-5
    b.close()


def test_batch_windowed_with_small_windows():
    """Window caps of 5 elements in a batch of uneven problems (every pair
    crosses many windows), against the double-double oracle: with windows
    this small the float32 sum is close to a naive one (bound 3e-5)."""
    import stablebear_gb300 as sb
    from stablebear_gb300.batch import PairwiseBatch
    from oracle import oracle as orc
    probs = _problems(8, 9, nmax=120, lmax=200)
    sb.set_window_cap(5)
    try:
        b = PairwiseBatch(probs, op="l1", graph=False)
    finally:
        sb.set_window_cap(0)
    outs = [o.cpu().numpy() for o in b.run()]
    for (pts, off), got in zip(probs, outs):
        if len(off) > 2:
            assert rel_err(got, orc.evaluate(pts, off, truth=True)) <= 3e-5
    b.close()


def test_pdist_and_kernel_batched_api():
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    from stablebear_gb300.batch import l2_kernel_batched, pdist_batched
    arrays = [sb.PcfArray.from_csr(*synthetic.plain_l1(n, seed=n)) for n in (5, 64, 200)]
    Ds = pdist_batched(arrays)
    Ks = l2_kernel_batched(arrays)
    for X, D, K in zip(arrays, Ds, Ks):
        assert isinstance(D, sb.DistanceMatrix) and D.size == X.shape[0]
        assert rel_err(D.data, sb.pdist(X).data) <= 1e-5
        assert rel_err(K.data, sb.l2_kernel(X).data, floor=1.0) <= 1e-5


@pytest.mark.parametrize("variant", [6, 4])
def test_batch_f64_windowed_and_hybrid(variant):
    """Double-precision batches run the hybrid kernel by default; the
    time-windowed one on request, with a window cap small enough that long
    PCFs take several windows, against the oracle (float64 1e-12)."""
    import stablebear_gb300 as sb
    from stablebear_gb300.batch import PairwiseBatch
    from oracle import oracle as orc
    probs = _problems(11, 7, dt=np.float64, nmax=150, lmax=700)
    sb.set_tuning(variant=variant)
    sb.set_window_cap(64 if variant == 6 else 0)
    try:
        b = PairwiseBatch(probs, op="l2_kernel", graph=False)
    finally:
        sb.set_tuning()
        sb.set_window_cap(0)
    outs = [o.cpu().numpy() for o in b.run()]
    for (pts, off), got in zip(probs, outs):
        if len(off) > 1:
            want = orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL, truth=True)
            assert rel_err(got, want, floor=1.0) <= 1e-12
    b.close()


def test_batch_autotune_with_window_cap():
    """With tune_window the autotune may move the window cap (the split of
    shared memory between the column block and the row buffers): the
    results stay within the float32 bound, and without the flag the cap the
    batch was made with is kept."""
    from stablebear_gb300.batch import PairwiseBatch
    from oracle import oracle as orc
    probs = _problems(11, 24, nmax=400, lmax=900)
    fixed = PairwiseBatch(probs, op="l1", graph=False)
    cap0 = fixed.info()["column_elements"]
    fixed.autotune()
    assert fixed.info()["column_elements"] == cap0
    fixed.close()
    b = PairwiseBatch(probs, op="l1", graph=True, tune_window=True)
    assert b.info()["column_elements"] == cap0
    assert b.autotune() > 0
    cap = b.info()["column_elements"]
    assert cap >= 8
    outs = [o.cpu().numpy() for o in b.run()]
    for (pts, off), got in zip(probs, outs):
        if len(off) > 2:
            assert rel_err(got, orc.evaluate(pts, off)) <= 1e-5
    b.close()
