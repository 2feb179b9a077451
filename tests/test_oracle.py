"""The oracle pinned against the reference: its own tests' known answers and
the golden fixtures produced by the reference's code (CPU only)."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests.conftest import GOLDEN

F32 = np.float32
F64 = np.float64


def P(rows, dt=F64):
    return np.array(rows, dtype=dt)


def csr(*pcfs):
    pts = np.concatenate(pcfs)
    off = np.zeros(len(pcfs) + 1, dtype=np.uint64)
    np.cumsum([len(p) for p in pcfs], out=off[1:])
    return pts, off


@pytest.mark.parametrize("dt", [F32, F64])
def test_known_answers_from_reference_tests(dt):
    # test/python/test_pdist.py:57-70 (2*5 + 3*5 = 25)
    assert orc.pair(P([[0, 10], [2, 5], [3, 0]], dt), P([[0, 5], [6, 0]], dt)) == 25.0
    # test/python/test_pdist.py:90-104 (L3 of 4 vs 1 on [0,1) = 3)
    assert orc.pair(P([[0, 4], [1, 0]], dt), P([[0, 1], [1, 0]], dt), op=orc.OP_LP, p=3.0) == pytest.approx(3.0)
    # test/test_l1_dist.cu:31-41 (= 3)
    assert orc.pair(P([[0, 3], [1, 0]], dt), P([[0, 1], [2, 0]], dt)) == 3.0
    # test/test_l1_dist.cu:98-107: default PCFs [(0,0)] are at distance 0
    assert orc.pair(P([[0, 0]], dt), P([[0, 0]], dt)) == 0.0
    # test/python/test_kernel.py:31-62: <f,f> = 18, Gram 48 / 24 / 12
    assert orc.pair(P([[0, 3], [2, 0]], dt), P([[0, 3], [2, 0]], dt), op=orc.OP_L2) == 18.0
    f, g = P([[0, 4], [3, 0]], dt), P([[0, 2], [3, 0]], dt)
    assert orc.pair(f, f, op=orc.OP_L2) == 48.0
    assert orc.pair(f, g, op=orc.OP_L2) == 24.0
    assert orc.pair(g, g, op=orc.OP_L2) == 12.0


LP_CASES = [  # test/python/test_lp_distance.py:15-137 (closed forms)
    ([[0, 5], [1, 0]], [[0, 5], [1, 0]], 1, 0.0),
    ([[0, 0]], [[0, 0]], 1, 0.0),
    ([[0, 5], [1, 0]], [[0, 0]], 1, 5.0),
    ([[0, 3], [1, 0]], [[0, 0], [1, 0]], 2, 3.0),
    ([[0, 4], [1, 0]], [[0, 1], [1, 0]], 3, 3.0),
    ([[0, 3], [1, 1], [2, 0]], [[0, 1], [1, 1], [2, 0]], 1, 2.0),
    ([[0, 2], [1, 0]], [[0, 1], [2, 0]], 1, 2.0),
    ([[0, 4], [1, 2], [3, 0]], [[0, 1], [2, 3], [4, 0]], 1, 8.0),
    ([[0, 6], [3, 0]], [[0, 2], [1, 4], [2, 0]], 1, 12.0),
    ([[0, 5], [0.5, 0]], [[0, 3], [1.5, 0]], 1, 4.0),
    ([[float(i), float(i)] for i in range(5)] + [[5.0, 0.0]], [[0, 0]], 1, 10.0),
    ([[0, -3], [1, 0]], [[0, 2], [1, 0]], 1, 5.0),
    ([[0, -1], [1, 0]], [[0, -4], [1, 0]], 1, 3.0),
]


@pytest.mark.parametrize("dt", [F32, F64])
@pytest.mark.parametrize("f,g,p,want", LP_CASES)
def test_lp_distance_closed_forms(dt, f, g, p, want):
    op = orc.OP_L1 if p == 1 else orc.OP_LP
    got = orc.pair(P(f, dt), P(g, dt), op=op, p=p)
    assert got == pytest.approx(want, rel=1e-6, abs=1e-6)
    assert orc.pair(P(f, dt), P(g, dt), op=op, p=p, truth=True) == pytest.approx(want, rel=1e-12, abs=1e-12)


def test_large_p_limit():
    # test/python/test_lp_distance.py:73-78 (p = 50 -> 2, abs 1e-2)
    assert orc.pair(P([[0, 2], [1, 0]]), P([[0, 0], [1, 0]]), op=orc.OP_LP, p=50) == pytest.approx(2.0, abs=1e-2)


def test_last_rectangle_runs_to_max():
    # a non-zero tail contributes (max - t_last) * op (time_point.hpp:10-14)
    got = orc.pair(P([[0, 1]], F32), P([[0, 0]], F32))
    assert got == float(np.finfo(F32).max)
    got64 = orc.pair(P([[0, 1]], F64), P([[0, 0]], F64))
    assert got64 == float(np.finfo(F64).max)


def test_rectangles_match_reference_unit_test():
    # test/test_iterate_rectangles.cpp:28-41, through the golden fixture made
    # by the reference's own iterate_rectangles
    import os
    from tests.conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "reference_rectangles.npz"))
    full = d["full"]
    big = np.finfo(F64).max
    want = np.array([[0, 1, 3, 2], [1, 3, 2, 2], [3, 4, 2, 4], [4, 5, 5, 2], [5, 6, 5, 1], [6, 8, 0, 1],
                     [8, big, 0, 3]], dtype=F64)
    np.testing.assert_array_equal(full, want)
    np.testing.assert_array_equal(d["end_early"][-1], [4, 4.5, 5, 2])
    assert len(d["start_late"]) == 6


def test_oracle_matches_golden_bitwise(golden_pairwise, tag):
    """The C restatement reproduces the reference's outputs bit for bit
    (same operation order; both built with -ffp-contract=off)."""
    g = golden_pairwise
    for case in ("ragged", "tails", "ties"):
        name = f"{case}_{tag}"
        pts, off = g[f"{name}__points"], g[f"{name}__offsets"]
        ypts, yoff = g[f"cols_{tag}__points"], g[f"cols_{tag}__offsets"]
        np.testing.assert_array_equal(orc.evaluate(pts, off, op=orc.OP_L1, mode=orc.MODE_PDIST, threads=2),
                                      g[f"{name}__pdist_l1"])
        np.testing.assert_array_equal(orc.evaluate(pts, off, op=orc.OP_LP, p=2.0, mode=orc.MODE_PDIST),
                                      g[f"{name}__pdist_l2"])
        np.testing.assert_array_equal(orc.evaluate(pts, off, op=orc.OP_LP, p=3.0, mode=orc.MODE_PDIST),
                                      g[f"{name}__pdist_l3"])
        np.testing.assert_array_equal(orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL),
                                      g[f"{name}__kernel"])
        np.testing.assert_array_equal(orc.evaluate(pts, off, op=orc.OP_L1, mode=orc.MODE_CROSS, col_points=ypts,
                                                   col_offsets=yoff), g[f"{name}__cdist_l1"])
        np.testing.assert_array_equal(orc.evaluate(pts, off, op=orc.OP_LP, p=1.5, mode=orc.MODE_CROSS,
                                                   col_points=ypts, col_offsets=yoff), g[f"{name}__cdist_l15"])


def test_truth_oracle_close_to_reference(golden_pairwise, tag):
    g = golden_pairwise
    name = f"ragged_{tag}"
    ref = g[f"{name}__pdist_l1"].astype(np.float64)
    truth = g[f"{name}__pdist_l1_truth"]
    tol = 1e-5 if tag == "f32" else 1e-12
    assert np.max(np.abs(ref - truth) / np.maximum(np.abs(truth), 1e-300)) < tol


def test_rows_subset_matches_full():
    from stablebear_gb300 import synthetic
    pts, off = synthetic.plain_l1(120, seed=3)
    full = orc.evaluate(pts, off)
    rows = np.array([0, 1, 7, 64, 119], dtype=np.uint64)
    vals, starts = orc.evaluate_rows(pts, off, rows)
    for k, i in enumerate(rows):
        i = int(i)
        np.testing.assert_array_equal(vals[starts[k]:starts[k + 1]], full[i * (i - 1) // 2: i * (i - 1) // 2 + i])


@pytest.mark.parametrize("mode", [orc.MODE_PDIST, orc.MODE_KERNEL])
def test_chunked_rows_match_whole_rows(mode):
    """Threads taking pieces of rows (the CPU-baseline schedule) compute the
    same bits as threads taking whole rows, including rows with no pairs."""
    from stablebear_gb300 import synthetic
    pts, off = synthetic.plain_l1(150, seed=5)
    rows = np.array([0, 1, 2, 149, 63, 64, 65, 100, 0], dtype=np.uint64)
    op = orc.OP_L2 if mode == orc.MODE_KERNEL else orc.OP_L1
    whole, s0 = orc.evaluate_rows(pts, off, rows, op=op, mode=mode, threads=3)
    for chunk in (1, 7, 64, 1000):
        part, s1 = orc.evaluate_rows(pts, off, rows, op=op, mode=mode, threads=5, chunk=chunk)
        np.testing.assert_array_equal(s0, s1)
        np.testing.assert_array_equal(part, whole)


def test_timed_builds_match_the_checker():
    """The -O3 host-CPU build without contraction is bit for bit the checker;
    with FMA contraction it stays within the f32 parity bound."""
    from stablebear_gb300 import synthetic
    pts, off = synthetic.plain_l1(200, seed=6)
    rows = np.arange(1, 200, 9, dtype=np.uint64)
    want, _ = orc.evaluate_rows(pts, off, rows)
    off_, _ = orc.evaluate_rows(pts, off, rows, build="o3_off", chunk=16)
    fast, _ = orc.evaluate_rows(pts, off, rows, build="o3_fast", chunk=16)
    np.testing.assert_array_equal(off_, want)
    assert np.max(np.abs(fast - want) / np.maximum(np.abs(want), 1e-30)) < 1e-5


def test_segment_formula_matches_count():
    from stablebear_gb300 import synthetic
    pts, off = synthetic.plain_l1(200, seed=4)
    assert synthetic.segment_count(off, pts, 1) == orc.count_segments(pts, off, orc.MODE_PDIST)
    assert synthetic.segment_count(off, pts, 2) == orc.count_segments(pts, off, orc.MODE_KERNEL)


@pytest.mark.skipif(orc.ref_lib() is None, reason="reference tree absent")
@pytest.mark.parametrize("dt", [F32, F64])
def test_oracle_matches_live_reference(dt):
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(90, synthetic.uniform_lengths(1, 60), dt, seed=21)
    for op, p, mode in ((orc.OP_L1, 1.0, orc.MODE_PDIST), (orc.OP_LP, 2.5, orc.MODE_PDIST),
                        (orc.OP_L2, 1.0, orc.MODE_KERNEL), (orc.OP_L1, 1.0, orc.MODE_KERNEL)):
        if True:
            np.testing.assert_array_equal(orc.evaluate(pts, off, op=op, p=p, mode=mode),
                                          orc.ref_evaluate(pts, off, op=op, p=p, mode=mode))


def oracle_gradient(pts, off, op, mode, w, dist=None):
    import ctypes
    lib = orc._load()
    lib.sbo_gradient_f64.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                              ctypes.c_double]
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    off = np.ascontiguousarray(off, dtype=np.uint64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    g = np.zeros_like(pts)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    d = np.ascontiguousarray(dist, dtype=np.float64) if dist is not None else None
    lib.sbo_gradient_f64(P(pts), P(off), len(off) - 1, op, mode, P(w), P(d) if d is not None else None, P(g),
                         float(np.finfo(np.float64).max))
    return g


@pytest.mark.parametrize("op,mode,p", [(orc.OP_L2, orc.MODE_KERNEL, 1.0), (orc.OP_LP, orc.MODE_PDIST, 2.0),
                                       (orc.OP_L1, orc.MODE_PDIST, 1.0)])
def test_oracle_gradient_matches_central_differences(op, mode, p):
    """The FP64 reference gradient against FP64 central finite differences
    of the double-double forward.  Excluded: t_0 (fixed at 0) and each PCF's
    last value, whose rectangle runs to numeric_limits<double>::max()."""
    from stablebear_gb300 import synthetic
    pts, off = synthetic.gaussian(8, synthetic.uniform_lengths(3, 9), np.float64, seed=3)
    M = orc.evaluate(pts, off, op=op, p=p, mode=mode, truth=True)
    w = np.random.default_rng(1).standard_normal(M.size)
    g = oracle_gradient(pts, off, op, mode, w, M if op == orc.OP_LP else None)
    loss = lambda q: float(w @ orc.evaluate(q, off, op=op, p=p, mode=mode, truth=True))
    starts = set(int(x) for x in off[:-1])
    lasts = set(int(x) - 1 for x in off[1:])
    eps = 1e-6
    checked = 0
    for k in range(len(pts)):
        for c in (0, 1):
            if (c == 0 and k in starts) or (c == 1 and k in lasts):
                continue
            q = pts.copy()
            q[k, c] += eps
            a = loss(q)
            q[k, c] -= 2 * eps
            b = loss(q)
            fd = (a - b) / (2 * eps)
            assert abs(fd - g[k, c]) <= 1e-6 * max(1.0, abs(fd)), (k, c, fd, g[k, c])
            checked += 1
    assert checked > 40


# ---- single-PCF Lp norms ------------------------------------------------------

@pytest.mark.parametrize("tag", ["f32", "f64"])
@pytest.mark.parametrize("p", [1.0, 1.5, 2.0, 3.0])
def test_norm_oracle_matches_reference_bitwise(tag, p):
    d = np.load(os.path.join(GOLDEN, "reference_norms.npz"))
    got = orc.lp_norm(d[f"{tag}_points"], d[f"{tag}_offsets"], p)
    np.testing.assert_array_equal(got, d[f"{tag}_p{p}"])


def test_norm_known_answers():
    """The reference's norm test cases (test/python/test_norms.py,
    test_norms_extended.py), restated."""
    pcfs = [[[0, 10], [2, 5], [4, 0]], [[0, 5], [3, 6], [5, 5], [8, 0]], [[0, 12], [3, 0]],
            [[0, 50], [0.5, 0]], [[0, 0]], [[0, 2], [3, 0]]]
    pts = np.concatenate([np.array(x, np.float64) for x in pcfs])
    off = np.zeros(len(pcfs) + 1, np.uint64)
    np.cumsum([len(x) for x in pcfs], out=off[1:])
    np.testing.assert_allclose(orc.lp_norm(pts, off, 1.0), [30, 42, 36, 25, 0, 6], rtol=1e-12)
    one = lambda x, p: orc.lp_norm(np.array(x, np.float64), np.array([0, len(x)], np.uint64), p)[0]
    assert one([[0, 3], [4, 0]], 2.0) == pytest.approx(6.0)
    assert one([[0, 1], [1, 2], [2, 0]], 2.0) == pytest.approx(np.sqrt(5.0))
    assert one([[0, -2], [1, 0]], 3.0) == pytest.approx(2.0)
    assert one([[0, 0]], 2.0) == 0.0
    # repeated t = 0: the walk starts at the last breakpoint with t <= 0
    assert one([[0, 7], [0, 1], [2, 0]], 1.0) == 2.0


# ---- barcodes to PCFs ------------------------------------------------------------

def _summary(bars, kind, dt=np.float64):
    b = np.array(bars, dt).reshape(-1, 2)
    pts, off = orc.barcodes_to_pcfs(b, np.array([0, len(b)], np.uint64), kind)
    return pts.tolist()


def test_stable_rank_known_answers():
    """test/python/persistence/test_stable_rank.py and
    test/test_barcode_and_stable_rank.cpp, restated."""
    for dt in (np.float32, np.float64):
        assert _summary([], 0, dt) == [[0, 0]]
        assert _summary([[0, 1], [0, 2], [0, 3]], 0, dt) == [[0, 3], [1, 2], [2, 1], [3, 0]]
        assert _summary([[0, 1], [0, 3], [0, 2], [0, 2], [1, 3]], 0, dt) == [[0, 5], [1, 4], [2, 1], [3, 0]]
        assert _summary([[0, 1], [0, 3], [0, 2], [0, np.inf], [1, 3]], 0, dt) == [[0, 5], [1, 4], [2, 2], [3, 1]]
        assert _summary([[0, 1], [0, 2]], 0, dt) == [[0, 2], [1, 1], [2, 0]]
        # a death at the dtype's maximum is infinite too
        assert _summary([[0, np.finfo(dt).max], [0, 1]], 0, dt) == [[0, 2], [1, 1]]
        # all bars infinite: only the first point
        assert _summary([[0, np.inf], [1, np.inf]], 0, dt) == [[0, 2]]


def test_betti_curve_known_answers():
    """test/python/persistence/test_betti_curve.py, restated."""
    for dt in (np.float32, np.float64):
        assert _summary([], 1, dt) == [[0, 0]]
        assert _summary([[0, 2]], 1, dt) == [[0, 1], [2, 0]]
        assert _summary([[1, 3]], 1, dt) == [[0, 0], [1, 1], [3, 0]]
        assert _summary([[0, 2], [1, 3], [0.5, 1.5]], 1, dt) == [[0, 1], [0.5, 2], [1, 3], [1.5, 2], [2, 1], [3, 0]]
        assert _summary([[0, 1], [0, 2], [0, 3]], 1, dt) == [[0, 3], [1, 2], [2, 1], [3, 0]]
        assert _summary([[0, np.inf], [1, 2]], 1, dt) == [[0, 1], [1, 2], [2, 1]]


def test_rectangle_walk_restatement_matches_reference_cases():
    """The oracle's rectangle walk against the reference's own walk, recorded
    on random pairs with repeated and shared breakpoints and assorted bounds
    (tests/golden/make_golden.py rectangle_cases)."""
    d = np.load(os.path.join(GOLDEN, "reference_rectangle_cases.npz"))
    k = 0
    while f"f_{k}" in d.files:
        a, b = d[f"ab_{k}"]
        got = orc.rectangles(d[f"f_{k}"], d[f"g_{k}"], a, b)
        np.testing.assert_array_equal(got, d[f"rects_{k}"])
        k += 1
    assert k == 40
