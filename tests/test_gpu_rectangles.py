"""iterate_rectangles on the device against the reference's own walk.

The golden fixtures hold the reference's rectangles (its C++
iterate_rectangles, compiled from its headers by oracle/ref_harness.cpp) for
its unit-test PCFs and for 40 random pairs with repeated times, breakpoints
shared by f and g, and bounds before, on and between breakpoints; all their
numbers are exact in float32 too.  Larger random pairs are checked against
the oracle's restatement of the walk.  Every comparison is exact: the walk
only compares and copies.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
DBL_MAX = np.finfo(np.float64).max


@pytest.fixture(scope="module", autouse=True)
def native():
    from stablebear_gb300 import build
    build.build()


def rows(rects):
    return np.array([(r.left, r.right, r.f_value, r.g_value) for r in rects], dtype=np.float64).reshape(-1, 4)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_reference_cases(dt):
    import stablebear_gb300 as sb
    d = np.load(os.path.join(GOLDEN, "reference_rectangle_cases.npz"))
    for k in range(40):
        f, g = sb.Pcf(d[f"f_{k}"].astype(dt)), sb.Pcf(d[f"g_{k}"].astype(dt))
        a, b = d[f"ab_{k}"]
        want = d[f"rects_{k}"]
        if dt == np.float32 and b == DBL_MAX:
            b = float(np.finfo(np.float32).max)
            want = want.copy()
            want[want[:, 1] == DBL_MAX, 1] = b
        got = rows(sb.iterate_rectangles(f, g, a, b))
        np.testing.assert_array_equal(got, want.astype(dt).astype(np.float64), err_msg=f"case {k}")


def test_reference_unit_test_pcfs():
    import stablebear_gb300 as sb
    d = np.load(os.path.join(GOLDEN, "reference_rectangles.npz"))
    f, g = sb.Pcf(d["f"]), sb.Pcf(d["g"])
    np.testing.assert_array_equal(rows(sb.iterate_rectangles(f, g, 0.0, DBL_MAX)), d["full"])
    np.testing.assert_array_equal(rows(sb.iterate_rectangles(f, g, 0.0, 4.5)), d["end_early"])
    np.testing.assert_array_equal(rows(sb.iterate_rectangles(f, g, 2.0, DBL_MAX)), d["start_late"])


def test_known_answers():
    """The reference's Python known answers (test/python/test_iterate_rectangles.py)."""
    import stablebear_gb300 as sb
    f = sb.Pcf([[0, 3], [1, 2], [4, 5], [6, 0]], dtype=sb.pcf32)
    g = sb.Pcf([[0, 2], [3, 4], [4, 2], [5, 1], [8, 3]], dtype=sb.pcf32)
    r = sb.iterate_rectangles(f, g)
    assert [x == y for x, y in zip(r[:6], [(0, 1, 3, 2), (1, 3, 2, 2), (3, 4, 2, 4), (4, 5, 5, 2), (5, 6, 5, 1),
                                           (6, 8, 0, 1)])] == [True] * 6
    assert len(r) == 7 and r[6].left == 8 and math.isinf(r[6].right) and (r[6].f_value, r[6].g_value) == (0, 3)
    assert len(sb.iterate_rectangles(f, g, b=4.0)) == 3
    assert sb.iterate_rectangles(f, g, a=1.0, b=1.0) == []
    r = sb.iterate_rectangles(f, g, a=2.0, b=4.5)
    assert [(x.left, x.right, x.f_value, x.g_value) for x in r] == [(2, 3, 2, 2), (3, 4, 2, 4), (4, 4.5, 5, 2)]
    fg, gf = sb.iterate_rectangles(f, g, b=6.0), sb.iterate_rectangles(g, f, b=6.0)
    assert [(x.left, x.right, x.f_value, x.g_value) for x in fg] == [(x.left, x.right, x.g_value, x.f_value) for x in gf]
    one = sb.iterate_rectangles(sb.Pcf([[0, 7]], dtype=sb.pcf64), sb.Pcf([[0, 3]], dtype=sb.pcf64))
    assert len(one) == 1 and one[0].left == 0 and math.isinf(one[0].right) and (one[0].f_value, one[0].g_value) == (7, 3)
    same = sb.iterate_rectangles(sb.Pcf([[0, 1], [2, 3], [4, 0]]), sb.Pcf([[0, 10], [2, 20], [4, 0]]))
    assert [(x.left, x.right, x.f_value, x.g_value) for x in same[:2]] == [(0, 2, 1, 10), (2, 4, 3, 20)]
    assert len(same) == 3


@pytest.mark.parametrize("dt", [np.float32, np.float64, np.int32, np.int64])
def test_random_pairs_against_oracle(dt):
    import stablebear_gb300 as sb
    from oracle import oracle as orc
    rng = np.random.default_rng(5)
    for case in range(30):
        def pcf():
            n = int(rng.integers(1, 3000))
            step = rng.choice([0, 1, 2, 3], size=n - 1, p=[0.2, 0.4, 0.3, 0.1])
            t = np.concatenate([[0], np.cumsum(step)]).astype(dt)
            v = rng.integers(-9, 10, size=n).astype(dt)
            return np.stack([t, v], 1)
        f, g = pcf(), pcf()
        a = int(rng.integers(-2, 50))
        b = float(rng.choice([np.inf, 100, 2000, a]))
        got = rows(sb.iterate_rectangles(sb.Pcf(f), sb.Pcf(g), a, b))
        bb = b if np.issubdtype(dt, np.floating) or math.isfinite(b) else float(np.iinfo(dt).max)
        want = orc.rectangles(f.astype(np.float64), g.astype(np.float64), float(a), bb)
        np.testing.assert_array_equal(got, want, err_msg=f"case {case}")


def test_type_errors():
    import stablebear_gb300 as sb
    f = sb.Pcf([[0, 1], [1, 0]], dtype=sb.pcf32)
    with pytest.raises(TypeError):
        sb.iterate_rectangles(f, sb.Pcf([[0, 1], [1, 0]], dtype=sb.pcf64))
    with pytest.raises(TypeError):
        sb.iterate_rectangles(f, [[0, 1]])
