"""Seeded random cases across the planner's choices, against the double-double
truth oracle.

Each case draws a PCF count, a length distribution (short, mixed, long), an
element type, an operation and mode (pdist L1 / L2 / Lp, L2 kernel, cdist),
and forces a kernel variant (automatic, the shared-memory ones, global
memory, hybrid, time-windowed with caps down to one element), a warp count
and a row chunk.  Every combination must give the same integrals: float32
within 3e-5 relative of the truth (window caps below 32 only with PCFs of at
most 150 elements, where the float32 sum they make close to a naive one stays
inside that), Lp with general p 1e-4; float64 within 1e-12 (general p:
1e-10, the reference's own GPU-vs-CPU bound for pow in double); the L2
kernel against max(|truth|, 1).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_CASES = 400


@pytest.fixture(scope="module", autouse=True)
def native():
    from stablebear_gb300 import build
    build.build()
    import stablebear_gb300 as sb
    yield
    sb.set_tuning()
    sb.set_window_cap(0)


def _pcfs(rng, n, dt):
    kind = rng.integers(0, 3)
    if kind == 0:
        lens = rng.integers(1, 6, size=n)
    elif kind == 1:
        lens = rng.integers(1, 120, size=n)
    else:
        lens = np.where(rng.random(n) < 0.3, rng.integers(300, 1500, size=n), rng.integers(1, 40, size=n))
    pts, off = [], [0]
    for L in lens:
        gaps = rng.exponential(1.0, L - 1)
        if rng.random() < 0.2:
            gaps = np.round(gaps * 2) / 2  # ties and zero-width segments
        t = np.concatenate([[0.0], np.cumsum(gaps)])
        v = rng.normal(size=L)
        v[-1] = 0.0
        pts.append(np.stack([t, v], 1))
        off.append(off[-1] + L)
    return np.concatenate(pts).astype(dt), np.array(off, dtype=np.uint64)


def _rel(got, want, floor):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), floor))) if want.size else 0.0


def test_random_cases_against_truth():
    import stablebear_gb300 as sb
    from oracle import oracle as orc
    rng = np.random.default_rng(20261203)
    failures = []
    ran = 0
    try:
        for case in range(N_CASES):
            dt = np.float32 if rng.random() < 0.75 else np.float64
            n = int(rng.integers(1, 70))
            pts, off = _pcfs(rng, n, dt)
            variant = int(rng.choice([0, 0, 1, 2, 3, 4, 5, 6, 6, 6]))
            cap = int(rng.choice([0, 0, 1, 3, 7, 32])) if variant in (0, 6) else 0
            if 0 < cap < 32 and int(np.diff(off.astype(np.int64)).max()) > 150:
                # a long pair hands its sum on once per window: with caps this
                # small that is a naive float32 sum of ~1500 terms, whose error
                # (~5e-5) is the reference's own, not the bound here
                cap = 32
            warps = int(rng.choice([0, 0, 4, 8, 16]))
            chunk = int(rng.choice([0, 0, 1, 2]))
            what = rng.integers(0, 5)
            X = sb.PcfArray.from_csr(pts, off)
            try:
                sb.set_tuning(warps=warps, row_chunk=chunk, variant=variant)
                sb.set_window_cap(cap)
                if what == 0:
                    got, want, floor, tol = sb.pdist(X).data, orc.evaluate(pts, off, truth=True), 1e-30, 3e-5
                elif what == 1:
                    got = sb.pdist(X, p=2).data
                    want, floor, tol = orc.evaluate(pts, off, op=orc.OP_LP, p=2.0, truth=True), 1e-30, 3e-5
                elif what == 2:
                    got = sb.pdist(X, p=1.5).data
                    want, floor, tol = orc.evaluate(pts, off, op=orc.OP_LP, p=1.5, truth=True), 1e-30, 1e-4
                elif what == 3:
                    got = sb.l2_kernel(X).data
                    want = orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL, truth=True)
                    floor, tol = 1.0, 3e-5
                else:
                    yp, yo = _pcfs(rng, int(rng.integers(1, 40)), dt)
                    got = sb.cdist(X, sb.PcfArray.from_csr(yp, yo)).reshape(-1)
                    want = orc.evaluate(pts, off, mode=orc.MODE_CROSS, col_points=yp, col_offsets=yo, truth=True)
                    floor, tol = 1e-30, 3e-5
            except ValueError as e:
                # a forced variant the PCFs cannot use (too long for shared memory)
                if "shared memory" in str(e):
                    continue
                raise
            ran += 1
            if dt == np.float64:
                tol = 1e-12 if tol < 1e-4 else 1e-10
            err = _rel(got, want, floor)
            if not err <= tol:
                failures.append((case, dt.__name__, n, variant, cap, warps, chunk, int(what), err))
    finally:
        sb.set_tuning()
        sb.set_window_cap(0)
    assert not failures, failures
    assert ran >= 0.8 * N_CASES, ran  # few cases skipped for a variant the PCFs cannot use
