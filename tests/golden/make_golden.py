"""Generate the golden fixtures in this directory from the stablebear
reference's own code.

Runs only where the reference tree is present: it compiles
``oracle/ref_harness.cpp`` against the reference's unmodified headers
(``oracle/build_oracle.py``) and records, for seeded small inputs, the
reference's outputs in its own DistanceMatrix / SymmetricMatrix / dense
layouts.  The GPU tests compare the CUDA path against these files, so they
need neither the reference nor the oracle at run time.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from stablebear_gb300 import synthetic  # noqa: E402


def _ragged(n, lo, hi, dtype, seed):
    return synthetic.gaussian(n, synthetic.uniform_lengths(lo, hi), dtype, seed)


def _with_tails(pts, off, seed):
    """Give some PCFs non-zero last values (the last rectangle then runs to
    numeric_limits<T>::max(), as in the reference)."""
    rng = np.random.default_rng(seed)
    pts = pts.copy()
    last = off[1:].astype(np.int64) - 1
    pick = rng.random(len(last)) < 0.15
    pts[last[pick], 1] = rng.uniform(-0.5, 0.5, size=pick.sum()).astype(pts.dtype)
    return pts


def _with_ties(pts, off, seed, dtype):
    """Snap times onto a coarse grid so PCFs share breakpoint times (ties
    across PCFs) while staying strictly increasing within each PCF."""
    rng = np.random.default_rng(seed)
    pts = pts.copy()
    lens = np.diff(off.astype(np.int64))
    for i in range(len(lens)):
        a, b = int(off[i]), int(off[i + 1])
        steps = rng.integers(1, 3, size=b - a).astype(np.float64)
        steps[0] = 0.0
        pts[a:b, 0] = (np.cumsum(steps) * 0.5).astype(dtype)
    return pts


def main():
    if orc.ref_lib() is None:
        raise SystemExit("reference tree absent: cannot generate golden fixtures")
    cases = []
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        pts, off = _ragged(48, 1, 40, dt, seed=11)
        cases.append((f"ragged_{tag}", pts, off))
        cases.append((f"tails_{tag}", _with_tails(pts, off, 5), off))
        cases.append((f"ties_{tag}", _with_ties(pts, off, 7, dt), off))
        ypts, yoff = _ragged(17, 1, 30, dt, seed=13)
        cases.append((f"cols_{tag}", ypts, yoff))

    out = {}
    for name, pts, off in cases:
        out[f"{name}__points"] = pts
        out[f"{name}__offsets"] = off
    for name, pts, off in cases:
        if name.startswith("cols_"):
            continue
        tag = name[-3:]
        ypts, yoff = out[f"cols_{tag}__points"], out[f"cols_{tag}__offsets"]
        out[f"{name}__pdist_l1"] = orc.ref_evaluate(pts, off, op=orc.OP_L1, mode=orc.MODE_PDIST)
        out[f"{name}__pdist_l2"] = orc.ref_evaluate(pts, off, op=orc.OP_LP, p=2.0, mode=orc.MODE_PDIST)
        out[f"{name}__pdist_l3"] = orc.ref_evaluate(pts, off, op=orc.OP_LP, p=3.0, mode=orc.MODE_PDIST)
        out[f"{name}__kernel"] = orc.ref_evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL)
        out[f"{name}__cdist_l1"] = orc.ref_evaluate(pts, off, op=orc.OP_L1, mode=orc.MODE_CROSS,
                                                    col_points=ypts, col_offsets=yoff)
        out[f"{name}__cdist_l2k"] = orc.ref_evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_CROSS,
                                                     col_points=ypts, col_offsets=yoff)
        out[f"{name}__cdist_l15"] = orc.ref_evaluate(pts, off, op=orc.OP_LP, p=1.5, mode=orc.MODE_CROSS,
                                                     col_points=ypts, col_offsets=yoff)
        # FP64 double-double truth for the same problems
        out[f"{name}__pdist_l1_truth"] = orc.evaluate(pts, off, op=orc.OP_L1, mode=orc.MODE_PDIST, truth=True)
        out[f"{name}__kernel_truth"] = orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL, truth=True)
    path = os.path.join(HERE, "reference_pairwise.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")

    # The reference's rectangle walk on its own unit-test PCFs, kept as rows
    # (left, right, f, g): test/test_iterate_rectangles.cpp:18-19 inputs.
    f = np.array([[0., 3.], [1., 2.], [4., 5.], [6., 0.]])
    g = np.array([[0., 2.], [3., 4.], [4., 2.], [5., 1.], [8., 3.]])
    rects = {
        "full": orc.ref_rectangles(f, g),
        "end_early": orc.ref_rectangles(f, g, 0.0, 4.5),
        "start_late": orc.ref_rectangles(f, g, 2.0),
    }
    np.savez(os.path.join(HERE, "reference_rectangles.npz"), f=f, g=g, **rects)
    rectangle_cases()

    # CudaBlockScheduler blocks for a few configurations.
    sched = {}
    for k, (nr, nc, mo, ns, lower, ms) in enumerate([
            (10, 10, 16, 1, True, 0), (100, 100, 400, 4, True, 0), (100, 37, 400, 4, False, 0),
            (1000, 1000, 10000, 32, True, 64), (5, 7, 1, 1, False, 0), (257, 257, 1 << 20, 32, True, 0)]):
        blocks, mh, mw = orc.ref_schedule(nr, nc, mo, ns, lower, ms)
        sched[f"cfg{k}"] = np.array([nr, nc, mo, ns, int(lower), ms, mh, mw], dtype=np.uint64)
        sched[f"blocks{k}"] = blocks
    np.savez(os.path.join(HERE, "reference_scheduler.npz"), **sched)

    # The reference's on-disk body of small DistanceMatrix / SymmetricMatrix
    # objects (u64 n, then the condensed storage).
    rng = np.random.default_rng(5)
    io_cases = {}
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        for kind, n, name in ((1, 6, "dist"), (2, 5, "sym"), (1, 0, "dist_empty"), (2, 1, "sym_one")):
            cnt = n * (n - 1) // 2 if kind == 1 else n * (n + 1) // 2
            st = rng.uniform(0, 10, cnt).astype(dt)
            io_cases[f"{name}_{tag}_storage"] = st
            io_cases[f"{name}_{tag}_n"] = np.array([n], np.uint64)
            io_cases[f"{name}_{tag}_body"] = np.frombuffer(orc.ref_matrix_body(kind, n, st), np.uint8)
    np.savez(os.path.join(HERE, "reference_matrix_io.npz"), **io_cases)

    # Lp norms through the reference's own iterate_segments: ragged PCFs with
    # tails, repeated t = 0 breakpoints and ties, p in {1, 1.5, 2, 3}.
    norms = {}
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        pts, off = _ragged(60, 1, 40, dt, 21)
        pts = _with_tails(pts, off, 22)
        pts = _with_ties(pts, off, 23, dt) if tag == "f64" else pts
        # a PCF whose first two breakpoints sit at t = 0
        a = int(off[3])
        if int(off[4]) - a >= 3:
            pts[a + 1, 0] = 0
        norms[f"{tag}_points"] = pts
        norms[f"{tag}_offsets"] = off
        for p in (1.0, 1.5, 2.0, 3.0):
            norms[f"{tag}_p{p}"] = orc.ref_lp_norm(pts, off, p)
    np.savez(os.path.join(HERE, "reference_norms.npz"), **norms)


def rectangle_cases():
    """The reference's rectangle walk on seeded random pairs with repeated
    times (zero-width segments), breakpoints shared by f and g, and bounds
    before, on and between breakpoints.  Times and values are multiples of
    1/2 below 64, exact in float32 as well."""
    from oracle import oracle as orc
    rng = np.random.default_rng(77)
    out = {}
    for k in range(40):
        def pcf():
            n = int(rng.integers(1, 13))
            t = np.concatenate([[0.0], np.cumsum(rng.choice([0.0, 0.5, 1.0, 1.5], size=n - 1))])
            v = rng.integers(-4, 5, size=n).astype(np.float64)
            return np.stack([t, v], 1)
        f, g = pcf(), pcf()
        if k % 3 == 0 and len(f) > 2:  # share some of f's breakpoints with g
            g = np.concatenate([g, f[1:3]])
            g = g[np.argsort(g[:, 0], kind="stable")]
            g[0, 0] = 0.0
        a = float(rng.choice([0.0, 0.0, 0.5, 1.25, 3.0, -1.0]))
        b = float(rng.choice([np.finfo(np.float64).max, 2.5, 4.0, 100.0, a]))
        out[f"f_{k}"], out[f"g_{k}"] = f, g
        out[f"ab_{k}"] = np.array([a, b])
        out[f"rects_{k}"] = orc.ref_rectangles(f, g, a, b)
    path = os.path.join(HERE, "reference_rectangle_cases.npz")
    np.savez(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    if "--rectangles" in sys.argv:
        rectangle_cases()
        sys.exit(0)
    main()
