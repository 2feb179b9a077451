"""The reference's 12 C++ factories through include/sbgpu/compat.hpp, on the
reference's five-PCF test input, against the oracle (f32 1e-5, f64 1e-12)."""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu


def _five(dt):
    rows = [[[0, 1], [1, 0]], [[0, 2], [0.5, 1], [1.5, 0]], [[0, 0], [1, 3], [2, 0]], [[0, 5]],
            [[0, 1], [0.25, 2], [0.75, 1], [1, 0]]]
    pts = np.concatenate([np.array(r, dt) for r in rows])
    off = np.zeros(6, np.uint64)
    np.cumsum([len(r) for r in rows], out=off[1:])
    return pts, off


def test_factories_match_oracle(tmp_path):
    from stablebear_gb300 import build
    from oracle import oracle as orc
    lib = build.build()
    exe = str(tmp_path / "test_factories")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_factories.cpp"), "-o", exe, "-L", os.path.dirname(lib),
                    "-lsbgpu", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got = {}
    for ln in r.stdout.splitlines():
        tag, key, *vals = ln.split()
        got.setdefault((tag, key), []).extend(float(v) for v in vals)
    for tag, dt, tol in (("f32", np.float32, 1e-5), ("f64", np.float64, 1e-12)):
        pts, off = _five(dt)
        cp, co = pts[int(off[2]):], (off[2:] - off[2]).astype(np.uint64)
        rp, ro = pts[:int(off[2])], off[:3]
        want = {
            "l1": orc.evaluate(pts, off),
            "l2": orc.evaluate(pts, off, op=orc.OP_LP, p=2.0),
            "k": orc.evaluate(pts, off, op=orc.OP_L2, mode=orc.MODE_KERNEL),
            "c": orc.evaluate(rp, ro, mode=orc.MODE_CROSS, col_points=cp, col_offsets=co),
        }
        for key, w in want.items():
            g = np.array(got[(tag, key)])
            assert g.shape == w.shape
            fin = np.isfinite(w)
            # PCF 3 never returns to zero: its distances are inf, as in the reference
            np.testing.assert_array_equal(g[~fin], w[~fin])
            rel = np.abs(g[fin] - w[fin]) / np.maximum(np.abs(w[fin]), 1.0 if key == "k" else 1e-30)
            assert rel.max() <= tol, (tag, key, g, w)
        assert got[(tag, "range_rejected")] == [1.0]
        # the reference's known answers (test/test_l1_dist.cu:98-124), exact
        assert got[(tag, "kat_empty")] == [0.0]
        assert got[(tag, "kat_two")] == [0.0, 3.0, 3.0, 0.0]
