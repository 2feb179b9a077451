"""The C++ drop-in header (include/sbgpu/compat.hpp): the kept scheduler and
result-writer interfaces, checked against the reference scheduler's own
blocks (golden fixture) and the writer's known answers.  CPU only."""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import GOLDEN, ROOT


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    from stablebear_gb300 import build
    lib = build.build()
    out = str(tmp_path_factory.mktemp("cpp") / "test_compat")
    src = os.path.join(ROOT, "tests", "cpp", "test_compat.cpp")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", out,
                    "-L", os.path.dirname(lib), "-lsbgpu", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return out


def test_writers_and_matrices(exe):
    r = subprocess.run([exe, "writers"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"


def test_scheduler_matches_reference_blocks(exe):
    d = np.load(os.path.join(GOLDEN, "reference_scheduler.npz"))
    k = 0
    while f"cfg{k}" in d:
        nr, nc, mo, ns, lower, ms, mh, mw = (int(x) for x in d[f"cfg{k}"])
        r = subprocess.run([exe, "schedule", str(nr), str(nc), str(mo), str(ns), str(lower), str(ms)],
                           capture_output=True, text=True, check=True)
        lines = r.stdout.strip().splitlines()
        count, gh, gw = (int(x) for x in lines[0].split())
        assert (gh, gw) == (mh, mw)
        blocks = np.array([[int(x) for x in ln.split()] for ln in lines[1:]], dtype=np.uint64).reshape(-1, 5)
        np.testing.assert_array_equal(blocks, d[f"blocks{k}"])
        k += 1
    assert k >= 5


@pytest.mark.parametrize("n,side,splits,lower", [(0, 4, 1, True), (1, 4, 1, True), (37, 5, 3, True), (37, 5, 3, False),
                                                (100, 200, 7, True)])
def test_scheduler_covers_exactly_once(exe, n, side, splits, lower):
    """test/test_block_scheduler.cpp:10-46: every (i, j) of the lower
    triangle (or the full matrix) is covered by exactly one block."""
    r = subprocess.run([exe, "schedule", str(n), str(n), str(side * side * splits), str(splits), str(int(lower)), "0"],
                       capture_output=True, text=True, check=True)
    lines = r.stdout.strip().splitlines()
    seen = np.zeros((n, n), np.int64)
    areas = []
    for ln in lines[1:]:
        rs, rh, cs, cw, _ = (int(x) for x in ln.split())
        seen[rs:rs + rh, cs:cs + cw] += 1
        areas.append(rh * cw)
    assert areas == sorted(areas, reverse=True)
    want = np.tril(np.ones((n, n), np.int64)) if lower else np.ones((n, n), np.int64)
    covered = seen * want
    assert (covered == want).all()
