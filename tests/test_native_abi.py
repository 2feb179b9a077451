"""The C-ABI library: builds, loads, exports every declared symbol, and its
host-only logic (argument checks, work-item tiling) — no GPU needed."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "sbgpu.h")


@pytest.fixture(scope="module")
def lib():
    from stablebear_gb300 import build, _native
    build.build()
    return _native.lib()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sbg_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    from stablebear_gb300 import _native
    names = declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), f"{name} declared in sbgpu.h but not exported"
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"


def test_alloc_limit_and_counters_need_no_device(lib):
    from stablebear_gb300 import _native
    held = lib.sbg_device_bytes_held()
    count = lib.sbg_device_allocations()
    assert lib.sbg_set_alloc_limit(0) == 0
    assert lib.sbg_set_alloc_limit(_native.ALLOC_UNLIMITED) == 0
    assert lib.sbg_device_bytes_held() == held and lib.sbg_device_allocations() == count


def test_tuning_cache_needs_no_device(lib):
    hit, w, r = ctypes.c_int(-1), ctypes.c_int(-1), ctypes.c_int(-1)
    assert lib.sbg_tuning_cache_clear() == 0
    assert lib.sbg_tuning_cache_lookup(0, 0, 1.0, 1, 1000, 200, ctypes.byref(w), ctypes.byref(r),
                                       ctypes.byref(hit)) == 0
    assert hit.value == 0 and w.value == 0 and r.value == 0
    assert lib.sbg_tuning_cache_lookup(0, 1, 0.5, 1, 1000, 200, None, None, ctypes.byref(hit)) == -1  # p < 1
    # the autotuner checks its arguments before any CUDA call
    assert lib.sbg_autotune_device(0, 0, 1.0, 1, None, None, 10, None, None, 0, 0, None, None, None, None,
                                   None) == -1


def test_every_device_allocation_goes_through_the_counted_allocator():
    """Only the library's allocator (engine.cu: device_malloc / device_free and
    their stream-ordered pair) calls the CUDA allocation routines, so the
    allocation limit and counter see every device allocation.  Checked on the
    sources, comments stripped."""
    csrc = os.path.join(ROOT, "stablebear_gb300", "csrc")
    raw = re.compile(r"\bcuda(Malloc|MallocAsync|MallocManaged|MallocPitch|Malloc3D|MallocArray|Free|FreeAsync)\s*\(")
    found = {}
    for f in sorted(os.listdir(csrc)):
        if not f.endswith((".cu", ".cuh", ".hpp", ".h")):
            continue
        text = open(os.path.join(csrc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        n = len(raw.findall(text))
        if n:
            found[f] = n
    assert found == {"engine.cu": 4}, found


def test_version_and_build_type(lib):
    assert lib.sbg_api_version() == 1
    assert lib.sbg_build_type() == b"CUDA"


def test_argument_errors_need_no_device(lib):
    h = ctypes.c_void_p()
    pts = np.zeros((2, 2), np.float32)
    off = np.array([0, 1, 2], np.uint64)
    out = np.zeros(1, np.float32)
    P = lambda a: ctypes.c_void_p(a.ctypes.data)
    # unknown dtype
    assert lib.sbg_create_integrate_task(7, 0, 1.0, 1, P(pts), P(off), 2, P(out), ctypes.byref(h)) == -1
    # p < 1 for Lp
    assert lib.sbg_create_integrate_task(0, 1, 0.5, 1, P(pts), P(off), 2, P(out), ctypes.byref(h)) == -1
    assert b"p must be >= 1" in lib.sbg_last_error()
    # cdist through the pairwise factory is rejected
    assert lib.sbg_create_integrate_task(0, 0, 1.0, 0, P(pts), P(off), 2, P(out), ctypes.byref(h)) == -1
    assert lib.sbg_set_tuning(99, 0, 0, 0, 0) == -1
    assert lib.sbg_set_block_dim(0, 1) == -1
    # the newer entries check their arguments before any CUDA call
    assert lib.sbg_block_device(7, 0, 1.0, 1, None, None, None, None, 0, 4, 0, 4, 8, None, None) == -1
    assert lib.sbg_block_device(0, 1, 0.5, 1, None, None, None, None, 0, 4, 0, 4, 8, None, None) == -1
    assert b"p must be >= 1" in lib.sbg_last_error()
    assert lib.sbg_block_device(0, 0, 1.0, 1, None, None, None, None, 0, 4, 0, 4, 8, None, None) == -1
    assert b"null pointer" in lib.sbg_last_error()
    assert lib.sbg_lp_norm_host(0, 0.5, P(pts), P(off), 2, P(out)) == -1
    assert lib.sbg_condensed_to_dense_device(0, 0, 4, None, None, 4, 0, 4, None) == -1  # cdist storage is not condensed
    assert lib.sbg_barcodes_to_pcfs_host(5, 0, None, None, 0, None, 0, None) == -1
    assert lib.sbg_barcode_pcf_capacity(0, 3, 10) == 13 and lib.sbg_barcode_pcf_capacity(1, 3, 10) == 23


def test_invalid_pcf_input_rejected_before_device(lib):
    h = ctypes.c_void_p()
    P = lambda a: ctypes.c_void_p(a.ctypes.data)
    out = np.zeros(1, np.float64)
    off = np.array([0, 2, 3], np.uint64)
    unsorted = np.array([[0, 1], [-1, 2], [0, 0]], np.float64)
    assert lib.sbg_create_integrate_task(1, 0, 1.0, 1, P(unsorted), P(off), 2, P(out), ctypes.byref(h)) == -2
    assert b"non-decreasing" in lib.sbg_last_error()
    bad_t0 = np.array([[1, 1], [2, 2], [0, 0]], np.float64)
    assert lib.sbg_create_integrate_task(1, 0, 1.0, 1, P(bad_t0), P(off), 2, P(out), ctypes.byref(h)) == -2
    assert b"t=0" in lib.sbg_last_error()
    nan_t = np.array([[0, 1], [np.nan, 2], [0, 0]], np.float64)
    assert lib.sbg_create_integrate_task(1, 0, 1.0, 1, P(nan_t), P(off), 2, P(out), ctypes.byref(h)) == -2
    empty = np.array([0, 0, 3], np.uint64)
    ok = np.array([[0, 1], [1, 2], [2, 0]], np.float64)
    assert lib.sbg_create_integrate_task(1, 0, 1.0, 1, P(ok), P(empty), 2, P(out), ctypes.byref(h)) == -2
    assert b"no breakpoints" in lib.sbg_last_error()


def test_large_input_validation_reports_first_invalid_pcf(lib):
    """Inputs of a million points and more are checked by the host thread
    pool in parallel ranges; the error still names the first invalid PCF."""
    h = ctypes.c_void_p()
    P = lambda a: ctypes.c_void_p(a.ctypes.data)
    out = np.zeros(1, np.float64)
    n, L = 3000, 400
    t = np.tile(np.arange(L, dtype=np.float64), n)
    pts = np.stack([t, np.ones(n * L)], 1)
    off = (np.arange(n + 1, dtype=np.uint64) * L).astype(np.uint64)
    bad = pts.copy()
    bad[2900 * L + 7, 0] = -1.0
    bad[1200 * L + 9, 0] = -1.0
    assert lib.sbg_create_integrate_task(1, 0, 1.0, 1, P(bad), P(off), n, P(out), ctypes.byref(h)) == -2
    assert b"PCF 1200:" in lib.sbg_last_error() and b"non-decreasing" in lib.sbg_last_error()
    last = pts.copy()
    last[(n - 1) * L, 0] = 0.5
    assert lib.sbg_create_integrate_task(1, 0, 1.0, 1, P(last), P(off), n, P(out), ctypes.byref(h)) == -2
    assert b"PCF 2999:" in lib.sbg_last_error() and b"t=0" in lib.sbg_last_error()

    # A child forked after the pool's threads started has none of them: the
    # same check there runs its parts on the calling thread, and the child
    # exits without waiting for threads it does not have.
    import multiprocessing as mp
    q = mp.get_context("fork").Queue()

    def child():
        st = lib.sbg_create_integrate_task(1, 0, 1.0, 1, P(bad), P(off), n, P(out), ctypes.byref(ctypes.c_void_p()))
        q.put((st, lib.sbg_last_error()))

    proc = mp.get_context("fork").Process(target=child)
    proc.start()
    proc.join(60)
    alive = proc.is_alive()
    if alive:
        proc.kill()
    assert not alive and proc.exitcode == 0
    st, msg = q.get(timeout=5)
    assert st == -2 and b"PCF 1200:" in msg


def test_settings_roundtrip(lib):
    import stablebear_gb300 as sb
    sb.set_cuda_threshold(123)
    assert sb.get_cuda_threshold() == 123
    sb.set_cuda_threshold(500)
    sb.set_device_verbose(True)
    assert lib.sbg_get_device_verbose() == 1
    sb.set_device_verbose(False)
    sb.force_cpu(True)
    assert lib.sbg_get_force_cpu() == 1
    sb.force_cpu(False)
    sb.set_tuning()
    # the time-windowed variant and its window cap
    assert lib.sbg_set_tuning(0, 0, 6, 0, 0) == 0
    assert lib.sbg_set_tuning(0, 0, 8, 0, 0) == 0  # the measurement variants 7 and 8
    assert lib.sbg_set_tuning(0, 0, 9, 0, 0) == -1
    assert b"variant" in lib.sbg_last_error()
    sb.set_window_cap(40)
    assert sb.get_window_cap() == 40
    assert lib.sbg_set_window_cap(-1) == -1
    assert lib.sbg_set_window_cap((1 << 20) + 1) == -1
    assert b"window cap" in lib.sbg_last_error()
    assert sb.get_window_cap() == 40
    sb.set_window_cap(0)
    sb.set_tuning()


def _items(lib, mode, nr, nc, rb, re, q):
    n = lib.sbg_enumerate_items(mode, nr, nc, rb, re, q, None, 0)
    buf = np.zeros(2 * max(n, 1), np.uint64)
    lib.sbg_enumerate_items(mode, nr, nc, rb, re, q, ctypes.c_void_p(buf.ctypes.data), n)
    return buf[: 2 * n].reshape(-1, 2)


def _covered(items, mode, nr, nc, rb, re, q):
    """Expand items to the set of (i, j) pairs the kernel visits (same row /
    lane masks as pairs_kernel), with multiplicity."""
    seen = np.zeros((nr, nc), np.int64)
    for c, g in items:
        lo = rb + int(c) * 32 * q
        hi = min(lo + 32 * q, re)
        col0 = 32 * int(g)
        if mode != 0:
            lo = max(lo, col0 + (1 if mode == 1 else 0))
        for i in range(lo, hi):
            for j in range(col0, min(col0 + 32, nc)):
                if mode == 0 or (j < i if mode == 1 else j <= i):
                    seen[i, j] += 1
    return seen


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("n,q", [(1, 1), (2, 1), (31, 1), (32, 1), (33, 1), (100, 2), (200, 1), (257, 4), (300, 16)])
def test_work_items_tile_exactly_once(lib, mode, n, q):
    nc = n if mode else max(1, n // 2 + 3)
    items = _items(lib, mode, n, nc, 0, n, q)
    seen = _covered(items, mode, n, nc, 0, n, q)
    want = np.ones((n, nc), np.int64)
    if mode == 1:
        want = np.tril(want, -1)
    elif mode == 2:
        want = np.tril(want)
    np.testing.assert_array_equal(seen, want)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_work_items_of_bands_tile_exactly_once(lib, mode):
    n, q = 700, 2
    nc = n if mode else 90
    seen = np.zeros((n, nc), np.int64)
    bands = [(0, 64), (64, 320), (320, 448), (448, 700)]
    for rb, re in bands:
        seen += _covered(_items(lib, mode, n, nc, rb, re, q), mode, n, nc, rb, re, q)
    want = np.ones((n, nc), np.int64)
    if mode == 1:
        want = np.tril(want, -1)
    elif mode == 2:
        want = np.tril(want)
    np.testing.assert_array_equal(seen, want)


def test_output_count(lib):
    assert lib.sbg_output_count(1, 5, 5) == 10
    assert lib.sbg_output_count(2, 5, 5) == 15
    assert lib.sbg_output_count(0, 5, 7) == 35
    assert lib.sbg_output_count(1, 0, 0) == 0
