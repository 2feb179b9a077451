"""ORACLE — test infrastructure only (ctypes front-end of ``pcf_oracle.c``).

Used by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg, as the parity reference.  The product package never imports it.

Inputs use the reference's CSR layout: ``points`` is an ``(M, 2)`` array of
``(t, v)`` rows (float32 or float64), ``offsets`` a ``uint64`` array of length
``N + 1``; PCF ``i`` is ``points[offsets[i]:offsets[i+1]]``
(``include/sbear/cuda/offset_data_manager.hpp:42-68`` in the reference).

Modes follow the reference's TriangleSkipMode
(``include/sbear/cuda/triangle_skip_mode.hpp:7-12``): 0 = cdist (dense),
1 = pdist (DistanceMatrix order), 2 = l2 kernel (SymmetricMatrix order).
Ops follow ``include/sbear/functional/operations.cuh``: 0 = L1, 1 = Lp,
2 = L2 inner product.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle as _build

OP_L1, OP_LP, OP_L2 = 0, 1, 2
MODE_CROSS, MODE_PDIST, MODE_KERNEL = 0, 1, 2

_libs = {}
_ref = None
_P = ctypes.c_void_p
_U64 = ctypes.c_uint64


def _load(build="check"):
    """The oracle library: ``"check"`` is the -O2 -ffp-contract=off build every
    parity test uses; ``"o3_off"`` / ``"o3_fast"`` are the -O3 host-CPU builds
    without / with FMA contraction that only the CPU-baseline timings use."""
    lib = _libs.get(build)
    if lib is None:
        if build == "check":
            path = _build.build_oracle()
        elif build in ("o3_off", "o3_fast"):
            path = _build.build_oracle_timed(build[3:])
        else:
            raise ValueError(f"unknown oracle build {build!r}")
        lib = ctypes.CDLL(path)
        lib.sbo_evaluate.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                     _P, _P, _U64, _P, _P, _U64, _P, ctypes.c_int]
        lib.sbo_evaluate.restype = ctypes.c_int
        lib.sbo_evaluate_rows.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                          _P, _P, _U64, _P, _P, _U64, _P, _U64, _P, _P, ctypes.c_int]
        lib.sbo_evaluate_rows.restype = ctypes.c_int
        lib.sbo_integrate_f32.argtypes = [_P, _U64, _P, _U64, ctypes.c_int, ctypes.c_float]
        lib.sbo_integrate_f32.restype = ctypes.c_float
        lib.sbo_integrate_f64.argtypes = [_P, _U64, _P, _U64, ctypes.c_int, ctypes.c_double]
        lib.sbo_integrate_f64.restype = ctypes.c_double
        lib.sbo_finalize_f32.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float]
        lib.sbo_finalize_f32.restype = ctypes.c_float
        lib.sbo_finalize_f64.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        lib.sbo_finalize_f64.restype = ctypes.c_double
        lib.sbo_integrate_dd_f32.argtypes = [_P, _U64, _P, _U64, ctypes.c_int, ctypes.c_double]
        lib.sbo_integrate_dd_f32.restype = ctypes.c_double
        lib.sbo_integrate_dd_f64.argtypes = [_P, _U64, _P, _U64, ctypes.c_int, ctypes.c_double]
        lib.sbo_integrate_dd_f64.restype = ctypes.c_double
        lib.sbo_count_total_segments.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, _U64, _P, _P, _U64]
        lib.sbo_count_total_segments.restype = _U64
        lib.sbo_lp_norm.argtypes = [ctypes.c_int, ctypes.c_double, _P, _P, _U64, _P]
        lib.sbo_lp_norm.restype = ctypes.c_int
        lib.sbo_barcodes_to_pcfs.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, _U64, _P, _P]
        lib.sbo_barcodes_to_pcfs.restype = ctypes.c_int
        lib.sbo_evaluate_rows_chunked.argtypes = lib.sbo_evaluate_rows.argtypes + [_U64]
        lib.sbo_evaluate_rows_chunked.restype = ctypes.c_int
        _libs[build] = lib
    return lib


def ref_lib():
    """The reference's own headers compiled into a shared library, or None
    where the reference tree is absent."""
    global _ref
    if _ref is None:
        try:
            path = _build.build_ref()
        except Exception:  # pragma: no cover - compiler problems mean "unavailable"
            path = None
        if path is None:
            _ref = False
        else:
            lib = ctypes.CDLL(path)
            lib.sbref_pair_f32.argtypes = [_P, _U64, _P, _U64, ctypes.c_int, ctypes.c_float]
            lib.sbref_pair_f32.restype = ctypes.c_float
            lib.sbref_pair_f64.argtypes = [_P, _U64, _P, _U64, ctypes.c_int, ctypes.c_double]
            lib.sbref_pair_f64.restype = ctypes.c_double
            lib.sbref_pairwise_f32.argtypes = [_P, _P, _U64, ctypes.c_int, ctypes.c_float, ctypes.c_int, _P]
            lib.sbref_pairwise_f32.restype = ctypes.c_int
            lib.sbref_pairwise_f64.restype = ctypes.c_int
            lib.sbref_pairwise_f64.argtypes = [_P, _P, _U64, ctypes.c_int, ctypes.c_double, ctypes.c_int, _P]
            lib.sbref_cross_f32.argtypes = [_P, _P, _U64, _P, _P, _U64, ctypes.c_int, ctypes.c_float, _P]
            lib.sbref_cross_f64.argtypes = [_P, _P, _U64, _P, _P, _U64, ctypes.c_int, ctypes.c_double, _P]
            lib.sbref_rectangles_f64.argtypes = [_P, _U64, _P, _U64, ctypes.c_double, ctypes.c_double, _P, _U64]
            lib.sbref_rectangles_f64.restype = _U64
            lib.sbref_schedule.argtypes = [_U64, _U64, _U64, _U64, ctypes.c_int, _U64, _P, _U64, _P, _P]
            lib.sbref_schedule.restype = _U64
            lib.sbref_subdivide.argtypes = [_U64, _U64, _P, _U64]
            lib.sbref_subdivide.restype = _U64
            lib.sbref_lp_norm_f32.argtypes = [_P, _U64, ctypes.c_float]
            lib.sbref_lp_norm_f32.restype = ctypes.c_float
            lib.sbref_lp_norm_f64.argtypes = [_P, _U64, ctypes.c_double]
            lib.sbref_lp_norm_f64.restype = ctypes.c_double
            for nm in ("sbref_matrix_body_f32", "sbref_matrix_body_f64"):
                getattr(lib, nm).argtypes = [ctypes.c_int, _U64, _P, _P, _U64]
                getattr(lib, nm).restype = _U64
            _ref = lib
    return _ref or None


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _dtype_code(points):
    if points.dtype == np.float32:
        return 0
    if points.dtype == np.float64:
        return 1
    raise TypeError(f"unsupported dtype {points.dtype}")


def _csr(points, offsets):
    points = np.ascontiguousarray(points)
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    if points.ndim != 2 or points.shape[1] != 2:
        raise ValueError("points must be (M, 2)")
    return points, offsets


def out_size(mode, n_rows, n_cols=None):
    if mode == MODE_PDIST:
        return n_rows * (n_rows - 1) // 2
    if mode == MODE_KERNEL:
        return n_rows * (n_rows + 1) // 2
    return n_rows * n_cols


def evaluate(points, offsets, *, op=OP_L1, p=1.0, mode=MODE_PDIST, col_points=None, col_offsets=None,
             truth=False, threads=None):
    """Naive restatement (``truth=False``; result in the input precision) or
    the double-double truth oracle (``truth=True``; result float64)."""
    lib = _load()
    points, offsets = _csr(points, offsets)
    dt = _dtype_code(points)
    nr = len(offsets) - 1
    if mode == MODE_CROSS:
        col_points, col_offsets = _csr(col_points, col_offsets)
        if col_points.dtype != points.dtype:
            raise TypeError("row and column PCFs must share a dtype")
        nc = len(col_offsets) - 1
    else:
        col_points, col_offsets, nc = points, offsets, nr
    odt = np.float64 if truth else points.dtype
    out = np.zeros(out_size(mode, nr, nc), dtype=odt)
    if threads is None:
        threads = os.cpu_count() or 1
    lib.sbo_evaluate(dt, 1 if truth else 0, op, float(p), mode, _ptr(points), _ptr(offsets), nr,
                     _ptr(col_points), _ptr(col_offsets), nc, _ptr(out), int(threads))
    return out


def evaluate_rows(points, offsets, rows, *, op=OP_L1, p=1.0, mode=MODE_PDIST, truth=False, threads=None,
                  col_points=None, col_offsets=None, chunk=0, build="check"):
    """Evaluate only the listed rows.  Returns (values, row_starts) where row
    ``rows[k]``'s results occupy ``values[row_starts[k]:row_starts[k+1]]``
    (columns 0..i-1 for pdist, 0..i for the kernel, all for cdist).
    ``chunk`` > 0 hands the threads pieces of at most that many pairs of a
    row instead of whole rows (no idle threads behind a few long rows);
    ``build`` picks the library (see ``_load``)."""
    lib = _load(build)
    points, offsets = _csr(points, offsets)
    dt = _dtype_code(points)
    nr = len(offsets) - 1
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    if mode == MODE_CROSS:
        col_points, col_offsets = _csr(col_points, col_offsets)
        nc = len(col_offsets) - 1
        counts = np.full(len(rows), nc, dtype=np.uint64)
    else:
        col_points, col_offsets, nc = points, offsets, nr
        counts = rows + (1 if mode == MODE_KERNEL else 0)
    starts = np.zeros(len(rows) + 1, dtype=np.uint64)
    np.cumsum(counts, out=starts[1:])
    odt = np.float64 if truth else points.dtype
    out = np.zeros(int(starts[-1]), dtype=odt)
    if threads is None:
        threads = os.cpu_count() or 1
    base = np.ascontiguousarray(starts[:-1])
    lib.sbo_evaluate_rows_chunked(dt, 1 if truth else 0, op, float(p), mode, _ptr(points), _ptr(offsets), nr,
                                  _ptr(col_points), _ptr(col_offsets), nc, _ptr(rows), len(rows), _ptr(base),
                                  _ptr(out), int(threads), int(chunk))
    return out, starts


def pair(f, g, *, op=OP_L1, p=1.0, truth=False):
    """One finalized pair value; ``f``/``g`` are (L, 2) arrays of one dtype."""
    lib = _load()
    f = np.ascontiguousarray(f)
    g = np.ascontiguousarray(g)
    if truth:
        fn = lib.sbo_integrate_dd_f32 if f.dtype == np.float32 else lib.sbo_integrate_dd_f64
        pp = float(np.float32(p)) if f.dtype == np.float32 else float(p)
        return float(fn(_ptr(f), len(f), _ptr(g), len(g), op, pp))
    if f.dtype == np.float32:
        v = lib.sbo_integrate_f32(_ptr(f), len(f), _ptr(g), len(g), op, float(p))
        return float(np.float32(lib.sbo_finalize_f32(op, float(p), v)))
    v = lib.sbo_integrate_f64(_ptr(f), len(f), _ptr(g), len(g), op, float(p))
    return float(lib.sbo_finalize_f64(op, float(p), v))


def count_segments(points, offsets, mode=MODE_PDIST, col_points=None, col_offsets=None):
    """Rectangles the reference's merge emits over the whole problem
    (counted pair by pair; small problems only)."""
    lib = _load()
    points, offsets = _csr(points, offsets)
    if mode == MODE_CROSS:
        col_points, col_offsets = _csr(col_points, col_offsets)
        nc = len(col_offsets) - 1
    else:
        col_points, col_offsets, nc = points, offsets, len(offsets) - 1
    return int(lib.sbo_count_total_segments(_dtype_code(points), mode, _ptr(points), _ptr(offsets),
                                            len(offsets) - 1, _ptr(col_points), _ptr(col_offsets), nc))


# --- the reference's own code (where the reference tree is present) -----------

def ref_evaluate(points, offsets, *, op=OP_L1, p=1.0, mode=MODE_PDIST, col_points=None, col_offsets=None):
    lib = ref_lib()
    if lib is None:
        raise RuntimeError("reference harness unavailable (reference tree absent)")
    points, offsets = _csr(points, offsets)
    nr = len(offsets) - 1
    f32 = points.dtype == np.float32
    if mode == MODE_CROSS:
        col_points, col_offsets = _csr(col_points, col_offsets)
        nc = len(col_offsets) - 1
        out = np.zeros(nr * nc, dtype=points.dtype)
        fn = lib.sbref_cross_f32 if f32 else lib.sbref_cross_f64
        fn(_ptr(points), _ptr(offsets), nr, _ptr(col_points), _ptr(col_offsets), nc, op, float(p), _ptr(out))
        return out
    out = np.zeros(out_size(mode, nr), dtype=points.dtype)
    fn = lib.sbref_pairwise_f32 if f32 else lib.sbref_pairwise_f64
    if fn(_ptr(points), _ptr(offsets), nr, op, float(p), mode, _ptr(out)) != 0:
        raise ValueError("the reference container rejected a value")
    return out


def ref_rectangles(f, g, a=0.0, b=None):
    lib = ref_lib()
    if lib is None:
        raise RuntimeError("reference harness unavailable (reference tree absent)")
    f = np.ascontiguousarray(f, dtype=np.float64)
    g = np.ascontiguousarray(g, dtype=np.float64)
    if b is None:
        b = np.finfo(np.float64).max
    cap = 4 * (len(f) + len(g) + 4)
    out = np.zeros(4 * cap, dtype=np.float64)
    n = lib.sbref_rectangles_f64(_ptr(f), len(f), _ptr(g), len(g), float(a), float(b), _ptr(out), cap)
    return out[: 4 * n].reshape(n, 4)


def ref_schedule(n_rows, n_cols, max_out, n_splits, lower, min_side):
    lib = ref_lib()
    if lib is None:
        raise RuntimeError("reference harness unavailable (reference tree absent)")
    cap = 1 << 20
    out = np.zeros(5 * cap, dtype=np.uint64)
    mh = np.zeros(1, dtype=np.uint64)
    mw = np.zeros(1, dtype=np.uint64)
    n = lib.sbref_schedule(n_rows, n_cols, max_out, n_splits, 1 if lower else 0, min_side, _ptr(out), cap,
                           _ptr(mh), _ptr(mw))
    return out[: 5 * n].reshape(n, 5), int(mh[0]), int(mw[0])


def ref_subdivide(block, n_items):
    lib = ref_lib()
    if lib is None:
        raise RuntimeError("reference harness unavailable (reference tree absent)")
    cap = n_items + 4
    out = np.zeros(2 * cap, dtype=np.uint64)
    n = lib.sbref_subdivide(block, n_items, _ptr(out), cap)
    return out[: 2 * n].reshape(n, 2)


def ref_matrix_body(kind, n, storage):
    """Bytes the reference's ``write_element`` emits for a DistanceMatrix
    (kind 1) or SymmetricMatrix (kind 2) holding ``storage``
    (``include/sbear/io/compressed_matrix_io.hpp:10-20``)."""
    lib = ref_lib()
    storage = np.ascontiguousarray(storage)
    fn = lib.sbref_matrix_body_f32 if storage.dtype == np.float32 else lib.sbref_matrix_body_f64
    cap = 8 + storage.nbytes
    out = np.zeros(cap, np.uint8)
    nb = fn(kind, n, _ptr(storage), _ptr(out), cap)
    assert nb == cap, (nb, cap)
    return out.tobytes()


def lp_norm(points, offsets, p=1.0):
    """Lp norm of every PCF (the restatement of l1_norm / lp_norm)."""
    lib = _load()
    pts, off = _csr(points, offsets)
    n = len(off) - 1
    out = np.zeros(n, dtype=pts.dtype)
    lib.sbo_lp_norm(_dtype_code(pts), float(p), _ptr(pts), _ptr(off), n, _ptr(out))
    return out


def ref_lp_norm(points, offsets, p=1.0):
    """Lp norm of every PCF through the reference's own iterate_segments."""
    lib = ref_lib()
    pts, off = _csr(points, offsets)
    fn = lib.sbref_lp_norm_f32 if pts.dtype == np.float32 else lib.sbref_lp_norm_f64
    out = np.zeros(len(off) - 1, dtype=pts.dtype)
    for i in range(len(off) - 1):
        a, b = int(off[i]), int(off[i + 1])
        out[i] = fn(_ptr(pts[a:b]), b - a, p)
    return out


def barcodes_to_pcfs(bars, bar_offsets, kind):
    """Stable rank (kind 0) or Betti curve (kind 1) PCFs of a CSR of bars
    ((birth, death) rows), as (points, offsets): the restatement of the
    reference's per-barcode loops."""
    lib = _load()
    bars = np.ascontiguousarray(bars)
    boff = np.ascontiguousarray(bar_offsets, dtype=np.uint64)
    n = len(boff) - 1
    cap = (len(bars) if kind == 0 else 2 * len(bars)) + n
    out = np.zeros((max(cap, 1), 2), dtype=bars.dtype)
    ooff = np.zeros(n + 1, np.uint64)
    rc = lib.sbo_barcodes_to_pcfs(kind, _dtype_code(bars), _ptr(bars), _ptr(boff), n, _ptr(out), _ptr(ooff))
    assert rc == 0
    return out[: int(ooff[-1])], ooff


_ref_gpu = None


def ref_gpu_kernel_available():
    """Whether the reference's own CUDA block kernel (a cubin built where the
    reference tree is) and its driver-API harness are present; a reason
    string otherwise."""
    import json
    if not os.path.exists(_build.REF_CUBIN) or not os.path.exists(_build.REF_ENTRIES):
        return "no oracle/_ref/ref_kernels.cubin (it is built where the reference tree is present)"
    try:
        _build.build_ref_gpu_harness()
    except Exception as e:  # pragma: no cover
        return f"harness not built: {e}"
    with open(_build.REF_ENTRIES) as f:
        if not json.load(f):
            return "no kernel entries recorded"
    return True


def ref_gpu_triangle(dev_points_ptr, dev_offsets_ptr, n, *, op="l1", p=1.0, kernel=False, host_out=None,
                     max_output_elements=0, dtype=np.float32):
    """Run the reference's own CUDA block kernel over the pdist (or, with
    kernel=True, the L2-kernel) triangle of n PCFs of `dtype` (float32 or
    float64) whose CSR is on the current CUDA device (points (t, v) pairs and
    uint64 offsets, given as device addresses), tile by tile with the
    reference scheduler's parameters.  Returns (summed tile-kernel
    milliseconds, tiles).  With host_out (an array of `dtype` and the
    condensed size) the tiles are also scattered into it."""
    _ref_gpu_lib()
    dtype, entry = _ref_gpu_entry(op, kernel, dtype)
    ms = ctypes.c_double(0.0)
    tiles = ctypes.c_uint64(0)
    err = ctypes.create_string_buffer(512)
    hp = None
    if host_out is not None:
        assert host_out.dtype == dtype and host_out.flags["C_CONTIGUOUS"]
        assert host_out.size == out_size(MODE_KERNEL if kernel else MODE_PDIST, n)
        hp = _ptr(host_out)
    rc = _ref_gpu.sbref_gpu_triangle(_build.REF_CUBIN.encode(), entry.encode(), dtype.itemsize,
                                     2 if kernel else 1, float(p),
                                     int(dev_points_ptr), int(dev_offsets_ptr), int(n), hp, int(max_output_elements),
                                     ctypes.byref(ms), ctypes.byref(tiles), err, len(err))
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return ms.value, int(tiles.value)


def _ref_gpu_lib():
    global _ref_gpu
    ok = ref_gpu_kernel_available()
    if ok is not True:
        raise RuntimeError(ok)
    if _ref_gpu is None:
        lib = ctypes.CDLL(_build.build_ref_gpu_harness())
        lib.sbref_gpu_triangle.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double, _U64, _U64, _U64, _P, _U64,
                                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64),
                                           ctypes.c_char_p, ctypes.c_size_t]
        lib.sbref_gpu_triangle.restype = ctypes.c_int
        lib.sbref_gpu_triangle_rows.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_double, _U64, _U64, _U64, _P, _P, _U64, _P, _U64,
                                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64),
                                                ctypes.c_char_p, ctypes.c_size_t]
        lib.sbref_gpu_triangle_rows.restype = ctypes.c_int
        _ref_gpu = lib
    return _ref_gpu


def _ref_gpu_entry(op, kernel, dtype):
    import json
    with open(_build.REF_ENTRIES) as f:
        entries = json.load(f)
    dtype = np.dtype(dtype)
    if dtype not in (np.float32, np.float64):
        raise TypeError("float32 or float64 PCFs")
    key = ("inner" if kernel else op) + ("_f32" if dtype == np.float32 else "_f64")
    if key not in entries:
        raise ValueError(f"no reference kernel for {key}")
    return dtype, entries[key]


def ref_gpu_triangle_rows(dev_points_ptr, dev_offsets_ptr, n, rows, *, op="l1", p=1.0, kernel=False,
                          dtype=np.float32, max_output_elements=0):
    """As ref_gpu_triangle, copying back only the listed rows of the
    triangle.  Returns (summed tile-kernel milliseconds, tiles, values,
    row_starts) with row ``rows[k]``'s entries (columns 0..i-1 for pdist,
    0..i for the kernel) at ``values[row_starts[k]:row_starts[k+1]]``."""
    lib = _ref_gpu_lib()
    dtype, entry = _ref_gpu_entry(op, kernel, dtype)
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    counts = rows + (1 if kernel else 0)
    starts = np.zeros(len(rows) + 1, dtype=np.uint64)
    np.cumsum(counts, out=starts[1:])
    vals = np.full(int(starts[-1]), np.nan, dtype=dtype)
    base = np.ascontiguousarray(starts[:-1])
    ms = ctypes.c_double(0.0)
    tiles = ctypes.c_uint64(0)
    err = ctypes.create_string_buffer(512)
    rc = lib.sbref_gpu_triangle_rows(_build.REF_CUBIN.encode(), entry.encode(), dtype.itemsize, 2 if kernel else 1,
                                     float(p), int(dev_points_ptr), int(dev_offsets_ptr), int(n), _ptr(rows),
                                     _ptr(base), len(rows), _ptr(vals), int(max_output_elements), ctypes.byref(ms),
                                     ctypes.byref(tiles), err, len(err))
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return ms.value, int(tiles.value), vals, starts


def rectangles(f, g, a=0.0, b=float("inf")):
    """The reference's rectangle walk for one pair, restated as a plain loop
    (include/sbear/algorithms/functional/iterate_rectangles.hpp:23-104):
    both sides start at their last point at or before a (the first point if
    none); while t < b the side with the earlier next breakpoint advances
    (both on a tie), and each step emits (tprev, min(max(f.t, g.t), b),
    f value, g value); once both are exhausted the last rectangle runs to b.
    f, g: (n, 2) arrays of (t, v).  Returns an (m, 4) array."""
    f = np.asarray(f)
    g = np.asarray(g)

    def start(p):
        i = int(np.searchsorted(p[:, 0], a, side="right"))
        return 0 if i == 0 else i - 1

    fi, gi = start(f), start(g)
    t = tprev = a
    out = []
    while t < b:
        tprev = t
        fv, gv = f[fi, 1], g[gi, 1]
        fn, gn = fi + 1 < len(f), gi + 1 < len(g)
        if fn and gn:
            delta = f[fi + 1, 0] - g[gi + 1, 0]
            if delta <= 0:
                fi += 1
            if delta >= 0:
                gi += 1
        elif fn:
            fi += 1
        elif gn:
            gi += 1
        else:
            out.append((tprev, b, fv, gv))
            break
        t = min(max(f[fi, 0], g[gi, 0]), b)
        out.append((tprev, t, fv, gv))
    return np.array(out, dtype=np.float64).reshape(-1, 4)
