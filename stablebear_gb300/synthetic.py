"""Seeded synthetic PCF workloads (numpy PCG64), in the reference's CSR.

The pairwise path has no public dataset; these generators reproduce the
shapes, sizes and value distributions of the workloads the benchmarks and
parity tests use:

* ``gaussian``      — L from a given sampler, t_0 = 0, t_k = t_{k-1} + Exp(1),
                      v ~ N(0, 1), last value 0 (the plain pdist / kernel /
                      differentiation workloads).
* ``stable_rank``   — L = round(exp(U[ln 16, ln 4096])), Exp(1) gaps, integer
                      values: v_0 ~ U{1..500}, v_k = max(v_{k-1} - G_k, 0) with
                      G_k ~ Geometric(0.3) on {1, 2, ...}, last value 0.  Values
                      reach 0 long before L for long PCFs; the generator
                      follows that recipe literally.
* ``betti``         — integer values from a reflected walk v_k = |v_{k-1} + xi|,
                      xi = +-1, v_0 ~ U{0..10}, last value 0, Exp(1) gaps
                      (generated as |v_0 + xi_1 + ... + xi_k|, the same law).

Times are generated in float64 and cast to the target type; a time that
collides with its predecessor after the cast is moved up by one ulp, so every
PCF has strictly increasing times.
"""
from __future__ import annotations

import numpy as np


def _times(rng, lens: np.ndarray, dtype) -> np.ndarray:
    total = int(lens.sum())
    gaps = rng.exponential(1.0, size=total)
    starts = np.zeros(len(lens), dtype=np.int64)
    np.cumsum(lens[:-1], out=starts[1:])
    gaps[starts] = 0.0
    t = np.cumsum(gaps)
    base = np.repeat(t[starts], lens)
    t = (t - base).astype(dtype)
    t[starts] = 0
    # strictly increasing within each PCF after the cast
    first = np.zeros(total, dtype=bool)
    first[starts] = True
    for _ in range(64):
        bad = np.zeros(total, dtype=bool)
        bad[1:] = (t[1:] <= t[:-1]) & ~first[1:]
        if not bad.any():
            break
        idx = np.nonzero(bad)[0]
        t[idx] = np.nextafter(t[idx - 1], np.array(np.inf, dtype=dtype))
    return t


def _pack(t: np.ndarray, v: np.ndarray, lens: np.ndarray, dtype):
    pts = np.empty((len(t), 2), dtype=dtype)
    pts[:, 0] = t
    pts[:, 1] = v
    off = np.zeros(len(lens) + 1, dtype=np.uint64)
    np.cumsum(lens, out=off[1:])
    return pts, off


def _last_index(lens: np.ndarray) -> np.ndarray:
    return np.cumsum(lens) - 1


def gaussian(n: int, lengths, dtype=np.float32, seed: int = 0):
    """``lengths``: an int array of breakpoint counts, or a callable
    ``(rng, n) -> lengths``."""
    rng = np.random.default_rng(seed)
    lens = np.asarray(lengths(rng, n) if callable(lengths) else lengths, dtype=np.int64)
    t = _times(rng, lens, dtype)
    v = rng.standard_normal(int(lens.sum()))
    v[_last_index(lens)] = 0.0
    return _pack(t, v.astype(dtype), lens, dtype)


def stable_rank(n: int, dtype=np.float64, seed: int = 0):
    rng = np.random.default_rng(seed)
    lens = np.rint(np.exp(rng.uniform(np.log(16), np.log(4096), size=n))).astype(np.int64)
    t = _times(rng, lens, dtype)
    total = int(lens.sum())
    starts = np.zeros(n, dtype=np.int64)
    np.cumsum(lens[:-1], out=starts[1:])
    dec = rng.geometric(0.3, size=total).astype(np.float64)
    dec[starts] = 0.0
    v0 = rng.integers(1, 501, size=n).astype(np.float64)
    # v_k = max(v0 - sum of decrements, 0): cumulative sum per PCF
    cs = np.cumsum(dec)
    cs -= np.repeat(cs[starts], lens)
    v = np.maximum(np.repeat(v0, lens) - cs, 0.0)
    v[_last_index(lens)] = 0.0
    return _pack(t, v.astype(dtype), lens, dtype)


def betti(n: int, lengths, dtype=np.float32, seed: int = 0):
    rng = np.random.default_rng(seed)
    lens = np.asarray(lengths(rng, n) if callable(lengths) else lengths, dtype=np.int64)
    t = _times(rng, lens, dtype)
    total = int(lens.sum())
    starts = np.zeros(n, dtype=np.int64)
    np.cumsum(lens[:-1], out=starts[1:])
    xi = rng.choice(np.array([-1.0, 1.0]), size=total)
    v0 = rng.integers(0, 11, size=n).astype(np.float64)
    xi[starts] = 0.0
    # The reflected walk R_k = |R_{k-1} + xi_k| from an integer v_0 >= 0 is the
    # Markov chain (0 -> 1; x -> x +- 1 with probability 1/2 each), which is
    # exactly the law of |S_k| for the free walk S_k = v_0 + xi_1 + ... + xi_k;
    # |S_k| is generated here without a per-point loop.
    s = np.cumsum(xi)
    s -= np.repeat(s[starts], lens)
    v = np.abs(np.repeat(v0, lens) + s)
    v[_last_index(lens)] = 0.0
    return _pack(t, v.astype(dtype), lens, dtype)


# --- the benchmark workloads ----------------------------------------------------

def uniform_lengths(lo: int, hi: int):
    return lambda rng, n: rng.integers(lo, hi + 1, size=n)


def poisson_lengths(lam: float, plus: int):
    return lambda rng, n: rng.poisson(lam, size=n) + plus


def plain_l1(n: int = 1000, seed: int = 0):
    """N PCFs, L ~ U{10..200}, float32."""
    return gaussian(n, uniform_lengths(10, 200), np.float32, seed)


def large_l1(n: int = 100_000, seed: int = 0):
    """N PCFs, L ~ Poisson(256) + 2, float32."""
    return gaussian(n, poisson_lengths(256.0, 2), np.float32, seed)


def differentiation(n: int = 4096, seed: int = 0):
    """N PCFs, L ~ U{16..512}, float32."""
    return gaussian(n, uniform_lengths(16, 512), np.float32, seed)


def batched_betti(n_problems: int = 512, seed: int = 0, n_range=(50, 2000), l_range=(8, 1024)):
    """Independent problems with N_i ~ U{n_range}, L ~ U{l_range}, Betti-like
    float32 values; returns a list of (points, offsets)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_range[0], n_range[1] + 1, size=n_problems)
    return [betti(int(n), uniform_lengths(*l_range), np.float32, seed * 100003 + k + 1) for k, n in enumerate(ns)]


def segment_count(offsets: np.ndarray, points: np.ndarray, mode: int = 1) -> int:
    """Merged rectangles of a pdist (mode 1) or l2 kernel (mode 2) problem:
    sum over pairs of |T_i U T_j| = (N - 1) sum L - sum_tau C(m_tau, 2), where
    m_tau counts PCFs with a breakpoint at tau (all N share tau = 0).  The
    kernel adds sum L for the diagonal.  Assumes strictly increasing times
    within each PCF (true for the generators above)."""
    lens = np.diff(offsets.astype(np.int64))
    n = len(lens)
    total_l = int(lens.sum())
    t = points[:, 0]
    _, counts = np.unique(t, return_counts=True)
    ties = int((counts.astype(np.int64) * (counts.astype(np.int64) - 1) // 2).sum())
    s = (n - 1) * total_l - ties
    if mode == 2:
        s += total_l
    return int(s)
