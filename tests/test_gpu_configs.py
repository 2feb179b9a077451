"""Parity on the benchmark configurations' own input shapes, at the bounds the
contract states: float32 within 1e-5 relative, float64 within 1e-12 of the
reference's CPU algorithm (the naive in-order sum of
include/sbear/algorithms/functional/matrix_integrate.hpp:18-29, restated by
the oracle), and the error against the double-double truth printed beside.

* Plain: L1 pdist of exactly N = 1000 float32 PCFs, L ~ U{10..200}, N(0,1)
  values with the last value 0, Exp(1) gaps, seed 0 (the CPU-runnable case).
* Stable rank: float64 "stable-rank-like" PCFs, L = round(exp(U[ln 16,
  ln 4096])), non-increasing integer values, at N = 1500 (the workload is
  N = 20,000); the automatic kernel for PCFs this long in float64 is the
  hybrid one (columns in shared memory, rows through L1).  L2 kernel and L2
  pdist.

The batched, differentiation and large configurations have their own tests
(test_gpu_batch.py, test_gpu_autograd.py, test_gpu_full_size.py).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def native():
    from stablebear_gb300 import build
    build.build()


def rel(got, want, floor):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), floor)))


def test_plain_config_n1000_l1_float32():
    import stablebear_gb300 as sb
    from oracle import oracle as orc
    from stablebear_gb300 import synthetic
    pts, off = synthetic.plain_l1(1000, seed=0)
    lens = np.diff(off.astype(np.int64))
    assert len(lens) == 1000 and lens.min() >= 10 and lens.max() <= 200
    D = sb.pdist(sb.PcfArray.from_csr(pts, off))
    assert D.data.dtype == np.float32 and D.data.size == 499_500
    ref = orc.evaluate(pts, off)                 # the reference's CPU algorithm
    truth = orc.evaluate(pts, off, truth=True)   # double-double
    e_ref, e_truth = rel(D.data, ref, 1e-30), rel(D.data, truth, 1e-30)
    print(f"plain N=1000 L1 f32: vs reference CPU {e_ref:.2e}, vs truth {e_truth:.2e}, "
          f"reference CPU vs truth {rel(ref, truth, 1e-30):.2e}")
    assert e_ref <= 1e-5 and e_truth <= 1e-5


@pytest.mark.parametrize("what", ["l2_kernel", "l2_pdist"])
def test_stable_rank_config_float64(what):
    import stablebear_gb300 as sb
    from oracle import oracle as orc
    from stablebear_gb300 import synthetic
    pts, off = synthetic.stable_rank(1500, seed=0)
    lens = np.diff(off.astype(np.int64))
    assert pts.dtype == np.float64 and lens.max() > 2000  # long enough for the hybrid kernel
    v = pts[:, 1]
    assert np.all(v == np.rint(v)) and np.all(v >= 0)
    X = sb.PcfArray.from_csr(pts, off)
    if what == "l2_kernel":
        got = sb.l2_kernel(X).data
        kw, floor = dict(op=orc.OP_L2, mode=orc.MODE_KERNEL), 1.0
    else:
        got = sb.pdist(X, p=2).data
        kw, floor = dict(op=orc.OP_LP, p=2.0), 1e-300
    ref = orc.evaluate(pts, off, **kw)
    truth = orc.evaluate(pts, off, truth=True, **kw)
    e_ref, e_truth = rel(got, ref, floor), rel(got, truth, floor)
    print(f"stable rank N=1500 {what} f64: vs reference CPU {e_ref:.2e}, vs truth {e_truth:.2e}, "
          f"reference CPU vs truth {rel(ref, truth, floor):.2e}")
    assert e_ref <= 1e-12 and e_truth <= 1e-12
