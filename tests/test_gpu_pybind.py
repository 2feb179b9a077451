"""The compiled pybind11 binding (_sb_gb300): the reference's classes
Distance_f32_f32 / Distance_f64_f64 / InnerProduct_f32_f32 / _f64_f64
(src/python/functional/py_distance.cpp:225-250, py_inner_product.cpp:71-90)
as C++ over the C ABI, checked against the values the reference's own code
produced (tests/golden/reference_pairwise.npz) and against the ctypes
binding, which must give the same bits (both call the same library).
Tolerances as in test_gpu_parity.py: float32 1e-5 (general p 1e-4), float64
1e-12 (general p 1e-10), the L2 kernel against max(|ref|, 1).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f32": 1e-5, "f64": 1e-12}
TOL_LP = {"f32": 1e-4, "f64": 1e-10}


@pytest.fixture(scope="module")
def mod():
    from stablebear_gb300 import build, _binding
    build.build()
    m = _binding.compiled()
    assert m is not None, "the pybind11 binding was not built (see build.build_pymodule)"
    return m


def rel(got, want, floor=1e-30):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), floor))) if want.size else 0.0


def _done(task_result):
    task, res = task_result
    task.wait()
    assert task.wait_for(0)
    task.close()
    return res


@pytest.mark.parametrize("case", ["ragged", "tails", "ties"])
def test_compiled_classes_match_reference_golden(mod, golden_pairwise, tag, case):
    import stablebear_gb300 as sb
    g = golden_pairwise
    name = f"{case}_{tag}"
    X = sb.PcfArray.from_csr(g[f"{name}__points"], g[f"{name}__offsets"])
    Y = sb.PcfArray.from_csr(g[f"cols_{tag}__points"], g[f"cols_{tag}__offsets"])
    D = mod.Distance_f32_f32 if tag == "f32" else mod.Distance_f64_f64
    K = mod.InnerProduct_f32_f32 if tag == "f32" else mod.InnerProduct_f64_f64
    assert rel(_done(D.pdist_l1(X)).data, g[f"{name}__pdist_l1"]) <= TOL[tag]
    assert rel(_done(D.pdist_lp(X, 2.0)).data, g[f"{name}__pdist_l2"]) <= TOL[tag]
    assert rel(_done(D.pdist_lp(X, 3.0)).data, g[f"{name}__pdist_l3"]) <= TOL_LP[tag]
    assert rel(_done(K.l2(X)).data, g[f"{name}__kernel"], floor=1.0) <= TOL[tag]
    assert rel(_done(D.cdist_l1(X, Y)).reshape(-1), g[f"{name}__cdist_l1"]) <= TOL[tag]
    assert rel(_done(D.cdist_lp(X, Y, 1.5)).reshape(-1), g[f"{name}__cdist_l15"]) <= TOL_LP[tag]


def test_compiled_and_ctypes_bindings_agree(mod):
    import stablebear_gb300 as sb
    from stablebear_gb300 import distance, synthetic
    pts, off = synthetic.plain_l1(400, seed=12)
    X = sb.PcfArray.from_csr(pts, off)
    ct = distance.CTYPES_BACKENDS
    for name, call in (("pdist_l1", lambda C: C.pdist_l1(X)), ("pdist_lp", lambda C: C.pdist_lp(X, 2.5))):
        a = _done(call(mod.Distance_f32_f32)).data
        b = _done(call(ct["Distance_f32_f32"])).data
        np.testing.assert_array_equal(a, b, err_msg=name)
    np.testing.assert_array_equal(_done(mod.InnerProduct_f32_f32.l2(X)).data,
                                  _done(ct["InnerProduct_f32_f32"].l2(X)).data)
    f, g = X[3], X[7]
    assert mod.Distance_f32_f32.lp_distance_l1(f, g) == ct["Distance_f32_f32"].lp_distance_l1(f, g)
    assert mod.Distance_f32_f32.lp_distance_lp(f, g, 2.0) == ct["Distance_f32_f32"].lp_distance_lp(f, g, 2.0)
    # the package's public functions use the compiled classes
    assert distance.Distance_f32_f32 is mod.Distance_f32_f32
    np.testing.assert_array_equal(sb.pdist(X).data, _done(mod.Distance_f32_f32.pdist_l1(X)).data)


def test_compiled_task_api(mod):
    """The reference's task surface (src/python/pymodule.cpp:91-106): progress,
    step text, stop; errors surface once, as Python exceptions."""
    import stablebear_gb300 as sb
    from stablebear_gb300 import synthetic
    pts, off = synthetic.plain_l1(1500, seed=13)
    X = sb.PcfArray.from_csr(pts, off)
    task, dm = mod.Distance_f32_f32.pdist_l1(X)
    while not task.wait_for(50):
        pass
    assert task.work_completed() == task.work_total() == 1500 * 1499 // 2
    assert task.work_step() >= 1 and task.work_step_unit() == "integral"
    assert "lower triangle" in task.work_step_desc()
    assert not task.stop_requested()
    task.close()
    with pytest.raises(ValueError, match="p must be >= 1"):
        mod.Distance_f32_f32.pdist_lp(X, 0.5)
    sb.set_tuning(band_bytes=256 << 10)
    try:
        big = sb.PcfArray.from_csr(*synthetic.plain_l1(6000, seed=14))
        task, dm = mod.Distance_f32_f32.pdist_l1(big)
        task.request_stop()
        with pytest.raises(InterruptedError):
            task.wait()
        assert task.stop_requested() and task.work_completed() < task.work_total()
        task.wait()  # once
        task.close()
    finally:
        sb.set_tuning()
