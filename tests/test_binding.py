"""The compiled pybind11 binding builds, loads and exposes the reference's
classes (no GPU needed: only argument checks and empty problems run here)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def mod():
    from stablebear_gb300 import build, _binding
    build.build()
    if build.pybind11_include() is None:
        pytest.skip("no pybind11 headers on this machine (the ctypes binding serves the API)")
    m = _binding.compiled()
    assert m is not None
    return m


def test_classes_and_task_surface(mod):
    for cls, names in (("Distance_f32_f32", ["pdist_l1", "pdist_lp", "cdist_l1", "cdist_lp", "lp_distance_l1",
                                             "lp_distance_lp"]),
                       ("Distance_f64_f64", ["pdist_l1", "pdist_lp", "cdist_l1", "cdist_lp", "lp_distance_l1",
                                             "lp_distance_lp"]),
                       ("InnerProduct_f32_f32", ["l2"]), ("InnerProduct_f64_f64", ["l2"])):
        for n in names:
            assert callable(getattr(getattr(mod, cls), n)), f"{cls}.{n}"
    for n in ("wait_for", "wait", "request_stop", "stop_requested", "work_total", "work_completed", "work_step",
              "work_step_desc", "work_step_unit", "close"):
        assert hasattr(mod.StoppableTask_void, n)
    assert mod._build_type() == "CUDA"


def test_public_classes_are_the_compiled_ones(mod):
    from stablebear_gb300 import distance, _binding
    assert _binding.name() == "pybind11"
    assert distance.Distance_f32_f32 is mod.Distance_f32_f32
    assert distance.InnerProduct_f64_f64 is mod.InnerProduct_f64_f64


def test_argument_errors_and_empty_problems(mod):
    import stablebear_gb300 as sb
    X = sb.zeros((1,))
    with pytest.raises(ValueError, match="p must be >= 1"):
        mod.Distance_f32_f32.pdist_lp(X, 0.5)
    with pytest.raises(ValueError, match="p must be >= 1"):
        mod.Distance_f32_f32.cdist_lp(X, X, 0.0)
    task, dm = mod.Distance_f32_f32.pdist_l1(X)       # one PCF: nothing to compute
    assert task.wait_for(0) and dm.size == 1 and dm.data.size == 0
    task.close()
    task, sm = mod.InnerProduct_f64_f64.l2(sb.zeros((0,), dtype=sb.pcf64))
    assert task.wait_for(0) and sm.size == 0
    task, out = mod.Distance_f64_f64.cdist_l1(sb.zeros((0,), dtype=sb.pcf64), sb.zeros((3,), dtype=sb.pcf64))
    assert task.wait_for(0) and out.shape == (0, 3) and out.dtype == np.float64
