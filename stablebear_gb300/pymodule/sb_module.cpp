// _sb_gb300: the compiled Python binding of the pairwise-integration classes.
//
// The reference exposes its computations to Python as pybind11 classes
// (src/python/functional/py_distance.cpp:225-250: Distance_f32_f32 and
// Distance_f64_f64 with the statics pdist_l1, pdist_lp, cdist_l1, cdist_lp,
// lp_distance_l1, lp_distance_lp; src/python/functional/py_inner_product.cpp:71-90:
// InnerProduct_f32_f32 / _f64_f64 with l2), each returning (task, result),
// and the task class of src/python/pymodule.cpp:91-106 (wait_for,
// request_stop, work_total, work_completed, work_step, work_step_desc,
// work_step_unit).  This module is the same surface, in C++ over pybind11,
// calling the CUDA library through its C ABI (include/sbgpu.h): no CUDA code
// here and no torch types.  PCF arrays come in as any object with a
// ``csr()`` method returning (points (M, 2), offsets (N + 1,) uint64) and
// results go out as the package's DistanceMatrix / SymmetricMatrix (filled by
// the running task, as in the reference) or a numpy array for cdist.
//
// Errors map as the reference's pybind layer maps its C++ exceptions:
// invalid argument / input -> ValueError, allocation -> MemoryError,
// cancellation -> InterruptedError, CUDA and the rest -> RuntimeError.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "sbgpu.h"

namespace py = pybind11;

namespace
{
  void check(int status)
  {
    if (status == SBG_OK) return;
    const char* m = sbg_last_error();
    const std::string msg = (m && *m) ? m : "stablebear_gb300: native error " + std::to_string(status);
    switch (status)
    {
      case SBG_ERR_INVALID_ARGUMENT:
      case SBG_ERR_INVALID_INPUT:
        throw py::value_error(msg);
      case SBG_ERR_OUT_OF_MEMORY:
        PyErr_SetString(PyExc_MemoryError, msg.c_str());
        throw py::error_already_set();
      case SBG_ERR_CANCELLED:
        PyErr_SetString(PyExc_InterruptedError, msg.c_str());
        throw py::error_already_set();
      default:
        throw std::runtime_error(msg);
    }
  }

  void device_verbose(const char* what)
  {
    if (sbg_get_device_verbose()) py::print(what);
  }

  // StoppableTask_void: one native task (or none: a result that needed no
  // work), plus the Python objects its worker writes into.
  class Task
  {
  public:
    Task(sbg_task* h, py::object keep) : m_h(h), m_keep(std::move(keep)) { }
    Task(const Task&) = delete;
    Task& operator=(const Task&) = delete;
    ~Task()
    {
      if (m_h)
      {
        py::gil_scoped_release nogil;
        sbg_task_destroy(m_h);  // joins the worker
      }
    }

    bool wait_for(int64_t ms)
    {
      if (!m_h) return true;
      int fin = 0, st;
      {
        py::gil_scoped_release nogil;
        st = sbg_task_wait_for(m_h, ms, &fin);
      }
      check(st);
      return fin != 0;
    }
    void wait()
    {
      if (!m_h) return;
      int st;
      {
        py::gil_scoped_release nogil;
        st = sbg_task_wait(m_h);
      }
      check(st);
    }
    void request_stop()
    {
      if (m_h) sbg_task_request_stop(m_h);
    }
    bool stop_requested() const { return m_h && sbg_task_stop_requested(m_h); }
    uint64_t work_total() const { return progress(0); }
    uint64_t work_completed() const { return progress(1); }
    uint64_t work_step() const { return progress(2); }
    std::string work_step_desc() const { return text(0); }
    std::string work_step_unit() const { return text(1); }
    void close()
    {
      if (m_h)
      {
        sbg_task* h = m_h;
        m_h = nullptr;
        py::gil_scoped_release nogil;
        sbg_task_destroy(h);
      }
      m_keep = py::none();
    }

  private:
    uint64_t progress(int which) const
    {
      if (!m_h) return 0;
      uint64_t v[3] = {0, 0, 0};
      check(sbg_task_progress(m_h, &v[0], &v[1], &v[2]));
      return v[which];
    }
    std::string text(int which) const
    {
      if (!m_h) return "";
      char desc[256] = {0}, unit[64] = {0};
      check(sbg_task_step_text(m_h, desc, sizeof desc, unit, sizeof unit));
      return which == 0 ? desc : unit;
    }

    sbg_task* m_h;
    py::object m_keep;
  };

  // A task as a Python object (the class is move-less: it owns the native handle).
  py::object make_task(sbg_task* h, py::object keep)
  {
    return py::cast(new Task(h, std::move(keep)), py::return_value_policy::take_ownership);
  }

  template <typename T>
  using Arr = py::array_t<T, py::array::c_style | py::array::forcecast>;

  template <typename T>
  struct Csr
  {
    Arr<T> points;
    Arr<uint64_t> offsets;
    uint64_t n = 0;
  };

  template <typename T>
  Csr<T> csr_of(const py::object& X)
  {
    py::tuple c = X.attr("csr")();
    Csr<T> r{Arr<T>(c[0]), Arr<uint64_t>(c[1]), 0};
    if (r.offsets.ndim() != 1 || r.offsets.shape(0) < 1) throw py::value_error("offsets must be a 1-D array of N + 1");
    r.n = (uint64_t)r.offsets.shape(0) - 1;
    return r;
  }

  py::object matrices(const char* name) { return py::module_::import("stablebear_gb300.matrices").attr(name); }

  // The matrix's own condensed storage, never a converted copy: the task
  // writes into it after this call returns.
  template <typename T>
  py::array_t<T, py::array::c_style> storage_of(const py::object& matrix)
  {
    py::object a = matrix.attr("data");
    if (!py::isinstance<py::array_t<T, py::array::c_style>>(a))
      throw std::runtime_error("matrix storage is not a contiguous array of the PCF type");
    return a.cast<py::array_t<T, py::array::c_style>>();
  }

  template <typename T, int DT>
  struct Distance
  {
    static py::tuple pdist(const py::object& X, int op, double p)
    {
      if (op == SBG_OP_LP && !(p >= 1.0)) throw py::value_error("p must be >= 1.");
      Csr<T> c = csr_of<T>(X);
      py::object dm = matrices("DistanceMatrix")(c.n, py::dtype::of<T>());
      if (c.n < 2) return py::make_tuple(make_task(nullptr, py::none()), dm);
      device_verbose("Integral computation on CUDA device(s)");
      auto data = storage_of<T>(dm);
      sbg_task* h = nullptr;
      check(sbg_create_integrate_task(DT, op, p, SBG_SKIP_LOWER_NODIAG, c.points.data(), c.offsets.data(), c.n,
                                      data.mutable_data(), &h));
      py::object t = make_task(h, data);
      check(sbg_task_start(h));
      return py::make_tuple(t, dm);
    }

    static py::tuple cdist(const py::object& X, const py::object& Y, int op, double p)
    {
      if (op == SBG_OP_LP && !(p >= 1.0)) throw py::value_error("p must be >= 1.");
      Csr<T> cx = csr_of<T>(X), cy = csr_of<T>(Y);
      std::vector<py::ssize_t> shape;
      for (auto s : py::tuple(X.attr("shape"))) shape.push_back(s.cast<py::ssize_t>());
      for (auto s : py::tuple(Y.attr("shape"))) shape.push_back(s.cast<py::ssize_t>());
      Arr<T> out(shape);
      std::fill(out.mutable_data(), out.mutable_data() + out.size(), T(0));
      if (cx.n == 0 || cy.n == 0) return py::make_tuple(make_task(nullptr, py::none()), out);
      device_verbose("Cross-distance computation on CUDA device(s)");
      sbg_task* h = nullptr;
      check(sbg_create_cdist_task(DT, op, p, cx.points.data(), cx.offsets.data(), cx.n, cy.points.data(),
                                  cy.offsets.data(), cy.n, out.mutable_data(), &h));
      py::object t = make_task(h, out);
      check(sbg_task_start(h));
      return py::make_tuple(t, out);
    }

    static T pair(const py::object& f, const py::object& g, int op, double p)
    {
      if (op == SBG_OP_LP && !(p >= 1.0)) throw py::value_error("p must be >= 1.");
      Arr<T> fp = Arr<T>::ensure(f.attr("_pts")), gp = Arr<T>::ensure(g.attr("_pts"));
      if (!fp || !gp || fp.ndim() != 2 || gp.ndim() != 2) throw py::value_error("f and g must be PCFs of (t, v) points");
      const uint64_t fo[2] = {0, (uint64_t)fp.shape(0)}, go[2] = {0, (uint64_t)gp.shape(0)};
      T out = T(0);
      check(sbg_pairwise_host(DT, op, p, SBG_SKIP_NONE, fp.data(), fo, 1, gp.data(), go, 1, &out, 1));
      return out;
    }
  };

  template <typename T, int DT>
  struct InnerProduct
  {
    static py::tuple l2(const py::object& X)
    {
      Csr<T> c = csr_of<T>(X);
      py::object sm = matrices("SymmetricMatrix")(c.n, py::dtype::of<T>());
      if (c.n == 0) return py::make_tuple(make_task(nullptr, py::none()), sm);
      device_verbose("Kernel computation on CUDA device(s)");
      auto data = storage_of<T>(sm);
      sbg_task* h = nullptr;
      check(sbg_create_integrate_task(DT, SBG_OP_L2_INNER, 1.0, SBG_SKIP_LOWER, c.points.data(), c.offsets.data(),
                                      c.n, data.mutable_data(), &h));
      py::object t = make_task(h, data);
      check(sbg_task_start(h));
      return py::make_tuple(t, sm);
    }
  };

  template <typename T, int DT>
  void bind_distance(py::module_& m, const char* name)
  {
    using D = Distance<T, DT>;
    py::class_<D>(m, name)
        .def_static("pdist_l1", [](const py::object& X) { return D::pdist(X, SBG_OP_L1, 1.0); })
        .def_static("pdist_lp", [](const py::object& X, double p) { return D::pdist(X, SBG_OP_LP, p); })
        .def_static("cdist_l1", [](const py::object& X, const py::object& Y) { return D::cdist(X, Y, SBG_OP_L1, 1.0); })
        .def_static("cdist_lp",
                    [](const py::object& X, const py::object& Y, double p) { return D::cdist(X, Y, SBG_OP_LP, p); })
        .def_static("lp_distance_l1", [](const py::object& f, const py::object& g) { return D::pair(f, g, SBG_OP_L1, 1.0); })
        .def_static("lp_distance_lp",
                    [](const py::object& f, const py::object& g, double p) { return D::pair(f, g, SBG_OP_LP, p); });
  }

  template <typename T, int DT>
  void bind_inner(py::module_& m, const char* name)
  {
    using I = InnerProduct<T, DT>;
    py::class_<I>(m, name).def_static("l2", [](const py::object& X) { return I::l2(X); });
  }
}

PYBIND11_MODULE(_sb_gb300, m)
{
  m.doc() = "stablebear_gb300 compiled binding: Distance_* / InnerProduct_* over the CUDA library's C ABI";
  py::class_<Task>(m, "StoppableTask_void")
      .def("wait_for", &Task::wait_for, py::arg("ms"))
      .def("wait", &Task::wait)
      .def("request_stop", &Task::request_stop)
      .def("stop_requested", &Task::stop_requested)
      .def("work_total", &Task::work_total)
      .def("work_completed", &Task::work_completed)
      .def("work_step", &Task::work_step)
      .def("work_step_desc", &Task::work_step_desc)
      .def("work_step_unit", &Task::work_step_unit)
      .def("close", &Task::close);
  bind_distance<float, SBG_F32>(m, "Distance_f32_f32");
  bind_distance<double, SBG_F64>(m, "Distance_f64_f64");
  bind_inner<float, SBG_F32>(m, "InnerProduct_f32_f32");
  bind_inner<double, SBG_F64>(m, "InnerProduct_f64_f64");
  m.def("_build_type", [] { return std::string(sbg_build_type()); });
}
