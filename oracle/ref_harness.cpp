// ORACLE — test infrastructure only.
//
// Drives the stablebear reference's own, unmodified, taskflow-free headers so
// that the C restatement in pcf_oracle.c (and the CUDA path through it) can be
// pinned to the reference's actual code:
//   sbear/algorithms/functional/iterate_rectangles.hpp  (the merge)
//   sbear/functional/operations.cuh                     (the pair operations)
//   sbear/distance_matrix.hpp, sbear/symmetric_matrix.hpp (storage order)
//   sbear/cuda/cuda_block_scheduler.hpp, sbear/algorithms/subdivide.hpp
//   sbear/cuda/offset_data_manager.hpp
//   sbear/io/compressed_matrix_io.hpp                   (matrix body on disk)
// The 5-line integrate() body (matrix_integrate.hpp:18-29) and compute_row()
// (matrix_integrate.hpp:80-90) are restated here, because matrix_integrate.hpp
// itself pulls in taskflow, which the reference does not vendor.
//
// Built only where the reference tree is present, by oracle/build_oracle.py,
// into oracle/_ref/libsbref.so.  Never linked into the product.
// time_point.hpp first: iterate_rectangles.hpp uses sb::infinity from it
// (the reference includes it through pcf.hpp).
#include <sbear/functional/time_point.hpp>
#include <sbear/algorithms/functional/iterate_rectangles.hpp>
#include <sbear/functional/operations.cuh>
#include <sbear/distance_matrix.hpp>
#include <sbear/symmetric_matrix.hpp>
#include <sbear/cuda/cuda_block_scheduler.hpp>
#include <sbear/algorithms/subdivide.hpp>
#include <sbear/cuda/offset_data_manager.hpp>
#include <sbear/io/compressed_matrix_io.hpp>

#include <cmath>
#include <cstdint>
#include <sstream>
#include <cstring>
#include <stdexcept>
#include <limits>
#include <vector>

namespace
{
  template <typename T>
  std::vector<sb::TimePoint<T, T>> to_points(const T* pts, uint64_t n)
  {
    std::vector<sb::TimePoint<T, T>> out;
    out.reserve(n);
    for (uint64_t k = 0; k < n; ++k)
      out.emplace_back(pts[2 * k], pts[2 * k + 1]);
    return out;
  }

  // matrix_integrate.hpp:18-29, with the reference's iterate_rectangles.
  template <typename T, typename Op>
  T integrate(const std::vector<sb::TimePoint<T, T>>& f, const std::vector<sb::TimePoint<T, T>>& g, Op op)
  {
    T val = T(0);
    sb::iterate_rectangles(f, g, [&val, &op](const sb::Rectangle<T, T>& rect) {
      val += (rect.right - rect.left) * op(rect.f_value, rect.g_value);
    }, T(0), std::numeric_limits<T>::max());
    return val;
  }

  template <typename T>
  T pair_value(const std::vector<sb::TimePoint<T, T>>& f, const std::vector<sb::TimePoint<T, T>>& g, int op, T p)
  {
    if (op == 0) { sb::OperationL1Dist<T, T> o; return o(integrate(f, g, o)); }
    if (op == 1) { sb::OperationLpDist<T, T> o(p); return o(integrate(f, g, o)); }
    sb::OperationL2InnerProduct<T, T> o;
    return o(integrate(f, g, o));
  }

  template <typename T>
  std::vector<std::vector<sb::TimePoint<T, T>>> to_pcfs(const T* pts, const uint64_t* off, uint64_t n)
  {
    std::vector<std::vector<sb::TimePoint<T, T>>> v;
    v.reserve(n);
    for (uint64_t i = 0; i < n; ++i)
      v.push_back(to_points(pts + 2 * off[i], off[i + 1] - off[i]));
    return v;
  }

  // compute_row() (matrix_integrate.hpp:80-90) into the reference's own
  // DistanceMatrix (mode 1) / SymmetricMatrix (mode 2) containers; the
  // condensed storage is then copied out verbatim.
  template <typename T>
  int pairwise(const T* pts, const uint64_t* off, uint64_t n, int op, T p, int mode, T* out)
  {
    auto fs = to_pcfs(pts, off, n);
    if (mode == 1)
    {
      sb::DistanceMatrix<T> m(n);
      for (size_t i = 0; i < n; ++i)
        for (size_t j = i + 1; j < n; ++j)
          m(i, j) = pair_value(fs[i], fs[j], op, p);
      std::memcpy(out, m.data(), sizeof(T) * m.storage_count());
      return 0;
    }
    sb::SymmetricMatrix<T> m(n);
    for (size_t i = 0; i < n; ++i)
      for (size_t j = i; j < n; ++j)
        m(i, j) = pair_value(fs[i], fs[j], op, p);
    std::memcpy(out, m.data(), sizeof(T) * m.storage_count());
    return 0;
  }

  template <typename T>
  int cross(const T* rp, const uint64_t* ro, uint64_t nr, const T* cp, const uint64_t* co, uint64_t nc,
            int op, T p, T* out)
  {
    auto rs = to_pcfs(rp, ro, nr);
    auto cs = to_pcfs(cp, co, nc);
    for (size_t i = 0; i < nr; ++i)
      for (size_t j = 0; j < nc; ++j)
        out[i * nc + j] = pair_value(rs[i], cs[j], op, p);
    return 0;
  }
  // The body the reference writes for a DistanceMatrix (kind 1) or
  // SymmetricMatrix (kind 2) (compressed_matrix_io.hpp:10-20), filled through
  // the containers' public element access.
  template <typename T>
  uint64_t matrix_body(int kind, uint64_t n, const T* storage, unsigned char* out, uint64_t cap)
  {
    std::ostringstream os;
    if (kind == 1)
    {
      sb::DistanceMatrix<T> m(n);
      for (uint64_t i = 1; i < n; ++i)
        for (uint64_t j = 0; j < i; ++j)
          m(i, j) = storage[i * (i - 1) / 2 + j];
      sb::io::detail::write_element(os, m);
    }
    else
    {
      sb::SymmetricMatrix<T> m(n);
      for (uint64_t i = 0; i < n; ++i)
        for (uint64_t j = 0; j <= i; ++j)
          m(i, j) = storage[i * (i + 1) / 2 + j];
      sb::io::detail::write_element(os, m);
    }
    const std::string b = os.str();
    std::memcpy(out, b.data(), b.size() < cap ? b.size() : cap);
    return b.size();
  }
}

extern "C"
{
  float sbref_pair_f32(const float* f, uint64_t lf, const float* g, uint64_t lg, int op, float p)
  { return pair_value(to_points(f, lf), to_points(g, lg), op, p); }

  double sbref_pair_f64(const double* f, uint64_t lf, const double* g, uint64_t lg, int op, double p)
  { return pair_value(to_points(f, lf), to_points(g, lg), op, p); }

  // Returns -1 when the reference container rejects a value (e.g. a negative
  // entry written into a DistanceMatrix, distance_matrix.hpp:45-57).
  int sbref_pairwise_f32(const float* pts, const uint64_t* off, uint64_t n, int op, float p, int mode, float* out)
  {
    try { return pairwise(pts, off, n, op, p, mode, out); } catch (const std::exception&) { return -1; }
  }

  int sbref_pairwise_f64(const double* pts, const uint64_t* off, uint64_t n, int op, double p, int mode, double* out)
  {
    try { return pairwise(pts, off, n, op, p, mode, out); } catch (const std::exception&) { return -1; }
  }

  int sbref_cross_f32(const float* rp, const uint64_t* ro, uint64_t nr, const float* cp, const uint64_t* co,
                      uint64_t nc, int op, float p, float* out)
  { return cross(rp, ro, nr, cp, co, nc, op, p, out); }

  int sbref_cross_f64(const double* rp, const uint64_t* ro, uint64_t nr, const double* cp, const uint64_t* co,
                      uint64_t nc, int op, double p, double* out)
  { return cross(rp, ro, nr, cp, co, nc, op, p, out); }

  // Rectangles of one pair as (left, right, f, g) quadruples in double.
  // Returns the count; writes at most cap quadruples.
  uint64_t sbref_rectangles_f64(const double* f, uint64_t lf, const double* g, uint64_t lg,
                                double a, double b, double* out, uint64_t cap)
  {
    uint64_t n = 0;
    sb::iterate_rectangles(to_points(f, lf), to_points(g, lg), [&](const sb::Rectangle<double, double>& r) {
      if (n < cap) { out[4 * n] = r.left; out[4 * n + 1] = r.right; out[4 * n + 2] = r.f_value; out[4 * n + 3] = r.g_value; }
      ++n;
    }, a, b);
    return n;
  }

  // CudaBlockScheduler (cuda_block_scheduler.hpp:29-129): blocks as
  // (rowStart,rowHeight,colStart,colWidth,blockIndex) quintuples.
  uint64_t sbref_schedule(uint64_t nRows, uint64_t nCols, uint64_t maxOut, uint64_t nSplits, int lowerTriangle,
                          uint64_t minSide, uint64_t* out, uint64_t cap, uint64_t* maxRowHeight, uint64_t* maxColWidth)
  {
    sb::CudaBlockScheduler::Config cfg{};
    cfg.nRows = nRows; cfg.nCols = nCols; cfg.maxOutputElements = maxOut; cfg.nSplitsHint = nSplits;
    cfg.triangleMode = lowerTriangle ? sb::BlockTriangleMode::LowerTriangle : sb::BlockTriangleMode::Full;
    cfg.minBlockSide = minSide;
    sb::CudaBlockScheduler s(cfg);
    auto const& bl = s.blocks();
    for (size_t i = 0; i < bl.size() && i < cap; ++i)
    {
      out[5 * i] = bl[i].rowStart; out[5 * i + 1] = bl[i].rowHeight;
      out[5 * i + 2] = bl[i].colStart; out[5 * i + 3] = bl[i].colWidth; out[5 * i + 4] = bl[i].blockIndex;
    }
    *maxRowHeight = s.max_row_height();
    *maxColWidth = s.max_col_width();
    return bl.size();
  }

  // subdivide (algorithms/subdivide.hpp:10-28) as (first,last) pairs.
  uint64_t sbref_subdivide(uint64_t blockSize, uint64_t nItems, uint64_t* out, uint64_t cap)
  {
    auto v = sb::subdivide(blockSize, nItems);
    for (size_t i = 0; i < v.size() && i < cap; ++i) { out[2 * i] = v[i].first; out[2 * i + 1] = v[i].second; }
    return v.size();
  }

  // l1_norm / lp_norm (apply_functional.hpp:63-100, restated: that header
  // pulls in taskflow) over the reference's own iterate_segments.
  double sbref_lp_norm_f64(const double* f, uint64_t lf, double p)
  {
    auto pts = to_points(f, lf);
    double out = 0.0;
    sb::iterate_segments(pts.cbegin(), pts.cend(), 0.0, std::numeric_limits<double>::max(),
                         [&out, p](const auto& seg) {
                           const double a = std::abs(seg.value);
                           out += (seg.right - seg.left) * (p == 1.0 ? a : std::pow(a, p));
                         });
    return p == 1.0 ? out : std::pow(out, 1.0 / p);
  }

  float sbref_lp_norm_f32(const float* f, uint64_t lf, float p)
  {
    auto pts = to_points(f, lf);
    float out = 0.0f;
    sb::iterate_segments(pts.cbegin(), pts.cend(), 0.0f, std::numeric_limits<float>::max(),
                         [&out, p](const auto& seg) {
                           const float a = std::abs(seg.value);
                           out += (seg.right - seg.left) * (p == 1.0f ? a : std::pow(a, p));
                         });
    return p == 1.0f ? out : std::pow(out, 1.0f / p);
  }

  // Returns the byte count of the body; copies at most cap bytes.
  uint64_t sbref_matrix_body_f32(int kind, uint64_t n, const float* storage, unsigned char* out, uint64_t cap)
  { return matrix_body(kind, n, storage, out, cap); }

  uint64_t sbref_matrix_body_f64(int kind, uint64_t n, const double* storage, unsigned char* out, uint64_t cap)
  { return matrix_body(kind, n, storage, out, cap); }
}
