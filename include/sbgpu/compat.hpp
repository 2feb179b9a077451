// compat.hpp — the reference's C++ interfaces for the pairwise path, over the
// C ABI of include/sbgpu.h.  Header-only; link with libsbgpu.so.
//
// Kept with the reference's names and behaviour so C++ callers switch by
// changing includes (namespace sb, as in the reference):
//   TriangleSkipMode            include/sbear/cuda/triangle_skip_mode.hpp:7-12
//   BlockInfo, BlockTriangleMode, CudaBlockScheduler
//                               include/sbear/cuda/cuda_block_scheduler.hpp:14-129,
//                               include/sbear/algorithms/subdivide.hpp:10-28
//   DistanceMatrix, SymmetricMatrix
//                               include/sbear/distance_matrix.hpp:27-150,
//                               include/sbear/symmetric_matrix.hpp:25-107
//   DenseMatrixView, BlockResultWriter and its aliases
//                               include/sbear/cuda/cuda_result_writer.hpp:17-108
//   TimePoint, Pcf (the part the factories read)
//                               include/sbear/functional/time_point.hpp:16-53, pcf.hpp:15-40
//   StoppableTask<void>         include/sbear/task.hpp:15-172 (backed by sbg_task)
//   the 12 create_cuda_block_* factories
//                               include/sbear/cuda/cuda_matrix_integrate_api.hpp:19-113
// The factories compute with this library's kernels; the scheduler and
// writer are the reference's tile interfaces for callers that produce or
// consume dense tiles themselves (the library's own pipeline writes the
// final layout directly and needs neither).
#ifndef SBGPU_COMPAT_HPP
#define SBGPU_COMPAT_HPP

#include "../sbgpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace sb
{
  enum class TriangleSkipMode : int
  {
    None = 0,
    LowerTriangleSkipDiag = 1,
    LowerTriangle = 2
  };

  // ---- block scheduler ------------------------------------------------------

  struct BlockInfo
  {
    size_t rowStart;
    size_t rowHeight;
    size_t colStart;
    size_t colWidth;
    size_t blockIndex;
  };

  enum class BlockTriangleMode
  {
    LowerTriangle,
    Full
  };

  // Inclusive [first, last] bands of blockSize items covering [0, nItems).
  inline std::vector<std::pair<size_t, size_t>> subdivide(size_t blockSize, size_t nItems)
  {
    std::vector<std::pair<size_t, size_t>> bands;
    if (nItems == 0 || blockSize == 0) return bands;
    for (size_t first = 0; first < nItems; first += blockSize)
      bands.emplace_back(first, std::min(first + blockSize, nItems) - 1);
    return bands;
  }

  // Square tiles of side clamp(floor(sqrt(maxOutputElements / nSplitsHint)),
  // minBlockSide, max(nRows, nCols)); in LowerTriangle mode tiles entirely
  // above the diagonal are dropped; tiles are ordered by area, largest first.
  class CudaBlockScheduler
  {
  public:
    struct Config
    {
      size_t nRows;
      size_t nCols;
      size_t maxOutputElements;
      size_t nSplitsHint;
      BlockTriangleMode triangleMode = BlockTriangleMode::Full;
      size_t minBlockSide = 0;
    };

    explicit CudaBlockScheduler(const Config& config) : m_triangleMode(config.triangleMode)
    {
      if (config.nRows == 0 || config.nCols == 0) return;
      const size_t side = block_side(config);
      const auto rows = subdivide(side, config.nRows);
      const auto cols = subdivide(side, config.nCols);
      for (const auto& r : rows)
      {
        const size_t h = r.second - r.first + 1;
        for (const auto& c : cols)
        {
          if (config.triangleMode == BlockTriangleMode::LowerTriangle && c.first > r.second) continue;
          const size_t w = c.second - c.first + 1;
          m_blocks.push_back(BlockInfo{r.first, h, c.first, w, m_blocks.size()});
          m_maxRowHeight = std::max(m_maxRowHeight, h);
          m_maxColWidth = std::max(m_maxColWidth, w);
        }
      }
      std::sort(m_blocks.begin(), m_blocks.end(), [](const BlockInfo& a, const BlockInfo& b) {
        return a.rowHeight * a.colWidth > b.rowHeight * b.colWidth;
      });
      for (size_t i = 0; i < m_blocks.size(); ++i) m_blocks[i].blockIndex = i;
    }

    const std::vector<BlockInfo>& blocks() const { return m_blocks; }
    size_t max_row_height() const { return m_maxRowHeight; }
    size_t max_col_width() const { return m_maxColWidth; }
    BlockTriangleMode triangle_mode() const { return m_triangleMode; }

  private:
    static size_t block_side(const Config& c)
    {
      const size_t per = c.maxOutputElements / std::max<size_t>(c.nSplitsHint, 1);
      size_t side = std::max<size_t>(static_cast<size_t>(std::sqrt(static_cast<double>(per))), 1);
      if (c.minBlockSide > 0) side = std::max(side, c.minBlockSide);
      return std::min(side, std::max(c.nRows, c.nCols));
    }

    std::vector<BlockInfo> m_blocks;
    size_t m_maxRowHeight = 0;
    size_t m_maxColWidth = 0;
    BlockTriangleMode m_triangleMode;
  };

  // ---- condensed matrices ----------------------------------------------------

  template <typename T>
  class DistanceMatrix
  {
  public:
    using value_type = T;

    // Reads give the stored value (0 on the diagonal); writes reject negative
    // values and non-zero diagonal values (distance_matrix.hpp:33-61).
    class EntryProxy
    {
    public:
      explicit EntryProxy(T* p) : m_p(p) { }
      operator T() const { return m_p ? *m_p : T{}; }
      EntryProxy& operator=(const T& v)
      {
        if (v < T{}) throw std::invalid_argument("Distance matrix entries must be nonnegative");
        if (!m_p)
        {
          if (v != T{}) throw std::invalid_argument("Diagonal entries of a distance matrix must be zero");
          return *this;
        }
        *m_p = v;
        return *this;
      }

    private:
      T* m_p;
    };

    explicit DistanceMatrix(size_t n, const T& init = {})
      : m_data(new T[storage_size(n)], std::default_delete<T[]>()), m_size(n)
    {
      if (init < T{}) throw std::invalid_argument("Distance matrix entries must be nonnegative");
      std::fill(m_data.get(), m_data.get() + storage_size(n), init);
    }
    DistanceMatrix() : DistanceMatrix(0) { }

    size_t size() const { return m_size; }
    size_t storage_count() const { return storage_size(m_size); }
    static size_t storage_size(size_t n) { return n == 0 ? 0 : n * (n - 1) / 2; }

    EntryProxy operator()(size_t i, size_t j)
    {
      check(i, j);
      return EntryProxy(i == j ? nullptr : m_data.get() + index(i, j));
    }
    T operator()(size_t i, size_t j) const
    {
      check(i, j);
      return i == j ? T{} : m_data.get()[index(i, j)];
    }
    const T* data() const { return m_data.get(); }
    // Storage the library fills in place (DistanceMatrix order).
    T* storage() { return m_data.get(); }

  private:
    static size_t index(size_t i, size_t j)
    {
      const size_t r = std::max(i, j), c = std::min(i, j);
      return r * (r - 1) / 2 + c;
    }
    void check(size_t i, size_t j) const
    {
      if (i >= m_size || j >= m_size)
      {
        std::ostringstream os;
        os << "DistanceMatrix index (" << i << ", " << j << ") out of range for matrix of size " << m_size;
        throw std::out_of_range(os.str());
      }
    }
    std::shared_ptr<T> m_data;
    size_t m_size;
  };

  template <typename T>
  class SymmetricMatrix
  {
  public:
    using value_type = T;
    explicit SymmetricMatrix(size_t n, const T& init = {})
      : m_data(new T[storage_size(n)], std::default_delete<T[]>()), m_size(n)
    {
      std::fill(m_data.get(), m_data.get() + storage_size(n), init);
    }
    SymmetricMatrix() : SymmetricMatrix(0) { }

    size_t size() const { return m_size; }
    size_t storage_count() const { return storage_size(m_size); }
    static size_t storage_size(size_t n) { return n * (n + 1) / 2; }

    T& operator()(size_t i, size_t j) { return m_data.get()[index(i, j)]; }
    const T& operator()(size_t i, size_t j) const { return m_data.get()[index(i, j)]; }
    const T* data() const { return m_data.get(); }
    T* storage() { return m_data.get(); }

  private:
    size_t index(size_t i, size_t j) const
    {
      if (i >= m_size || j >= m_size)
      {
        std::ostringstream os;
        os << "SymmetricMatrix index (" << i << ", " << j << ") out of range for matrix of size " << m_size;
        throw std::out_of_range(os.str());
      }
      const size_t r = std::max(i, j), c = std::min(i, j);
      return r * (r + 1) / 2 + c;
    }
    std::shared_ptr<T> m_data;
    size_t m_size;
  };

  // Row-major view over caller-owned dense storage (stands in for the
  // reference's Tensor<Tv>).
  template <typename Tv>
  class DenseMatrixView
  {
  public:
    DenseMatrixView(Tv* data, size_t nCols) : m_data(data), m_nCols(nCols) { }
    Tv& operator()(size_t i, size_t j) { return m_data[i * m_nCols + j]; }
    Tv* data() { return m_data; }

  private:
    Tv* m_data;
    size_t m_nCols;
  };

  // Scatters a dense host tile into a matrix; in the triangular modes the
  // skipped entries must be zero (cuda_result_writer.hpp:54-94).
  template <typename MatrixT, TriangleSkipMode Mode>
  class BlockResultWriter
  {
  public:
    explicit BlockResultWriter(MatrixT mat) : m_mat(std::move(mat)) { }

    template <typename Tv>
    void scatter(const Tv* hostBlock, const BlockInfo& block)
    {
      for (size_t il = 0; il < block.rowHeight; ++il)
      {
        const size_t i = block.rowStart + il;
        for (size_t jl = 0; jl < block.colWidth; ++jl)
        {
          const size_t j = block.colStart + jl;
          const Tv v = hostBlock[il * block.colWidth + jl];
          const bool skip = (Mode == TriangleSkipMode::LowerTriangleSkipDiag && i <= j)
                         || (Mode == TriangleSkipMode::LowerTriangle && i < j);
          if (skip)
          {
            if (v != Tv(0))
              throw std::logic_error("Non-zero value at skipped position (" + std::to_string(i) + ", "
                                     + std::to_string(j) + ") in "
                                     + (Mode == TriangleSkipMode::LowerTriangle ? "symmetric" : "distance")
                                     + " matrix scatter");
            continue;
          }
          m_mat(i, j) = v;
        }
      }
    }

  private:
    MatrixT m_mat;
  };

  template <typename Tv>
  using DistanceMatrixResultWriter = BlockResultWriter<DistanceMatrix<Tv>, TriangleSkipMode::LowerTriangleSkipDiag>;
  template <typename Tv>
  using SymmetricMatrixResultWriter = BlockResultWriter<SymmetricMatrix<Tv>, TriangleSkipMode::LowerTriangle>;
  template <typename Tv>
  using DenseResultWriter = BlockResultWriter<DenseMatrixView<Tv>, TriangleSkipMode::None>;

  // ---- PCFs ------------------------------------------------------------------

  template <typename Tt, typename Tv>
  struct TimePoint
  {
    Tt t = Tt(0);
    Tv v = Tv(0);
    TimePoint() = default;
    TimePoint(Tt it, Tv iv) : t(it), v(iv) { }
  };

  template <typename Tt, typename Tv = Tt>
  class Pcf
  {
  public:
    using point_type = TimePoint<Tt, Tv>;
    Pcf() { m_points.emplace_back(Tt(0), Tv(0)); }
    explicit Pcf(std::vector<point_type>&& pts) : m_points(std::move(pts)) { }
    const std::vector<point_type>& points() const { return m_points; }
    size_t size() const { return m_points.size(); }

  private:
    std::vector<point_type> m_points;
  };

  // ---- tasks -------------------------------------------------------------------

  inline void throw_status(int st)
  {
    if (st == SBG_OK) return;
    const std::string msg = sbg_last_error();
    if (st == SBG_ERR_INVALID_ARGUMENT || st == SBG_ERR_INVALID_INPUT) throw std::invalid_argument(msg);
    if (st == SBG_ERR_LOGIC) throw std::logic_error(msg);
    throw std::runtime_error(msg);
  }

  // The reference's task executor (include/sbear/executor.hpp): callers pass
  // default_executor() to start_async.  Tasks here run on their own worker
  // thread, so the executor carries nothing.
  struct Executor
  {
  };
  inline Executor& default_executor()
  {
    static Executor e;
    return e;
  }

  template <typename RetT = void>
  class StoppableTask;

  template <>
  class StoppableTask<void>
  {
  public:
    explicit StoppableTask(sbg_task* t) : m_task(t) { }
    ~StoppableTask() { if (m_task) sbg_task_destroy(m_task); }
    StoppableTask(const StoppableTask&) = delete;
    StoppableTask& operator=(const StoppableTask&) = delete;

    // The executor argument of the reference is accepted and unused: the
    // task runs on its own worker thread.
    template <typename Exec = int>
    StoppableTask& start_async(Exec&& = 0)
    {
      throw_status(sbg_task_start(m_task));
      return *this;
    }
    bool wait_for(std::chrono::milliseconds d)
    {
      int fin = 0;
      throw_status(sbg_task_wait_for(m_task, static_cast<int64_t>(d.count()), &fin));
      return fin != 0;
    }
    void wait() { throw_status(sbg_task_wait(m_task)); }
    void request_stop() { sbg_task_request_stop(m_task); }
    bool stop_requested() const { return sbg_task_stop_requested(m_task) != 0; }
    size_t work_total() const { uint64_t t = 0; sbg_task_progress(m_task, &t, nullptr, nullptr); return (size_t)t; }
    size_t work_completed() const { uint64_t c = 0; sbg_task_progress(m_task, nullptr, &c, nullptr); return (size_t)c; }
    size_t work_step() const { uint64_t s = 0; sbg_task_progress(m_task, nullptr, nullptr, &s); return (size_t)s; }

  private:
    sbg_task* m_task;
  };

  // ---- the 12 factories ------------------------------------------------------------

  namespace detail
  {
    template <typename T>
    void flatten(const std::vector<Pcf<T, T>>& pcfs, std::vector<T>& pts, std::vector<uint64_t>& off)
    {
      off.assign(1, 0);
      pts.clear();
      for (const auto& f : pcfs)
      {
        for (const auto& p : f.points()) { pts.push_back(p.t); pts.push_back(p.v); }
        off.push_back(pts.size() / 2);
      }
      if (pts.empty()) pts.resize(2);
    }

    template <typename T> constexpr int dtype_of() { return sizeof(T) == 4 ? SBG_F32 : SBG_F64; }

    inline void check_range(double a, double b, double maxv)
    {
      if (a != 0.0 || b != maxv)
        throw std::invalid_argument("only the full range [0, numeric_limits<T>::max()] is supported");
    }

    template <typename T, typename M>
    std::unique_ptr<StoppableTask<void>> integrate(M& out, const std::vector<Pcf<T, T>>& pcfs, int op, double p,
                                                   int skip, T a, T b)
    {
      check_range(a, b, std::numeric_limits<T>::max());
      if (out.size() != pcfs.size()) throw std::invalid_argument("output matrix size does not match the PCF count");
      std::vector<T> pts;
      std::vector<uint64_t> off;
      flatten(pcfs, pts, off);
      sbg_task* t = nullptr;
      throw_status(sbg_create_integrate_task(dtype_of<T>(), op, p, skip, pts.data(), off.data(), pcfs.size(),
                                             out.storage(), &t));
      return std::make_unique<StoppableTask<void>>(t);
    }

    template <typename T>
    std::unique_ptr<StoppableTask<void>> cross(T* out, const std::vector<Pcf<T, T>>& rows,
                                               const std::vector<Pcf<T, T>>& cols, int op, double p, T a, T b)
    {
      check_range(a, b, std::numeric_limits<T>::max());
      std::vector<T> rp, cp;
      std::vector<uint64_t> ro, co;
      flatten(rows, rp, ro);
      flatten(cols, cp, co);
      sbg_task* t = nullptr;
      throw_status(sbg_create_cdist_task(dtype_of<T>(), op, p, rp.data(), ro.data(), rows.size(), cp.data(), co.data(),
                                         cols.size(), out, &t));
      return std::make_unique<StoppableTask<void>>(t);
    }
  }

#define SBG_COMPAT_FACTORIES(T)                                                                                     \
  inline std::unique_ptr<StoppableTask<void>> create_cuda_block_integrate_l1_task(                                  \
      DistanceMatrix<T>& out, const std::vector<Pcf<T, T>>& pcfs, T a = T(0), T b = std::numeric_limits<T>::max()) \
  { return detail::integrate(out, pcfs, SBG_OP_L1, 1.0, SBG_SKIP_LOWER_NODIAG, a, b); }                            \
  inline std::unique_ptr<StoppableTask<void>> create_cuda_block_integrate_lp_task(                                  \
      DistanceMatrix<T>& out, const std::vector<Pcf<T, T>>& pcfs, T p, T a = T(0),                                  \
      T b = std::numeric_limits<T>::max())                                                                          \
  { return detail::integrate(out, pcfs, SBG_OP_LP, (double)p, SBG_SKIP_LOWER_NODIAG, a, b); }                      \
  inline std::unique_ptr<StoppableTask<void>> create_cuda_block_integrate_l2_kernel_task(                           \
      SymmetricMatrix<T>& out, const std::vector<Pcf<T, T>>& pcfs, T a = T(0), T b = std::numeric_limits<T>::max()) \
  { return detail::integrate(out, pcfs, SBG_OP_L2_INNER, 1.0, SBG_SKIP_LOWER, a, b); }                             \
  inline std::unique_ptr<StoppableTask<void>> create_cuda_block_cdist_l1_task(                                      \
      T* out, const std::vector<Pcf<T, T>>& rows, const std::vector<Pcf<T, T>>& cols, T a = T(0),                   \
      T b = std::numeric_limits<T>::max())                                                                          \
  { return detail::cross(out, rows, cols, SBG_OP_L1, 1.0, a, b); }                                                  \
  inline std::unique_ptr<StoppableTask<void>> create_cuda_block_cdist_lp_task(                                      \
      T* out, const std::vector<Pcf<T, T>>& rows, const std::vector<Pcf<T, T>>& cols, T p, T a = T(0),              \
      T b = std::numeric_limits<T>::max())                                                                          \
  { return detail::cross(out, rows, cols, SBG_OP_LP, (double)p, a, b); }                                            \
  inline std::unique_ptr<StoppableTask<void>> create_cuda_block_cdist_l2_kernel_task(                               \
      T* out, const std::vector<Pcf<T, T>>& rows, const std::vector<Pcf<T, T>>& cols, T a = T(0),                   \
      T b = std::numeric_limits<T>::max())                                                                          \
  { return detail::cross(out, rows, cols, SBG_OP_L2_INNER, 1.0, a, b); }

  SBG_COMPAT_FACTORIES(float)
  SBG_COMPAT_FACTORIES(double)
#undef SBG_COMPAT_FACTORIES
}

#endif
