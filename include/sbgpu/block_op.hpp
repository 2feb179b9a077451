// block_op.hpp — the reference's BlockOp for PCFs, for callers that drive
// their own block pipeline (scheduler -> exec_block -> result writer), over
// the C ABI entry sbg_block_device.  Needs the CUDA runtime headers and
// library (it hands out device arrays), unlike compat.hpp.
//
// Kept with the reference's names and behaviour:
//   CudaDeviceArray<T>          include/sbear/cuda/cuda_device_array.cuh
//   CudaPcfDataManager<Tt, Tv>  include/sbear/cuda/cuda_pcf_data_manager.cuh:13-23 (holds the CSR)
//   OperationL1Dist / OperationLpDist / OperationL2InnerProduct
//                               include/sbear/functional/operations.cuh:19-65 (as operation tags)
//   PcfBlockOp<Tt, Tv, ComboOp> include/sbear/cuda/pcf_block_op.cuh:32-123, the BlockOp concept of
//                               include/sbear/cuda/cuda_block_executor.cuh:12-23:
//     GpuStorage, init_gpu_storage(gpuId, scheduler),
//     exec_block(storage, block, gpuOutputMatrix, blockDim)
// exec_block computes the block's dense tile on the current device and
// stream-orders it on the default stream without synchronising, as the
// concept asks; the output matrix must be cleared beforehand.  Storage holds
// the whole CSR, uploaded once (the reference re-uploads each block's rows and
// columns).
#ifndef SBGPU_BLOCK_OP_HPP
#define SBGPU_BLOCK_OP_HPP

#include "compat.hpp"

#include <cuda_runtime.h>

#include <type_traits>

namespace sb
{
  namespace detail
  {
    inline void check_cuda(cudaError_t e)
    {
      if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
    }
  }

  template <typename T>
  class CudaDeviceArray
  {
  public:
    CudaDeviceArray() = default;
    explicit CudaDeviceArray(size_t n) : m_n(n)
    {
      if (n) detail::check_cuda(cudaMalloc(reinterpret_cast<void**>(&m_ptr), n * sizeof(T)));
    }
    ~CudaDeviceArray() { if (m_ptr) cudaFree(m_ptr); }
    CudaDeviceArray(CudaDeviceArray&& o) noexcept : m_ptr(o.m_ptr), m_n(o.m_n) { o.m_ptr = nullptr; o.m_n = 0; }
    CudaDeviceArray& operator=(CudaDeviceArray&& o) noexcept
    {
      if (this != &o)
      {
        if (m_ptr) cudaFree(m_ptr);
        m_ptr = o.m_ptr; m_n = o.m_n; o.m_ptr = nullptr; o.m_n = 0;
      }
      return *this;
    }
    CudaDeviceArray(const CudaDeviceArray&) = delete;
    CudaDeviceArray& operator=(const CudaDeviceArray&) = delete;

    T* get() const { return m_ptr; }
    size_t size() const { return m_n; }
    void upload(const T* src, size_t n) { detail::check_cuda(cudaMemcpy(m_ptr, src, n * sizeof(T), cudaMemcpyHostToDevice)); }
    void download(T* dst, size_t n) const { detail::check_cuda(cudaMemcpy(dst, m_ptr, n * sizeof(T), cudaMemcpyDeviceToHost)); }
    void clear() { if (m_n) detail::check_cuda(cudaMemset(m_ptr, 0, m_n * sizeof(T))); }

  private:
    T* m_ptr = nullptr;
    size_t m_n = 0;
  };

  // The PCFs of one side of the matrix, flattened once into the CSR.
  template <typename Tt, typename Tv>
  class CudaPcfDataManager
  {
    static_assert(std::is_same<Tt, Tv>::value, "time and value types are the same on this path");

  public:
    explicit CudaPcfDataManager(const std::vector<Pcf<Tt, Tv>>& pcfs) : m_n(pcfs.size())
    {
      detail::flatten(pcfs, m_points, m_offsets);
      for (size_t i = 0; i < m_n; ++i)
        m_maxPoints = std::max<uint64_t>(m_maxPoints, m_offsets[i + 1] - m_offsets[i]);
    }
    size_t size() const { return m_n; }
    uint32_t max_points() const { return (uint32_t)std::max<uint64_t>(m_maxPoints, 1); }
    const std::vector<Tt>& points() const { return m_points; }
    const std::vector<uint64_t>& offsets() const { return m_offsets; }

  private:
    size_t m_n;
    std::vector<Tt> m_points;
    std::vector<uint64_t> m_offsets;
    uint64_t m_maxPoints = 0;
  };

  template <typename Tt, typename Tv>
  struct OperationL1Dist
  {
    static constexpr int sbg_op = SBG_OP_L1;
    double p() const { return 1.0; }
  };

  template <typename Tt, typename Tv>
  struct OperationLpDist
  {
    static constexpr int sbg_op = SBG_OP_LP;
    explicit OperationLpDist(Tv p) : m_p(p)
    {
      if (!(p >= Tv(1))) throw std::invalid_argument("p must be >= 1.");
    }
    double p() const { return (double)m_p; }
    Tv m_p;
  };

  template <typename Tt, typename Tv>
  struct OperationL2InnerProduct
  {
    static constexpr int sbg_op = SBG_OP_L2_INNER;
    double p() const { return 1.0; }
  };

  template <typename Tt, typename Tv, typename ComboOp>
  class PcfBlockOp
  {
  public:
    struct GpuStorage
    {
      CudaDeviceArray<uint64_t> rowOffsets;
      CudaDeviceArray<Tt> rowPoints;
      CudaDeviceArray<uint64_t> colOffsets;
      CudaDeviceArray<Tt> colPoints;
    };

    PcfBlockOp(CudaPcfDataManager<Tt, Tv>& rowDataManager, CudaPcfDataManager<Tt, Tv>& colDataManager, ComboOp op,
               Tt a, Tt b, TriangleSkipMode skipMode)
      : m_rows(rowDataManager), m_cols(colDataManager), m_op(op), m_skip(skipMode)
    {
      detail::check_range((double)a, (double)b, (double)std::numeric_limits<Tt>::max());
    }

    GpuStorage init_gpu_storage(size_t gpuId, const CudaBlockScheduler&)
    {
      detail::check_cuda(cudaSetDevice((int)gpuId));
      GpuStorage s;
      s.rowOffsets = CudaDeviceArray<uint64_t>(m_rows.offsets().size());
      s.rowOffsets.upload(m_rows.offsets().data(), m_rows.offsets().size());
      s.rowPoints = CudaDeviceArray<Tt>(m_rows.points().size());
      s.rowPoints.upload(m_rows.points().data(), m_rows.points().size());
      s.colOffsets = CudaDeviceArray<uint64_t>(m_cols.offsets().size());
      s.colOffsets.upload(m_cols.offsets().data(), m_cols.offsets().size());
      s.colPoints = CudaDeviceArray<Tt>(m_cols.points().size());
      s.colPoints.upload(m_cols.points().data(), m_cols.points().size());
      return s;
    }

    template <typename Dim3>
    void exec_block(GpuStorage& s, const BlockInfo& block, CudaDeviceArray<Tv>& gpuOutputMatrix, Dim3)
    {
      if (gpuOutputMatrix.size() < block.rowHeight * block.colWidth)
        throw std::invalid_argument("output matrix smaller than the block");
      throw_status(sbg_block_device(detail::dtype_of<Tt>(), ComboOp::sbg_op, m_op.p(), static_cast<int>(m_skip),
                                    s.rowPoints.get(), s.rowOffsets.get(), s.colPoints.get(), s.colOffsets.get(),
                                    block.rowStart, block.rowHeight, block.colStart, block.colWidth,
                                    std::max(m_rows.max_points(), m_cols.max_points()), gpuOutputMatrix.get(),
                                    nullptr));
    }

  private:
    CudaPcfDataManager<Tt, Tv>& m_rows;
    CudaPcfDataManager<Tt, Tv>& m_cols;
    ComboOp m_op;
    TriangleSkipMode m_skip;
  };
}

#endif
