// Internal host-side declarations shared by the engine, the task layer and
// the C ABI.  Not installed; the public surface is include/sbgpu.h and
// include/sbgpu/*.hpp.
#pragma once

#include "pair_kernels.cuh"

#include <atomic>
#include <cstdint>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

namespace sbg
{
  // Status codes of the C ABI (include/sbgpu.h).
  enum Status : int
  {
    ST_OK = 0,
    ST_INVALID_ARGUMENT = -1,
    ST_INVALID_INPUT = -2,
    ST_CUDA = -3,
    ST_OUT_OF_MEMORY = -4,
    ST_CANCELLED = -5,
    ST_NO_DEVICE = -6,
    ST_TIMEOUT = -7,
    ST_INTERNAL = -8,
    ST_LOGIC = -9,
  };

  // Exception carrying a C-ABI status; converted at the ABI boundary.
  struct Error : std::runtime_error
  {
    int status;
    Error(int st, const std::string& msg) : std::runtime_error(msg), status(st) { }
  };

  // "file:line: <cuda message>", as the reference's CHK_CUDA does
  // (include/sbear/cuda/cuda_util.cuh:8-10), raised as an Error.
  [[noreturn]] void throw_cuda(cudaError_t e, const char* file, int line);
#define SBG_CUDA(expr)                                      \
  do {                                                      \
    cudaError_t sbg_e_ = (expr);                            \
    if (sbg_e_ != cudaSuccess) ::sbg::throw_cuda(sbg_e_, __FILE__, __LINE__); \
  } while (0)

  void set_last_error(const std::string& msg);
  const char* last_error();

  // Process-wide settings; mirrors sb::Settings (include/sbear/settings.hpp:8-23).
  struct Settings
  {
    std::atomic<bool> forceCpu{false};
    std::atomic<uint64_t> cudaThreshold{500};
    std::atomic<bool> deviceVerbose{false};
    std::atomic<unsigned> blockDimX{1};
    std::atomic<unsigned> blockDimY{32};
    std::atomic<uint64_t> minBlockSide{0};
    std::atomic<int> gpuLimit{-1};
    std::atomic<int> cpuLimit{-1};
    // Engine knobs (0 = automatic).
    std::atomic<int> warps{0};
    std::atomic<int> rowChunk{0};        // Q: rows per work item = 32 * Q
    std::atomic<int> variant{0};         // 0 auto, 1 shared-memory (8-byte row elements), 2 global-memory, 3 shared-memory pointer walk, 4 hybrid, 5 shared-memory with row times and values apart, 6 time-windowed shared memory
    std::atomic<int> windowCap{0};       // time-windowed variant: elements per slice (0 = the most that fit)
    std::atomic<int> order{0};           // 0 auto, 1 caller order, 2 length-sorted
    std::atomic<uint64_t> bandBytes{0};  // output bytes per pipeline band (0 = auto)
    std::atomic<int> outputMode{0};      // host results: 0 auto (staged), 1 staged copy, 2 direct stores (coherent hosts)
  };
  Settings& settings();

  // RAII device buffer.
  class DeviceBuffer
  {
  public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) { reset(bytes); }
    ~DeviceBuffer() { release(); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : m_ptr(o.m_ptr), m_bytes(o.m_bytes) { o.m_ptr = nullptr; o.m_bytes = 0; }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept
    {
      if (this != &o) { release(); m_ptr = o.m_ptr; m_bytes = o.m_bytes; o.m_ptr = nullptr; o.m_bytes = 0; }
      return *this;
    }
    void reset(size_t bytes);
    void release();
    void* get() const { return m_ptr; }
    template <typename U> U* as() const { return static_cast<U*>(m_ptr); }
    size_t bytes() const { return m_bytes; }

  private:
    void* m_ptr = nullptr;
    size_t m_bytes = 0;
  };

  struct DeviceInfo
  {
    int device = 0;
    int sms = 0;
    size_t smem_optin = 0;   // shared memory one CTA may opt in to
    size_t smem_per_sm = 0;  // shared memory of one SM (all its CTAs)
    int threads_per_sm = 0;
  };
  DeviceInfo device_info();

  // Resident CTAs per SM of a persistent pair kernel (64 registers per
  // thread, launch_bounds(1024, 1)) with `warps` warps and `smem_bytes` of
  // dynamic shared memory (plus 1 KB the runtime reserves per CTA).
  int ctas_per_sm(const DeviceInfo& dev, int warps, size_t smem_bytes);

  // A set of PCFs in the reference's CSR layout.
  template <typename T>
  struct PcfSet
  {
    const T* pts = nullptr;        // interleaved (t, v)
    const uint64_t* off = nullptr; // n + 1 offsets
    uint64_t n = 0;
  };

  // Host-side checks of the input contract (pypcf_support.hpp:76-89):
  // offsets non-decreasing from 0, every PCF non-empty, first time 0, times
  // non-decreasing and finite.  Throws Error(ST_INVALID_INPUT).
  template <typename T>
  void validate_pcfs(const PcfSet<T>& s, const char* what);

  // Launch plan for one pairwise problem on the device.
  struct Plan
  {
    bool smem = true;
    int kvar = 2;      // kernel variant: 0 global memory, 1 shared two-load walk, 2 shared predicated walk,
                       // 3 hybrid (columns in shared memory, rows through L1), 5 shared with row times and
                       // values apart, 6 time-windowed shared memory
    bool packed = false;  // the kernel reads the packed segment layout (variants 0 and 3)
    int warps = 16;
    int grid = 1;
    uint32_t q = 1;
    uint32_t lmax_c = 0;
    uint32_t row_cap = 0;
    uint32_t win_r = 0;      // time-windowed variant: row slice cap (lmax_c is the column slice cap)
    uint32_t row_slots = 0;  // time-windowed variant: rows per item with saved slice starts
    size_t smem_bytes = 0;
  };

  // Length statistics used for planning.
  struct LengthStats
  {
    uint32_t lmax = 0;
    uint32_t lmin = 0;
    double mean = 0.0;
  };

  // The float32 measurement variants 7 (replicated row, one unified load per
  // step) and 8 (merge path, one pair per warp), pair_variants.cu.
  cudaError_t launch_pair_variant(const LaunchParams<float>& L, int opk, int variant, int warps, int grid,
                                  size_t smem, cudaStream_t s);
  int padded_words(int k);  // k + k / 32: variant 8's padded index

  // opk: the operation kind, for the launch-shape cache (-1: no lookup).
  template <typename T>
  Plan make_plan(int mode, uint64_t n_rows, uint64_t n_cols, const LengthStats& rows, const LengthStats& cols,
                 const DeviceInfo& dev, int opk);

  int op_kind(int op, double p);

  // Kernel launchers (pair_kernels.cu).
  template <typename T>
  cudaError_t launch_pairs(const LaunchParams<T>& L, int opk, int variant, int warps, int grid,
                           size_t smem_bytes, cudaStream_t s);
  template <typename T>
  cudaError_t launch_pack(const T* pts, const uint64_t* off, uint64_t n, Elem<T>* out, uint64_t cap, int sms,
                          cudaStream_t s);
  int kernel_unroll(bool f64);

  // Shared-memory layout of the time-windowed variant for `warps` warps and
  // items of up to rows_per_item rows: slice caps (`cap`, else the setting,
  // else the largest multiple of 8 that fits, at most lmax rounded up to 8),
  // row buffer, row slots and bytes.  False when it does not fit.
  bool window_layout(Plan& pl, size_t elem_bytes, int warps, uint32_t rows_per_item, uint32_t lmax, size_t usable,
                     uint32_t cap = 0);

  // Control block of one host-side run (progress, cancellation).
  struct RunControl
  {
    std::atomic<bool>* stop = nullptr;
    std::function<void(uint64_t)> progress;
  };

  // Whole pipeline for host buffers: H2D of the CSR, kernel launches over
  // row bands, D2H of each band straight into the caller's condensed/dense
  // output.  mode: MODE_PDIST, MODE_KERNEL (cols ignored) or MODE_CROSS.
  template <typename T>
  void compute_host(int mode, int op, double p, const PcfSet<T>& rows, const PcfSet<T>* cols, T* out,
                    bool validate, const RunControl& ctl);

  // Stream-ordered computation on device buffers.  Uses cached scratch for
  // the descriptor and queue counter; packed copies for the global-memory
  // variant are allocated per call.
  template <typename T>
  void compute_device(int mode, int op, double p, const PcfSet<T>& rows, const PcfSet<T>* cols,
                      const uint32_t* rperm, const uint32_t* cperm, uint32_t lmax, T* out, uint64_t out_base,
                      uint64_t row_begin, uint64_t row_end, cudaStream_t stream);

  // The device computation with caller-provided scratch (no allocation):
  // the work-queue counter at scratch[0..8) and, when the PCFs are too long
  // for the shared-memory kernel, the packed segment layout after it.
  // Throws ST_INVALID_ARGUMENT when scratch_bytes is too small.
  template <typename T>
  void compute_device_scratch(int mode, int op, double p, const PcfSet<T>& rows, const PcfSet<T>* cols,
                              const uint32_t* rperm, const uint32_t* cperm, uint32_t lmax, uint64_t row_points,
                              uint64_t col_points, T* out, uint64_t out_base, uint64_t row_begin, uint64_t row_end,
                              void* scratch, size_t scratch_bytes, cudaStream_t stream);
  template <typename T>
  size_t scratch_needed(int mode, uint64_t n_rows, uint64_t n_cols, uint32_t lmax, uint64_t row_points,
                        uint64_t col_points);

  uint64_t output_count(int mode, uint64_t n_rows, uint64_t n_cols);
  uint64_t row_output_start(int mode, uint64_t row, uint64_t n_cols);

  // Length order (sort.cu): within each window of LENGTH_ORDER_WINDOW
  // consecutive PCFs, by breakpoint count, ties by index.  The device
  // version; `scratch` holds length_order_scratch_bytes(n) bytes.
  constexpr uint64_t LENGTH_ORDER_WINDOW = 1024;
  uint64_t length_order_scratch_bytes(uint64_t n);
  void length_order_device(const uint64_t* off, uint64_t n, uint32_t* perm, void* scratch, cudaStream_t st);

  // Launch accounting: every kernel launch of the library is followed by
  // launched(), which counts it and returns the launch error.  A CUDA graph
  // replay counts the kernels it holds.
  cudaError_t launched();
  void count_launches(uint64_t n);
  void uncount_launches(uint64_t n);
  uint64_t kernel_launches();

  // Every device allocation of the library goes through these four calls
  // (no other file calls cudaMalloc / cudaMallocAsync / cudaFree /
  // cudaFreeAsync).  They count allocations and the bytes they hold, and
  // refuse, with ST_OUT_OF_MEMORY and before any CUDA call, an allocation
  // that would take the bytes held above the limit set by
  // sbg_set_alloc_limit: host-side fault injection of the reference's
  // CHK_CUDA out-of-memory failure (include/sbear/cuda/cuda_util.cuh:8-10).
  void* device_malloc(size_t bytes);
  void device_free(void* p, size_t bytes) noexcept;
  void* device_malloc_async(size_t bytes, cudaStream_t st);
  void device_free_async(void* p, size_t bytes, cudaStream_t st) noexcept;
  void set_alloc_limit(uint64_t bytes);
  uint64_t device_allocations();
  uint64_t device_bytes_held();

  // Launch-shape cache of the single-problem planner, filled by
  // sbg_autotune_device.  Key: element size, operation, mode and the
  // problem's shape bucket (floor(log2) of the PCF count and of the longest
  // PCF).  Value: warps per CTA and rows per work item (32 q), the two knobs
  // that change no bit of a result.
  struct TuneKey
  {
    int elem_bytes, opk, mode, n_log2, lmax_log2;
    bool operator<(const TuneKey& o) const
    {
      return std::tie(elem_bytes, opk, mode, n_log2, lmax_log2) <
             std::tie(o.elem_bytes, o.opk, o.mode, o.n_log2, o.lmax_log2);
    }
  };
  TuneKey tune_key(int elem_bytes, int opk, int mode, uint64_t n, uint32_t lmax);
  bool tune_cache_get(const TuneKey& k, int* warps, int* q);
  void tune_cache_put(const TuneKey& k, int warps, int q);
  void tune_cache_clear();

  // RAII stream-ordered device buffer (device_malloc_async / device_free_async).
  class StreamBuffer
  {
  public:
    StreamBuffer(size_t bytes, cudaStream_t st) : m_bytes(bytes), m_stream(st)
    {
      if (bytes) m_ptr = device_malloc_async(bytes, st);
    }
    ~StreamBuffer() { device_free_async(m_ptr, m_bytes, m_stream); }
    StreamBuffer(const StreamBuffer&) = delete;
    StreamBuffer& operator=(const StreamBuffer&) = delete;
    void* get() const { return m_ptr; }
    template <typename U> U* as() const { return static_cast<U*>(m_ptr); }

  private:
    void* m_ptr = nullptr;
    size_t m_bytes = 0;
    cudaStream_t m_stream = nullptr;
  };
}
