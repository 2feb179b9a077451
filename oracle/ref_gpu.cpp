// Test and benchmark infrastructure (reference arm), never part of the
// library: drives the stablebear reference's own CUDA block kernel
// (sb::internal::cuda_pcf_block_integrate, include/sbear/cuda/cuda_pcf_kernel.cuh:95-136,
// compiled into oracle/_ref/ref_kernels.cubin by ref_gpu_kernel.cu) over a
// whole pdist / l2-kernel triangle, tile by tile, the way the reference's
// CudaPairwiseIntegrationTask does (include/sbear/cuda/pcf_block_op.cuh:155-180
// and :84-116):
//   * tiles from the reference's block scheduler (restated in
//     include/sbgpu/compat.hpp: square tiles, side from maxOutputElements /
//     nSplitsHint, at least minBlockSide, upper-triangle tiles dropped,
//     sorted by area), with nSplitsHint = 32 (one GPU), minBlockSide =
//     sqrt(SMs * 1024) and maxOutputElements = 80 % of free memory / 2 /
//     sizeof(T) rounded down to 1024 (include/sbear/block_matrix_support.cuh:45-93);
//   * one launch per tile with the reference's default block of 1 x 32
//     threads and its grid (block_matrix_support.cuh:26-35).
// The CSR stays on the device for the whole run (the reference re-uploads
// each tile's rows and columns), and the timed region holds the tile
// kernels only: no per-tile clearing, no copies, no host scatter.  That is
// the reference kernel's best case.  With a host output the tiles are
// copied back and scattered into condensed storage (parity checks); with a
// row sample only the sampled rows of each tile are copied back.
//
// The kernel is reached through the CUDA driver API (cuModuleLoad,
// cuLaunchKernel) with the parameter block of PcfBlockKernelParams<T, T>
// (cuda_pcf_kernel.cuh:19-31, T = float or double) restated below; every
// launch is checked.
#include <cuda.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../include/sbgpu/compat.hpp"

namespace
{
  // PcfBlockKernelParams<T, T>: pointers, sizes, TriangleSkipMode (int).
  struct RefParams
  {
    void* matrix;
    uint64_t* rowTimePointOffsets;
    uint64_t* colTimePointOffsets;
    const void* rowPoints;  // SimplePoint<T, T> {t, v}: the CSR's interleaved layout
    const void* colPoints;
    uint64_t nRows, nCols, globalRowStart, globalColStart;
    int skipMode;
  };
  static_assert(sizeof(RefParams) == 80, "parameter block of the reference kernel");

  struct Fail
  {
    std::string msg;
  };

  void check(CUresult r, const char* what)
  {
    if (r != CUDA_SUCCESS)
    {
      const char* s = nullptr;
      cuGetErrorString(r, &s);
      throw Fail{std::string(what) + ": " + (s ? s : "CUDA driver error")};
    }
  }
}

namespace
{
  // Sampled rows to copy back instead of the whole triangle: row srows[k]'s
  // entries j (j < i for pdist, j <= i for the kernel) land at sout[sbase[k] + j].
  template <typename T>
  struct RowSample
  {
    const uint64_t* rows = nullptr;
    const uint64_t* base = nullptr;
    uint64_t count = 0;
    T* out = nullptr;
  };

  template <typename T>
  int run_triangle(const char* cubin, const char* entry, int skip_mode, double p, uint64_t dpts, uint64_t doff,
                   uint64_t n, T* host_out, uint64_t max_output_elements, double* kernel_ms, uint64_t* n_tiles,
                   char* err, size_t errlen, const RowSample<T>& sample = RowSample<T>())
{
  CUmodule mod = nullptr;
  CUdeviceptr tile = 0;
  CUevent e0 = nullptr, e1 = nullptr;
  std::vector<T> htile;
  try
  {
    if (skip_mode != 1 && skip_mode != 2) throw Fail{"skip_mode must be 1 (pdist) or 2 (kernel)"};
    check(cuInit(0), "cuInit");
    CUcontext ctx = nullptr;
    check(cuCtxGetCurrent(&ctx), "cuCtxGetCurrent");
    if (!ctx) throw Fail{"no current CUDA context (initialise the runtime first)"};
    CUdevice dev;
    check(cuCtxGetDevice(&dev), "cuCtxGetDevice");
    int sms = 0;
    check(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev), "SM count");
    check(cuModuleLoad(&mod, cubin), "cuModuleLoad");
    CUfunction fn;
    check(cuModuleGetFunction(&fn, mod, entry), "cuModuleGetFunction");

    if (max_output_elements == 0)
    {
      size_t freeb = 0, totalb = 0;
      check(cuMemGetInfo(&freeb, &totalb), "cuMemGetInfo");
      max_output_elements = (uint64_t)((double)freeb * 0.8) / 2 / sizeof(T) / 1024 * 1024;
    }
    const uint64_t min_side = (uint64_t)std::sqrt((double)sms * 1024.0);
    sb::CudaBlockScheduler sched({(size_t)n, (size_t)n, (size_t)max_output_elements, 32,
                                  sb::BlockTriangleMode::LowerTriangle, (size_t)min_side});
    const auto& blocks = sched.blocks();
    if (n_tiles) *n_tiles = blocks.size();
    const size_t cap = sched.max_row_height() * sched.max_col_width();
    if (cap == 0) { if (kernel_ms) *kernel_ms = 0; cuModuleUnload(mod); return 0; }
    check(cuMemAlloc(&tile, cap * sizeof(T)), "tile buffer");
    if (host_out) htile.resize(cap);
    else if (sample.count) htile.resize(sched.max_col_width());
    check(cuEventCreate(&e0, CU_EVENT_DEFAULT), "event");
    check(cuEventCreate(&e1, CU_EVENT_DEFAULT), "event");

    const unsigned bx = 1, by = 32;  // the reference's default block (settings blockDimX, blockDimY)
    const T a = T(0), b = sizeof(T) == 4 ? T(FLT_MAX) : T(DBL_MAX);  // numeric_limits<T>::max()
    const unsigned char op_l1 = 0;  // empty operation objects (L1 distance, L2 inner product)
    const T op_lp = T(p);           // OperationLpDist holds p
    const bool lp = std::strstr(entry, "OperationLpDist") != nullptr;
    double total_ms = 0.0;
    for (const auto& blk : blocks)
    {
      RefParams prm;
      prm.matrix = reinterpret_cast<void*>(tile);
      prm.rowTimePointOffsets = reinterpret_cast<uint64_t*>(doff) + blk.rowStart;
      prm.colTimePointOffsets = reinterpret_cast<uint64_t*>(doff) + blk.colStart;
      prm.rowPoints = reinterpret_cast<const void*>(dpts);
      prm.colPoints = reinterpret_cast<const void*>(dpts);
      prm.nRows = blk.rowHeight;
      prm.nCols = blk.colWidth;
      prm.globalRowStart = blk.rowStart;
      prm.globalColStart = blk.colStart;
      prm.skipMode = skip_mode;
      const unsigned gx = (unsigned)((blk.rowHeight + bx - 1) / bx);
      const unsigned gy = (unsigned)((blk.colWidth + by - 1) / by);
      void* args[] = {&prm, const_cast<T*>(&a), const_cast<T*>(&b),
                      lp ? (void*)&op_lp : (void*)&op_l1};
      check(cuEventRecord(e0, nullptr), "event record");
      check(cuLaunchKernel(fn, gx, gy, 1, bx, by, 1, 0, nullptr, args, nullptr), "cuLaunchKernel");
      check(cuEventRecord(e1, nullptr), "event record");
      check(cuEventSynchronize(e1), "kernel");
      float ms = 0.f;
      check(cuEventElapsedTime(&ms, e0, e1), "event time");
      total_ms += ms;
      if (host_out)
      {
        check(cuMemcpyDtoH(htile.data(), tile, blk.rowHeight * blk.colWidth * sizeof(T)), "tile copy");
        for (size_t il = 0; il < blk.rowHeight; ++il)
        {
          const uint64_t i = blk.rowStart + il;
          for (size_t jl = 0; jl < blk.colWidth; ++jl)
          {
            const uint64_t j = blk.colStart + jl;
            if (skip_mode == 1 ? j >= i : j > i) continue;
            const uint64_t idx = skip_mode == 1 ? i * (i - 1) / 2 + j : i * (i + 1) / 2 + j;
            host_out[idx] = htile[il * blk.colWidth + jl];
          }
        }
      }
      else if (sample.count)
      {
        for (uint64_t k = 0; k < sample.count; ++k)
        {
          const uint64_t i = sample.rows[k];
          if (i < blk.rowStart || i >= blk.rowStart + blk.rowHeight) continue;
          const uint64_t il = i - blk.rowStart;
          check(cuMemcpyDtoH(htile.data(), tile + il * blk.colWidth * sizeof(T), blk.colWidth * sizeof(T)),
                "row copy");
          for (size_t jl = 0; jl < blk.colWidth; ++jl)
          {
            const uint64_t j = blk.colStart + jl;
            if (skip_mode == 1 ? j >= i : j > i) continue;
            sample.out[sample.base[k] + j] = htile[jl];
          }
        }
      }
    }
    if (kernel_ms) *kernel_ms = total_ms;
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    cuMemFree(tile);
    cuModuleUnload(mod);
    return 0;
  }
  catch (const Fail& f)
  {
    if (err && errlen) std::snprintf(err, errlen, "%s", f.msg.c_str());
    if (e0) cuEventDestroy(e0);
    if (e1) cuEventDestroy(e1);
    if (tile) cuMemFree(tile);
    if (mod) cuModuleUnload(mod);
    return -1;
  }
}
}

// elem_bytes 4: float CSR and output, 8: double.
extern "C" int sbref_gpu_triangle(const char* cubin, const char* entry, int elem_bytes, int skip_mode, double p,
                                  uint64_t dpts, uint64_t doff, uint64_t n, void* host_out,
                                  uint64_t max_output_elements, double* kernel_ms, uint64_t* n_tiles, char* err,
                                  size_t errlen)
{
  if (elem_bytes == 4)
    return run_triangle<float>(cubin, entry, skip_mode, p, dpts, doff, n, static_cast<float*>(host_out),
                               max_output_elements, kernel_ms, n_tiles, err, errlen);
  if (elem_bytes == 8)
    return run_triangle<double>(cubin, entry, skip_mode, p, dpts, doff, n, static_cast<double*>(host_out),
                                max_output_elements, kernel_ms, n_tiles, err, errlen);
  if (err && errlen) std::snprintf(err, errlen, "elem_bytes must be 4 or 8");
  return -1;
}

// As sbref_gpu_triangle, copying back only the listed rows (a few rows of a
// 20 GB triangle instead of a host scatter of all of it): row rows[k]'s
// entries j land at sample_out[row_base[k] + j].
extern "C" int sbref_gpu_triangle_rows(const char* cubin, const char* entry, int elem_bytes, int skip_mode, double p,
                                       uint64_t dpts, uint64_t doff, uint64_t n, const uint64_t* rows,
                                       const uint64_t* row_base, uint64_t n_rows, void* sample_out,
                                       uint64_t max_output_elements, double* kernel_ms, uint64_t* n_tiles, char* err,
                                       size_t errlen)
{
  if (elem_bytes == 4)
  {
    RowSample<float> s{rows, row_base, n_rows, static_cast<float*>(sample_out)};
    return run_triangle<float>(cubin, entry, skip_mode, p, dpts, doff, n, nullptr, max_output_elements, kernel_ms,
                               n_tiles, err, errlen, s);
  }
  if (elem_bytes == 8)
  {
    RowSample<double> s{rows, row_base, n_rows, static_cast<double*>(sample_out)};
    return run_triangle<double>(cubin, entry, skip_mode, p, dpts, doff, n, nullptr, max_output_elements, kernel_ms,
                                n_tiles, err, errlen, s);
  }
  if (err && errlen) std::snprintf(err, errlen, "elem_bytes must be 4 or 8");
  return -1;
}
