// One block of the output matrix, for callers that keep the reference's
// block pipeline: the reference's BlockOp::exec_block
// (include/sbear/cuda/pcf_block_op.cuh:82-122) computes the dense
// rowHeight x colWidth tile of a scheduler block (cuda_block_scheduler.hpp)
// into a pre-cleared device matrix, leaving the entries its triangle skip
// mode excludes untouched.
//
// Here the tile is a cdist of the block's row range against its column range
// (the CSR offsets are absolute, so a range is a plain sub-array of them), run
// by the persistent pair kernel; a second pass writes zeros back over the
// excluded entries of a block that crosses the diagonal, so the tile holds
// exactly what the reference's kernel leaves in it.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

namespace sbg
{
  namespace
  {
    template <typename T>
    __global__ void clear_skipped_kernel(T* tile, uint64_t h, uint64_t w, uint64_t r0, uint64_t c0, bool keep_diag)
    {
      const uint64_t total = h * w;
      for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (uint64_t)gridDim.x * blockDim.x)
      {
        const uint64_t i = r0 + k / w, j = c0 + k % w;
        if (j > i || (!keep_diag && j == i)) tile[k] = T(0);
      }
    }

    template <typename T>
    void block_device(int op, double p, int skip, const T* rpts, const uint64_t* roff, const T* cpts,
                      const uint64_t* coff, uint64_t r0, uint64_t h, uint64_t c0, uint64_t w, uint32_t lmax, T* tile,
                      cudaStream_t st)
    {
      if (h == 0 || w == 0) return;
      PcfSet<T> rows{rpts, roff + r0, h};
      PcfSet<T> cols{cpts, coff + c0, w};
      compute_device<T>(MODE_CROSS, op, p, rows, &cols, nullptr, nullptr, lmax, tile, 0, 0, h, st);
      // a block reaching the diagonal or beyond has excluded entries
      if (skip != SBG_SKIP_NONE && c0 + w > r0)
      {
        const DeviceInfo dev = device_info();
        const unsigned blocks = (unsigned)std::min<uint64_t>((h * w + 255) / 256, (uint64_t)dev.sms * 8);
        clear_skipped_kernel<T><<<blocks, 256, 0, st>>>(tile, h, w, r0, c0, skip == SBG_SKIP_LOWER);
        SBG_CUDA(launched());
      }
    }
  }
}

using namespace sbg;

extern "C" int sbg_block_device(int dtype, int op, double p, int skip_mode, const void* row_points,
                                const uint64_t* row_offsets, const void* col_points, const uint64_t* col_offsets,
                                uint64_t row_start, uint64_t row_height, uint64_t col_start, uint64_t col_width,
                                uint32_t max_points, void* tile, void* stream)
{
  try
  {
    if (dtype != SBG_F32 && dtype != SBG_F64) throw Error(ST_INVALID_ARGUMENT, "dtype must be SBG_F32 or SBG_F64");
    if (skip_mode < SBG_SKIP_NONE || skip_mode > SBG_SKIP_LOWER) throw Error(ST_INVALID_ARGUMENT, "bad skip mode");
    if (op == SBG_OP_LP && !(p >= 1.0)) throw Error(ST_INVALID_ARGUMENT, "p must be >= 1.");
    if (row_height && col_width && (!row_points || !row_offsets || !col_points || !col_offsets || !tile))
      throw Error(ST_INVALID_ARGUMENT, "null pointer");
    if (max_points == 0) throw Error(ST_INVALID_ARGUMENT, "max_points must be given");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == SBG_F32)
      block_device<float>(op, p, skip_mode, static_cast<const float*>(row_points), row_offsets,
                          static_cast<const float*>(col_points), col_offsets, row_start, row_height, col_start,
                          col_width, max_points, static_cast<float*>(tile), st);
    else
      block_device<double>(op, p, skip_mode, static_cast<const double*>(row_points), row_offsets,
                           static_cast<const double*>(col_points), col_offsets, row_start, row_height, col_start,
                           col_width, max_points, static_cast<double*>(tile), st);
    set_last_error("");
    return ST_OK;
  }
  catch (const Error& e)
  {
    set_last_error(e.what());
    return e.status;
  }
  catch (const std::exception& e)
  {
    set_last_error(e.what());
    return ST_INTERNAL;
  }
}
