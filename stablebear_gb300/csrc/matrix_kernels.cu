// Device-resident consumers and producers of the condensed results.
//
// The reference turns a DistanceMatrix / SymmetricMatrix into a dense n x n
// array with a serial host loop over all n^2 entries
// (src/python/py_distance_matrix.hpp:37-49, py_symmetric_matrix.hpp), and
// builds one from a dense array with another host loop that checks the
// diagonal, sign and symmetry (py_distance_matrix.hpp:50-73).  Here both run
// on the GPU over HBM-resident data:
//
//   condensed_to_dense: rows [row_begin, row_end) of the dense matrix;
//   dense_to_condensed: the whole condensed storage, with the reference's
//                       checks reported as flags.
//
// Both work on 32 x 32 tiles of the lower triangle.  A tile (a, b), a >= b,
// is read once, coalesced along its columns, into shared memory and written
// as the dense tile (a, b) and, transposed through shared memory, as the
// dense tile (b, a): each condensed value is read once and both of its dense
// copies are written once, which is the algorithmic traffic.  The kernels
// are HBM-bound; CTAs loop over tiles (grid = a multiple of the SM count).
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <cmath>

namespace sbg
{
  namespace
  {
    constexpr int ROWS = 8;  // thread rows per CTA: TD x 8 threads, TD / 8 rows of a TD-wide tile each
#ifndef D2C_TILE
#define D2C_TILE 64
#endif
// condensed -> dense keeps two 32-wide tiles per iteration: its writes
// merge in L2, and one 64-wide tile measured slower (12.2 against 11.7 ms
// at N = 100,000)
#ifndef C2D_TILE
#define C2D_TILE 32
#endif

    __device__ __forceinline__ uint64_t cond_index(bool diag, uint64_t i, uint64_t j)
    {
      return diag ? i * (i + 1) / 2 + j : i * (i - 1) / 2 + j;  // i >= j (i > j without the diagonal)
    }

    // Tiles (a, b) with a >= b that touch the row band of block rows
    // [Bb, Be): first every tile whose row block a lies in the band (b <= a),
    // then every tile below the band whose column block b lies in it.
    struct TileSet
    {
      uint64_t Bb, Be, nb;
      uint64_t base;    // Bb (Bb + 1) / 2: tiles of the rows before the band
      uint64_t count1;  // tiles with a in [Bb, Be)
      uint64_t count;   // all tiles

      __host__ __device__ void init(uint64_t Bb_, uint64_t Be_, uint64_t nb_)
      {
        Bb = Bb_; Be = Be_; nb = nb_;
        base = Bb * (Bb + 1) / 2;
        count1 = Be * (Be + 1) / 2 - base;
        count = count1 + (Be - Bb) * (nb - Be);
      }

      __device__ void decode(uint64_t k, uint64_t* a, uint64_t* b) const
      {
        if (k < count1)
        {
          const uint64_t g = base + k;  // index in the full lower-triangle order
          // FP32 estimate (FP64 is a slow pipe here), then exact correction
          uint64_t r = (uint64_t)((sqrtf(8.0f * (float)g + 1.0f) - 1.0f) * 0.5f);
          while (r * (r + 1) / 2 > g) --r;
          while ((r + 1) * (r + 2) / 2 <= g) ++r;
          *a = r;
          *b = g - r * (r + 1) / 2;
        }
        else
        {
          const uint64_t k2 = k - count1, w = Be - Bb;
          *a = Be + k2 / w;
          *b = Bb + k2 % w;
        }
      }
    };

    // NT tiles of TD x TD per CTA iteration, all loaded before the barrier,
    // so each thread keeps NT * TD / ROWS loads in flight (eight for both
    // shapes used: two 32-wide tiles, or one 64-wide tile whose row pieces,
    // read and written, are 256 contiguous bytes instead of 128).
    template <typename T, int TD, int NT>
    __global__ void __launch_bounds__(TD * ROWS) condensed_to_dense_kernel(
        const T* __restrict__ cond, uint64_t n, bool diag, T* __restrict__ dense, uint64_t ld,
        uint64_t row_begin, uint64_t row_end, TileSet ts)
    {
      __shared__ T tile[NT][TD][TD + 1];
      const int tx = threadIdx.x, ty = threadIdx.y;
      for (uint64_t k0 = (uint64_t)NT * blockIdx.x; k0 < ts.count; k0 += (uint64_t)NT * gridDim.x)
      {
        uint64_t a[NT], b[NT];
        const int nt = k0 + NT <= ts.count ? NT : (int)(ts.count - k0);
        T v[NT][TD / ROWS];
#pragma unroll
        for (int u = 0; u < NT; ++u)
        {
          if (u < nt) ts.decode(k0 + u, &a[u], &b[u]);
          else { a[u] = 0; b[u] = 0; }
          const uint64_t i0 = a[u] * TD, j = b[u] * TD + tx;
          if (u < nt && a[u] > b[u] && i0 + TD <= n)
          {
            // interior tile: every element exists, no per-element checks;
            // consecutive rows' starts differ by i (+1 with the diagonal)
            uint64_t i = i0 + ty;
            const T* src = cond + cond_index(diag, i, 0) + j;
#pragma unroll
            for (int q = 0; q < TD / ROWS; ++q)
            {
              v[u][q] = src[0];
              // start of row i + ROWS minus start of row i
              src += ROWS * i + (diag ? ROWS * (ROWS + 1) / 2 : ROWS * (ROWS - 1) / 2);
              i += ROWS;
            }
          }
          else
          {
#pragma unroll
            for (int q = 0; q < TD / ROWS; ++q)
            {
              const uint64_t i = i0 + ty + q * ROWS;
              v[u][q] = (u < nt && i < n && j < n && (j < i || (diag && j == i))) ? cond[cond_index(diag, i, j)] : T(0);
            }
          }
        }
#pragma unroll
        for (int u = 0; u < NT; ++u)
#pragma unroll
          for (int q = 0; q < TD / ROWS; ++q) tile[u][ty + q * ROWS][tx] = v[u][q];
        __syncthreads();
        for (int u = 0; u < nt; ++u)
        {
          const uint64_t i0 = a[u] * TD, j0 = b[u] * TD;
          if (a[u] > b[u] && i0 + TD <= n && j0 >= row_begin && i0 + TD <= row_end)
          {
            // interior tile with both copies inside the band (the band is
            // contiguous and j0 < i0): plain row-pointer walks
            T* d1 = dense + (i0 + ty - row_begin) * ld + j0 + tx;
            T* d2 = dense + (j0 + ty - row_begin) * ld + i0 + tx;
#pragma unroll
            for (int q = 0; q < TD / ROWS; ++q)
            {
              const int r = ty + q * ROWS;
              d1[0] = tile[u][r][tx];
              d2[0] = tile[u][tx][r];
              d1 += ROWS * ld;
              d2 += ROWS * ld;
            }
            continue;
          }
          // dense tile (a, b): rows of block a inside the band; on the
          // diagonal tile the upper half is the transposed lower half
          for (int r = ty; r < TD; r += ROWS)
          {
            const uint64_t i = i0 + r, j = j0 + tx;
            if (i >= row_begin && i < row_end && j < n)
              dense[(i - row_begin) * ld + j] = (a[u] != b[u] || tx <= r) ? tile[u][r][tx] : tile[u][tx][r];
          }
          // dense tile (b, a), a > b: the transpose
          if (a[u] != b[u])
          {
            for (int r = ty; r < TD; r += ROWS)
            {
              const uint64_t i = j0 + r, j = i0 + tx;
              if (i >= row_begin && i < row_end && j < n) dense[(i - row_begin) * ld + j] = tile[u][tx][r];
            }
          }
        }
        __syncthreads();
      }
    }

    // Flags (bit set = violated somewhere): 1 not symmetric, 2 non-zero
    // diagonal (distance matrices), 4 negative entry (distance matrices).
    // FOLD: no checks; each stored entry receives dense[i][j] + dense[j][i]
    // (the diagonal itself for symmetric-matrix storage), the adjoint of the
    // symmetric expansion, which gradients through it need.
    // TD x TD tiles (TD = 64: each row piece of a tile, and of its mirror,
    // is 256 contiguous bytes read by two warps, against 128 with 32-wide
    // tiles; the reads of the two triangles dominate this kernel's traffic).
    template <typename T, int TD, bool FOLD = false>
    __global__ void __launch_bounds__(TD * ROWS) dense_to_condensed_kernel(
        const T* __restrict__ dense, uint64_t n, uint64_t ld, bool diag, T* __restrict__ cond,
        unsigned int* __restrict__ flags, TileSet ts)
    {
      __shared__ T upper[TD][TD + 1];
      const int tx = threadIdx.x, ty = threadIdx.y;
      unsigned int f = 0;
      for (uint64_t k = blockIdx.x; k < ts.count; k += gridDim.x)
      {
        uint64_t a, b;
        ts.decode(k, &a, &b);
        const uint64_t i0 = a * TD, j0 = b * TD;
        if (a > b && i0 + TD <= n)
        {
          // interior tile: no bound checks, row-pointer walks, and the
          // condensed row starts advance by i (+1 with the diagonal)
          const T* up = dense + (j0 + ty) * ld + i0 + tx;
          const T* lo = dense + (i0 + ty) * ld + j0 + tx;
          T low[TD / ROWS];
#pragma unroll
          for (int q = 0; q < TD / ROWS; ++q)
          {
            upper[tx][ty + q * ROWS] = up[0];
            low[q] = lo[0];
            up += ROWS * ld;
            lo += ROWS * ld;
          }
          __syncthreads();
          uint64_t i = i0 + ty;
          T* dst = cond + cond_index(diag, i, 0) + j0 + tx;
#pragma unroll
          for (int q = 0; q < TD / ROWS; ++q)
          {
            const T v = low[q];
            if constexpr (FOLD)
              dst[0] = v + upper[ty + q * ROWS][tx];
            else
            {
              if (!(v == upper[ty + q * ROWS][tx])) f |= 1u;
              if (!diag && v < T(0)) f |= 4u;
              dst[0] = v;
            }
            dst += ROWS * i + (diag ? ROWS * (ROWS + 1) / 2 : ROWS * (ROWS - 1) / 2);
            i += ROWS;
          }
          __syncthreads();
          continue;
        }
        // The mirror tile (b, a), read coalesced and kept transposed, and
        // this thread's values of the lower tile, all loads before the barrier.
        T low[TD / ROWS];
#pragma unroll
        for (int q = 0; q < TD / ROWS; ++q)
        {
          const int r = ty + q * ROWS;
          const uint64_t i = j0 + r, j = i0 + tx;
          upper[tx][r] = (i < n && j < n) ? dense[i * ld + j] : T(0);
          const uint64_t li = i0 + r, lj = j0 + tx;
          low[q] = (li < n && lj < n && lj <= li) ? dense[li * ld + lj] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < TD / ROWS; ++q)
        {
          const int r = ty + q * ROWS;
          const uint64_t i = i0 + r, j = j0 + tx;
          if (FOLD && i < n && j < n && j <= i)
          {
            // the adjoint of the symmetric expansion: both mirror entries
            // flow into the one stored value, the diagonal into itself
            if (j == i)
            {
              if (diag) cond[cond_index(true, i, j)] = low[q];
            }
            else
              cond[cond_index(diag, i, j)] = low[q] + upper[r][tx];
          }
          else if (!FOLD && i < n && j < n && j <= i)
          {
            const T v = low[q];
            if (!(v == upper[r][tx])) f |= 1u;  // NaN counts as asymmetric, as != does in the reference
            if (j == i)
            {
              if (diag) cond[cond_index(true, i, j)] = v;
              else if (v != T(0)) f |= 2u;
            }
            else
            {
              if (!diag && v < T(0)) f |= 4u;
              cond[cond_index(diag, i, j)] = v;
            }
          }
        }
        __syncthreads();
      }
      if constexpr (!FOLD)
      {
        f = __reduce_or_sync(0xffffffffu, f);
        if (f && (threadIdx.x & 31) == 0) atomicOr(flags, f);
      }
    }

    template <typename F>
    int abi_call(F&& f)
    {
      try
      {
        f();
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

    void check_kind(int dtype, int skip)
    {
      if (dtype != SBG_F32 && dtype != SBG_F64) throw Error(ST_INVALID_ARGUMENT, "dtype must be SBG_F32 or SBG_F64");
      if (skip != SBG_SKIP_LOWER_NODIAG && skip != SBG_SKIP_LOWER)
        throw Error(ST_INVALID_ARGUMENT, "skip must be SBG_SKIP_LOWER_NODIAG (DistanceMatrix) or SBG_SKIP_LOWER "
                                         "(SymmetricMatrix)");
    }
  }
}

using namespace sbg;

extern "C"
{
  int sbg_condensed_to_dense_device(int dtype, int skip, uint64_t n, const void* condensed, void* dense, uint64_t ld,
                                    uint64_t row_begin, uint64_t row_end, void* stream)
  {
    return abi_call([&] {
      check_kind(dtype, skip);
      if (row_end > n) row_end = n;
      if (row_begin >= row_end) return;
      if (ld < n) throw Error(ST_INVALID_ARGUMENT, "ld must be >= n");
      if (!dense || (!condensed && output_count(skip, n, n) > 0))
        throw Error(ST_INVALID_ARGUMENT, "null matrix pointer");
      constexpr int TD = C2D_TILE, NT = C2D_TILE == 32 ? 2 : 1;
      const uint64_t nb = ceil_div_u64(n, TD);
      TileSet ts;
      ts.init(row_begin / TD, ceil_div_u64(row_end, TD), nb);
      const bool diag = skip == SBG_SKIP_LOWER;
      cudaStream_t st = (cudaStream_t)stream;
      const dim3 block(TD, ROWS);
      const uint64_t iters = (ts.count + NT - 1) / NT;
      const int grid = (int)std::min<uint64_t>(std::max<uint64_t>(iters, 1),
                                               (uint64_t)device_info().sms * (2048 / (TD * ROWS)));
      if (dtype == SBG_F32)
        condensed_to_dense_kernel<float, TD, NT><<<grid, block, 0, st>>>((const float*)condensed, n, diag,
                                                                          (float*)dense, ld, row_begin, row_end, ts);
      else
        condensed_to_dense_kernel<double, TD, NT><<<grid, block, 0, st>>>((const double*)condensed, n, diag,
                                                                           (double*)dense, ld, row_begin, row_end, ts);
      SBG_CUDA(launched());
    });
  }

  int sbg_dense_to_condensed_device(int dtype, int skip, uint64_t n, const void* dense, uint64_t ld, void* condensed,
                                    unsigned int* flags, void* stream)
  {
    return abi_call([&] {
      check_kind(dtype, skip);
      if (!flags) throw Error(ST_INVALID_ARGUMENT, "flags must point to a device word");
      if (n == 0) return;
      if (ld < n) throw Error(ST_INVALID_ARGUMENT, "ld must be >= n");
      if (!dense || (!condensed && output_count(skip, n, n) > 0))
        throw Error(ST_INVALID_ARGUMENT, "null matrix pointer");
      constexpr int TD = D2C_TILE;
      const uint64_t nb = ceil_div_u64(n, TD);
      TileSet ts;
      ts.init(0, nb, nb);
      cudaStream_t st = (cudaStream_t)stream;
      const dim3 block(TD, ROWS);
      // 8 x 256 threads per SM at TD = 32; the same threads in 4 x 512 at 64
      const int grid = (int)std::min<uint64_t>(std::max<uint64_t>(ts.count, 1),
                                               (uint64_t)device_info().sms * (2048 / (TD * ROWS)));
      const bool diag = skip == SBG_SKIP_LOWER;
      if (dtype == SBG_F32)
        dense_to_condensed_kernel<float, TD><<<grid, block, 0, st>>>((const float*)dense, n, ld, diag,
                                                                      (float*)condensed, flags, ts);
      else
        dense_to_condensed_kernel<double, TD><<<grid, block, 0, st>>>((const double*)dense, n, ld, diag,
                                                                       (double*)condensed, flags, ts);
      SBG_CUDA(launched());
    });
  }

  int sbg_dense_fold_to_condensed_device(int dtype, int skip, uint64_t n, const void* dense, uint64_t ld,
                                         void* condensed, void* stream)
  {
    return abi_call([&] {
      check_kind(dtype, skip);
      if (n == 0) return;
      if (ld < n) throw Error(ST_INVALID_ARGUMENT, "ld must be >= n");
      if (!dense || (!condensed && output_count(skip, n, n) > 0))
        throw Error(ST_INVALID_ARGUMENT, "null matrix pointer");
      constexpr int TD = D2C_TILE;
      const uint64_t nb = ceil_div_u64(n, TD);
      TileSet ts;
      ts.init(0, nb, nb);
      cudaStream_t st = (cudaStream_t)stream;
      const dim3 block(TD, ROWS);
      const int grid = (int)std::min<uint64_t>(std::max<uint64_t>(ts.count, 1),
                                               (uint64_t)device_info().sms * (2048 / (TD * ROWS)));
      const bool diag = skip == SBG_SKIP_LOWER;
      if (dtype == SBG_F32)
        dense_to_condensed_kernel<float, TD, true><<<grid, block, 0, st>>>((const float*)dense, n, ld, diag,
                                                                            (float*)condensed, nullptr, ts);
      else
        dense_to_condensed_kernel<double, TD, true><<<grid, block, 0, st>>>((const double*)dense, n, ld, diag,
                                                                             (double*)condensed, nullptr, ts);
      SBG_CUDA(launched());
    });
  }
}
