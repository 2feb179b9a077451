// Lp norms of single PCFs: ||f||_p = (integral over [0, inf) of |f(t)|^p dt)^(1/p),
// the reference's l1_norm / lp_norm (include/sbear/algorithms/functional/
// apply_functional.hpp:63-100) over its iterate_segments
// (algorithms/functional/iterate_rectangles.hpp:106-155), which the reference
// runs on the CPU only (src/python/functional/py_norms.cpp:24-46).
//
// Segments follow iterate_segments with a = 0 and b = numeric_limits<T>::max():
//   * the first segment starts at the last breakpoint with t <= 0, so the
//     zero-width segments between repeated t = 0 breakpoints are skipped;
//   * segment k is [t_k, min(t_{k+1}, b)) with value v_k, the last one
//     [t_last, b); the walk stops after the first segment that reaches b,
//     i.e. segment k counts only while t_k < b.
// p = 1 sums (r - l) |v|; any other p sums (r - l) pow(|v|, p) and returns
// pow(sum, 1/p), as the reference does (it uses pow for p = 2 too).
//
// One warp per PCF: lanes take segments k = lane, lane + 32, ... (coalesced
// breakpoint reads) and the 32 partial sums are added with shuffles.  The
// kernel reads each breakpoint once and writes one value per PCF: it is
// HBM-bound.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <cmath>

namespace sbg
{
  namespace
  {
    template <typename T>
    __global__ void __launch_bounds__(256) lp_norm_kernel(const T* __restrict__ pts, const uint64_t* __restrict__ off,
                                                          uint64_t n, T p, bool l1, T* __restrict__ out)
    {
      const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
      const int lane = threadIdx.x & 31;
      if (warp >= n) return;  // whole warps leave together
      const uint64_t a = off[warp], b = off[warp + 1];
      const uint64_t L = b - a;
      const T* P = pts + 2 * a;
      const T B = tmax_of<T>();
      T sum = T(0);
      for (uint64_t k = lane; k < L; k += 32)
      {
        const T tk = P[2 * k], vk = P[2 * k + 1];
        const T tn = k + 1 < L ? P[2 * (k + 1)] : B;
        // k < first index with t > 0, minus one: a zero-width segment before the start
        if (k + 1 < L && !(tn > T(0))) continue;
        if (!(tk < B)) continue;  // past the segment that reached b
        const T left = tk > T(0) ? tk : T(0);
        const T right = tn < B ? tn : B;
        const T w = right - left;
        const T av = fabs(vk);
        sum += w * (l1 ? av : pow(av, p));
      }
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
      if (lane == 0) out[warp] = (L == 0) ? T(0) : (l1 ? sum : pow(sum, T(1) / p));
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

    template <typename T>
    void launch_norm(const void* pts, const uint64_t* off, uint64_t n, double p, void* out, cudaStream_t st)
    {
      if (n == 0) return;
      const uint64_t threads = n * 32;
      const unsigned grid = (unsigned)ceil_div_u64(threads, 256);
      lp_norm_kernel<T><<<grid, 256, 0, st>>>((const T*)pts, off, n, (T)p, p == 1.0, (T*)out);
      SBG_CUDA(launched());
    }

    void check_norm_args(int dtype, double p)
    {
      if (dtype != SBG_F32 && dtype != SBG_F64) throw Error(ST_INVALID_ARGUMENT, "dtype must be SBG_F32 or SBG_F64");
      if (!(p >= 1.0)) throw Error(ST_INVALID_ARGUMENT, "p must be >= 1.");
    }
  }
}

using namespace sbg;

extern "C"
{
  int sbg_lp_norm_device(int dtype, double p, const void* points, const uint64_t* offsets, uint64_t n, void* out,
                         void* stream)
  {
    return abi_call([&] {
      check_norm_args(dtype, p);
      if (n == 0) return;
      if (!points || !offsets || !out) throw Error(ST_INVALID_ARGUMENT, "null pointer");
      if (n > (uint64_t)UINT32_MAX * 8) throw Error(ST_INVALID_ARGUMENT, "too many PCFs for one launch");
      if (dtype == SBG_F32) launch_norm<float>(points, offsets, n, p, out, (cudaStream_t)stream);
      else launch_norm<double>(points, offsets, n, p, out, (cudaStream_t)stream);
    });
  }

  int sbg_lp_norm_host(int dtype, double p, const void* points, const uint64_t* offsets, uint64_t n, void* out)
  {
    return abi_call([&] {
      check_norm_args(dtype, p);
      if (n == 0) return;
      if (!points || !offsets || !out) throw Error(ST_INVALID_ARGUMENT, "null pointer");
      const size_t es = dtype == SBG_F32 ? 4 : 8;
      if (dtype == SBG_F32) validate_pcfs(PcfSet<float>{(const float*)points, offsets, n}, "lp_norm");
      else validate_pcfs(PcfSet<double>{(const double*)points, offsets, n}, "lp_norm");
      const uint64_t npts = offsets[n];
      cudaStream_t st;
      SBG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{st};
      DeviceBuffer dp(npts * 2 * es), doff((n + 1) * sizeof(uint64_t)), dout(n * es);
      if (npts) SBG_CUDA(cudaMemcpyAsync(dp.get(), points, npts * 2 * es, cudaMemcpyHostToDevice, st));
      SBG_CUDA(cudaMemcpyAsync(doff.get(), offsets, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
      if (dtype == SBG_F32) launch_norm<float>(dp.get(), (const uint64_t*)doff.get(), n, p, dout.get(), st);
      else launch_norm<double>(dp.get(), (const uint64_t*)doff.get(), n, p, dout.get(), st);
      SBG_CUDA(cudaMemcpyAsync(out, dout.get(), n * es, cudaMemcpyDeviceToHost, st));
      SBG_CUDA(cudaStreamSynchronize(st));
    });
  }
}
