// Issue-rate probes reported beside the roofline: sustained FP32 FFMA and
// FP64 DFMA lane-operations per second on the current device.  Each thread
// runs 8 independent FMA chains (enough ILP to keep the pipe full), unrolled
// 32 times so the loop's own instructions are under 1 % of those issued,
// and ten launches of about 4 ms each keep the gaps between launches small;
// one FMA instruction per lane counts as one lane-op.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

namespace sbg
{
  template <typename T, int ITERS>
  __global__ void __launch_bounds__(256) fma_rate_kernel(T seed, T* sink)
  {
    T a0 = seed + T(threadIdx.x), a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
    T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
    const T m = T(0.999999), c = T(1e-7);
#pragma unroll 32
    for (int i = 0; i < ITERS; ++i)
    {
      a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
      a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
    const T s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == T(-1)) sink[threadIdx.x] = s;  // never true; keeps the chains live
  }

  template <typename T, int ITERS>
  static double measure(int blocks_per_sm)
  {
    const DeviceInfo dev = device_info();
    const int blocks = dev.sms * blocks_per_sm;
    DeviceBuffer sink(256 * sizeof(T));
    cudaEvent_t e0, e1;
    SBG_CUDA(cudaEventCreate(&e0));
    SBG_CUDA(cudaEventCreate(&e1));
    for (int w = 0; w < 2; ++w) fma_rate_kernel<T, ITERS><<<blocks, 256>>>(T(1), sink.as<T>());
    SBG_CUDA(launched());
    count_launches(1);
    SBG_CUDA(cudaEventRecord(e0));
    const int reps = 10;
    for (int r = 0; r < reps; ++r) fma_rate_kernel<T, ITERS><<<blocks, 256>>>(T(1), sink.as<T>());
    SBG_CUDA(launched());
    count_launches(reps - 1);
    SBG_CUDA(cudaEventRecord(e1));
    SBG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    SBG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double ops = (double)reps * blocks * 256.0 * ITERS * 8.0;
    return ops / (ms * 1e-3);
  }
}

extern "C" int sbg_measure_peak(int kind, double* lane_ops_per_s)
{
  try
  {
    if (!lane_ops_per_s) throw sbg::Error(sbg::ST_INVALID_ARGUMENT, "null output");
    if (kind == 0) *lane_ops_per_s = sbg::measure<float, 1 << 16>(8);
    else if (kind == 1) *lane_ops_per_s = sbg::measure<double, 1 << 9>(8);
    else throw sbg::Error(sbg::ST_INVALID_ARGUMENT, "kind must be 0 (fp32) or 1 (fp64)");
    sbg::set_last_error("");
    return SBG_OK;
  }
  catch (const sbg::Error& e)
  {
    sbg::set_last_error(e.what());
    return e.status;
  }
}
