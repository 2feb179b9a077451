// Length order of a PCF set on the device: within each window of
// LENGTH_ORDER_WINDOW consecutive PCFs, the PCFs by increasing breakpoint
// count, ties by index (the same permutation as a stable host sort of each
// window).  Grouping columns of similar length keeps the warp-uniform step
// count of the pair kernels close to the work each lane does.  Sorting only
// within windows keeps the output locality: the 32 results of a warp land in
// one window of a condensed row, which the CTAs working on neighbouring
// column groups fill at the same time, so L2 writes whole sectors back (a
// global sort scatters every store and multiplied DRAM traffic ~9x).  The
// order is computed on the stream, with no host round trip.
//
// Keys (min(length, 2^32 - 1) << 10 | index in window) are unique within a
// window, so a bitonic network (not stable by itself) gives the one
// deterministic order.  Each window is keyed, sorted and written out by one
// CTA in shared memory, in one launch.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <algorithm>

namespace sbg
{
  namespace
  {
    constexpr int SORT_THREADS = LENGTH_ORDER_WINDOW / 2;  // one compare-exchange per thread and stage

    __device__ __forceinline__ void cmp_swap(uint64_t& a, uint64_t& b, bool ascending)
    {
      if ((a > b) == ascending)
      {
        const uint64_t t = a;
        a = b;
        b = t;
      }
    }

    // One CTA per window: keys (min(length, 2^32 - 1) << 10 | index in
    // window) built from the offsets, a bitonic network in shared memory,
    // the permutation written out.  A stage whose partner distance j is at
    // most 32 pairs elements inside the 64 that one warp handles, so it only
    // needs the warp's own barrier after a stage of the same kind; a block
    // barrier precedes every stage that crosses warps and the stage after it.
    // The last window is padded with all-ones keys, which sort last.
    __global__ void __launch_bounds__(SORT_THREADS) window_order_kernel(const uint64_t* __restrict__ off, uint64_t n,
                                                                        uint32_t* __restrict__ perm)
    {
      __shared__ uint64_t s[LENGTH_ORDER_WINDOW];
      const uint64_t base = (uint64_t)blockIdx.x * LENGTH_ORDER_WINDOW;
      for (uint32_t i = threadIdx.x; i < LENGTH_ORDER_WINDOW; i += SORT_THREADS)
      {
        const uint64_t g = base + i;
        uint64_t key = ~0ull;
        if (g < n)
        {
          uint64_t len = off[g + 1] - off[g];
          if (len > 0xffffffffull) len = 0xffffffffull;
          key = (len << 10) | i;
        }
        s[i] = key;
      }
      uint32_t prev_j = LENGTH_ORDER_WINDOW;  // the loads cross warps
      for (uint32_t k = 2; k <= LENGTH_ORDER_WINDOW; k <<= 1)
      {
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
        {
          if (j >= 64 || prev_j >= 64) __syncthreads(); else __syncwarp();
          const uint32_t t = threadIdx.x;
          const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1));  // j is a power of two
          cmp_swap(s[i], s[i + j], (i & k) == 0);
          prev_j = j;
        }
      }
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < LENGTH_ORDER_WINDOW; i += SORT_THREADS)
        if (base + i < n) perm[base + i] = (uint32_t)(base + (s[i] & 1023));
    }
  }

  static_assert(LENGTH_ORDER_WINDOW == 1024, "the key layout holds 10 bits of index within a window");

  // The order needs no global scratch; kept for callers that size one.
  uint64_t length_order_scratch_bytes(uint64_t) { return 0; }

  void length_order_device(const uint64_t* off, uint64_t n, uint32_t* perm, void*, cudaStream_t st)
  {
    if (n == 0) return;
    if (n > 0xffffffffull) throw Error(ST_INVALID_ARGUMENT, "too many PCFs for a 32-bit processing order");
    const uint64_t windows = (n + LENGTH_ORDER_WINDOW - 1) / LENGTH_ORDER_WINDOW;
    window_order_kernel<<<(unsigned)windows, SORT_THREADS, 0, st>>>(off, n, perm);
    SBG_CUDA(launched());
  }
}

extern "C" int sbg_length_order_device(const uint64_t* offsets, uint64_t n, uint32_t* perm, void* stream)
{
  using namespace sbg;
  try
  {
    if (n && (!offsets || !perm)) throw Error(ST_INVALID_ARGUMENT, "null pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n) length_order_device(offsets, n, perm, nullptr, st);
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
