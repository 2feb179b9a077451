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
// Keys (window << 42 | min(length, 2^32 - 1) << 10 | index in window) are
// unique, so a bitonic network (not stable by itself) gives the one
// deterministic order.  Each window is sorted by one CTA in shared memory;
// the last window is padded with all-ones keys, which sort last.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <algorithm>

namespace sbg
{
  namespace
  {
    constexpr int SORT_THREADS = 1024;
    constexpr uint64_t SORT_TILE = 2 * SORT_THREADS;

    __device__ __forceinline__ void cmp_swap(uint64_t& a, uint64_t& b, bool ascending)
    {
      if ((a > b) == ascending)
      {
        const uint64_t t = a;
        a = b;
        b = t;
      }
    }

    // Stages k = k_first .. k_last (powers of two) with partner distances
    // j = min(k / 2, j_first) .. 1, on one tile in shared memory.  Every tile
    // is sorted on its own, ascending: the direction of a comparison comes
    // from the index inside the tile.
    __global__ void __launch_bounds__(SORT_THREADS) tile_stages_kernel(uint64_t* keys, uint64_t n, uint64_t tile,
                                                                       uint64_t k_first, uint64_t k_last,
                                                                       uint64_t j_first)
    {
      __shared__ uint64_t s[SORT_TILE];
      const uint64_t base = (uint64_t)blockIdx.x * tile;
      for (uint64_t i = threadIdx.x; i < tile; i += blockDim.x) s[i] = keys[base + i];
      __syncthreads();
      for (uint64_t k = k_first; k <= k_last; k <<= 1)
      {
        for (uint64_t j = (k / 2 < j_first ? k / 2 : j_first); j > 0; j >>= 1)
        {
          for (uint64_t t = threadIdx.x; t < tile / 2; t += blockDim.x)
          {
            const uint64_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1));  // j is a power of two
            cmp_swap(s[i], s[i + j], (i & k) == 0);
          }
          __syncthreads();
        }
      }
      for (uint64_t i = threadIdx.x; i < tile; i += blockDim.x) keys[base + i] = s[i];
      (void)n;
    }

    __global__ void make_keys_kernel(const uint64_t* __restrict__ off, uint64_t n, uint64_t npad,
                                     uint64_t* __restrict__ keys)
    {
      for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npad; i += (uint64_t)gridDim.x * blockDim.x)
      {
        if (i < n)
        {
          uint64_t len = off[i + 1] - off[i];
          if (len > 0xffffffffull) len = 0xffffffffull;
          keys[i] = ((i >> 10) << 42) | (len << 10) | (i & 1023);
        }
        else keys[i] = ~0ull;
      }
    }

    __global__ void keys_to_perm_kernel(const uint64_t* __restrict__ keys, uint64_t n, uint32_t* __restrict__ perm)
    {
      for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        perm[i] = (uint32_t)(((keys[i] >> 42) << 10) | (keys[i] & 1023));
    }
  }

  static_assert(LENGTH_ORDER_WINDOW == 1024, "the key layout holds 10 bits of index within a window");
  static_assert(LENGTH_ORDER_WINDOW <= SORT_TILE, "a window is sorted inside one tile");

  // Keys padded to whole windows (or, below one window, to a power of two).
  static uint64_t padded_keys(uint64_t n)
  {
    if (n >= LENGTH_ORDER_WINDOW) return (n + LENGTH_ORDER_WINDOW - 1) / LENGTH_ORDER_WINDOW * LENGTH_ORDER_WINDOW;
    uint64_t npad = 1;
    while (npad < n) npad <<= 1;
    return npad;
  }

  uint64_t length_order_scratch_bytes(uint64_t n) { return padded_keys(n) * sizeof(uint64_t); }

  void length_order_device(const uint64_t* off, uint64_t n, uint32_t* perm, void* scratch, cudaStream_t st)
  {
    if (n == 0) return;
    if (n > 0xffffffffull) throw Error(ST_INVALID_ARGUMENT, "too many PCFs for a 32-bit processing order");
    const uint64_t npad = padded_keys(n);
    uint64_t* keys = static_cast<uint64_t*>(scratch);
    const unsigned blocks = (unsigned)std::min<uint64_t>((npad + 255) / 256, 4096);
    make_keys_kernel<<<blocks, 256, 0, st>>>(off, n, npad, keys);
    SBG_CUDA(launched());
    // The window sits in the keys' high bits, so sorting every window on its
    // own (one tile each) is the whole sort.
    const uint64_t tile = npad < LENGTH_ORDER_WINDOW ? npad : LENGTH_ORDER_WINDOW;
    if (tile >= 2)
    {
      tile_stages_kernel<<<(unsigned)(npad / tile), SORT_THREADS, 0, st>>>(keys, npad, tile, 2, tile, tile / 2);
      SBG_CUDA(launched());
    }
    keys_to_perm_kernel<<<blocks, 256, 0, st>>>(keys, n, perm);
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
    void* keys = nullptr;
    if (n)
    {
      SBG_CUDA(cudaMallocAsync(&keys, length_order_scratch_bytes(n), st));
      struct Free { void* p; cudaStream_t s; ~Free() { cudaFreeAsync(p, s); } } guard{keys, st};
      length_order_device(offsets, n, perm, keys, st);
    }
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
