// Barcodes to PCFs on the GPU: stable rank and Betti curve, the producers
// that feed the pairwise path (barcodes -> PCFs -> l2_kernel / pdist) without
// a host round trip.  The reference converts one barcode at a time on the CPU
// (include/sbear/persistence/stable_rank.hpp:17-66,
// include/sbear/persistence/betti_curve.hpp:21-84).
//
// Stable rank of a barcode with m bars and lifetimes l (death - birth, or
// numeric_limits<T>::max() when death is that value), sorted ascending: the
// points are (0, m) and, for every distinct finite lifetime u in increasing
// order, (u, #{l > u}).  "Finite" is the reference's is_infinite test (not
// +inf and not max).  This is what the reference's loop emits: it writes the
// previous run's lifetime with the count of longer bars whenever the lifetime
// changes, stops at the first infinite lifetime, and closes a finite last run.
//
// Betti curve: events +1 at every birth and -1 at every finite death, sorted
// by time.  With d_1 < d_2 < ... the distinct event times and C(d) the sum of
// the events at times <= d, the points are (0, 0) when d_1 != 0, then
// (d_k, C(d_k)) for every k: the reference emits (last time, count) whenever
// the time changes, starting from time 0 with count 0, and once at the end.
// The order of events at equal times does not change these points.
//
// An empty barcode gives the default PCF, the single point (0, 0).
//
// One CTA per barcode (a persistent loop over barcodes): the keys are sorted
// with a bitonic network in shared memory, or in global scratch when the
// barcode is longer than the shared block, then one CTA-wide scan finds the
// runs and writes the points at a per-barcode upper bound (m + 1 points for
// the stable rank, 2m + 1 for the Betti curve).  A scan of the point counts
// gives the output offsets and a last kernel packs the points.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <algorithm>
#include <limits>

namespace sbg
{
  namespace
  {
    constexpr int PB_THREADS = 256;

    template <typename T>
    struct PKey
    {
      T t;
      int d;  // event weight (+1 / -1); 2 marks padding, which sorts after every real key
    };

    // Keys sorted in shared memory (32 KB); longer barcodes use global scratch.
    template <typename T>
    struct SmemKeys { static constexpr uint32_t value = 32768 / sizeof(PKey<T>); };

    template <typename T>
    __device__ __forceinline__ bool key_less(const PKey<T>& a, const PKey<T>& b)
    {
      if (a.t < b.t) return true;
      if (b.t < a.t) return false;
      return (a.d == 2 ? 1 : 0) < (b.d == 2 ? 1 : 0);
    }

    template <typename T>
    __device__ __forceinline__ bool is_infinite(T v)
    {
      return v == std::numeric_limits<T>::infinity() || v == std::numeric_limits<T>::max();
    }

    // Ascending bitonic sort of npad (a power of two) keys by one CTA.
    template <typename T>
    __device__ void cta_bitonic_sort(PKey<T>* s, uint32_t npad)
    {
      for (uint32_t k = 2; k <= npad; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
        {
          for (uint32_t t = threadIdx.x; t < npad / 2; t += blockDim.x)
          {
            const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
            const bool asc = (i & k) == 0;
            PKey<T> a = s[i], b = s[i + j];
            if (key_less(b, a) == asc)
            {
              s[i] = b;
              s[i + j] = a;
            }
          }
          __syncthreads();
        }
    }

    // Exclusive scan of one (count, sum) pair per thread across the CTA.
    __device__ void cta_scan2(int& cnt, long long& sum, int* s_cnt, long long* s_sum)
    {
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
      int c = cnt;
      long long v = sum;
      for (int o = 1; o < 32; o <<= 1)
      {
        const int c2 = __shfl_up_sync(0xffffffffu, c, o);
        const long long v2 = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) { c += c2; v += v2; }
      }
      if (lane == 31) { s_cnt[warp] = c; s_sum[warp] = v; }
      __syncthreads();
      if (warp == 0)
      {
        int wc = lane < nw ? s_cnt[lane] : 0;
        long long wv = lane < nw ? s_sum[lane] : 0;
        for (int o = 1; o < 32; o <<= 1)
        {
          const int c2 = __shfl_up_sync(0xffffffffu, wc, o);
          const long long v2 = __shfl_up_sync(0xffffffffu, wv, o);
          if (lane >= o) { wc += c2; wv += v2; }
        }
        if (lane < nw) { s_cnt[lane] = wc; s_sum[lane] = wv; }
      }
      __syncthreads();
      const int wbase_c = warp ? s_cnt[warp - 1] : 0;
      const long long wbase_v = warp ? s_sum[warp - 1] : 0;
      cnt = wbase_c + c - cnt;  // exclusive
      sum = wbase_v + v - sum;
      __syncthreads();
    }

    template <typename T, int KIND>
    __global__ void __launch_bounds__(PB_THREADS) barcode_summary_kernel(
        const T* __restrict__ bars, const uint64_t* __restrict__ boff, uint64_t n, PKey<T>* __restrict__ gscratch,
        T* __restrict__ padded, uint32_t* __restrict__ counts)
    {
      constexpr uint32_t SMK = SmemKeys<T>::value;
      __shared__ PKey<T> skeys[SMK];
      __shared__ int s_cnt[PB_THREADS / 32];
      __shared__ long long s_sum[PB_THREADS / 32];
      const T TMAXV = std::numeric_limits<T>::max();
      for (uint64_t bi = blockIdx.x; bi < n; bi += gridDim.x)
      {
        const uint64_t b0 = boff[bi], m = boff[bi + 1] - b0;
        const T* B = bars + 2 * b0;
        // upper bound layout of the padded output
        T* P = padded + 2 * (KIND == 0 ? b0 + bi : 2 * b0 + bi);
        if (m == 0)
        {
          if (threadIdx.x == 0) { P[0] = T(0); P[1] = T(0); counts[bi] = 1; }
          continue;
        }
        const uint64_t nk = KIND == 0 ? m : 2 * m;  // keys before dropping infinite deaths
        uint32_t npad = 1;
        while (npad < nk) npad <<= 1;
        PKey<T>* K = npad <= SMK ? skeys : gscratch + 4 * b0;  // 4 m >= npad for Betti keys
        for (uint32_t k = threadIdx.x; k < npad; k += blockDim.x)
        {
          PKey<T> e;
          e.t = std::numeric_limits<T>::infinity();
          e.d = 2;
          if (KIND == 0)
          {
            if (k < m)
            {
              const T birth = B[2 * k], death = B[2 * k + 1];
              e.t = death == TMAXV ? TMAXV : death - birth;
              e.d = 0;
            }
          }
          else if (k < 2 * m)
          {
            const uint64_t bar = k >> 1;
            const T birth = B[2 * bar], death = B[2 * bar + 1];
            if ((k & 1) == 0) { e.t = birth; e.d = 1; }
            else if (!is_infinite(death)) { e.t = death; e.d = -1; }
          }
          K[k] = e;
        }
        __syncthreads();
        cta_bitonic_sort(K, npad);

        // real keys: the first m (stable rank) or the non-padding ones (Betti)
        uint32_t nreal = (uint32_t)m;
        if (KIND == 1)
        {
          int c = 0;
          for (uint32_t k = threadIdx.x; k < npad; k += blockDim.x) c += K[k].d != 2;
          c = __reduce_add_sync(0xffffffffu, c);
          if ((threadIdx.x & 31) == 0) s_cnt[threadIdx.x >> 5] = c;
          __syncthreads();
          if (threadIdx.x == 0)
          {
            int tot = 0;
            for (int w = 0; w < PB_THREADS / 32; ++w) tot += s_cnt[w];
            s_cnt[0] = tot;
          }
          __syncthreads();
          nreal = (uint32_t)s_cnt[0];
          __syncthreads();
        }

        // contiguous chunk of keys per thread
        const uint32_t per = (nreal + blockDim.x - 1) / blockDim.x;
        const uint32_t k0 = min(nreal, threadIdx.x * per), k1 = min(nreal, k0 + per);
        int emit = 0;
        long long dsum = 0;
        for (uint32_t k = k0; k < k1; ++k)
        {
          const bool runend = k + 1 == nreal || K[k + 1].t != K[k].t;
          if (KIND == 0) emit += (runend && !is_infinite(K[k].t)) ? 1 : 0;
          else { emit += runend ? 1 : 0; dsum += K[k].d; }
        }
        int epos = emit;
        long long dpre = dsum;
        cta_scan2(epos, dpre, s_cnt, s_sum);
        const int lead = KIND == 0 ? 1 : (K[0].t != T(0) ? 1 : 0);
        if (threadIdx.x == 0)
        {
          if (KIND == 0) { P[0] = T(0); P[1] = (T)m; }
          else if (lead) { P[0] = T(0); P[1] = T(0); }
        }
        int pos = lead + epos;
        long long c = dpre;
        for (uint32_t k = k0; k < k1; ++k)
        {
          const bool runend = k + 1 == nreal || K[k + 1].t != K[k].t;
          if (KIND == 0)
          {
            if (runend && !is_infinite(K[k].t))
            {
              P[2 * pos] = K[k].t;
              P[2 * pos + 1] = (T)(m - 1 - k);
              ++pos;
            }
          }
          else
          {
            c += K[k].d;
            if (runend)
            {
              P[2 * pos] = K[k].t;
              P[2 * pos + 1] = (T)c;
              ++pos;
            }
          }
        }
        // the last thread holding keys knows the total
        if (k1 == nreal && k0 < k1) counts[bi] = (uint32_t)pos;
        if (nreal == 0 && threadIdx.x == 0) counts[bi] = (uint32_t)lead;
        __syncthreads();
      }
    }

    // Exclusive scan of n 32-bit counts into n + 1 offsets, in three passes
    // (block sums, one block over the sums, block scans plus their base).
    constexpr int SCAN_BLOCK = 1024;

    __global__ void scan_block_sums_kernel(const uint32_t* __restrict__ in, uint64_t n, uint64_t* __restrict__ sums)
    {
      __shared__ unsigned long long s[32];
      const uint64_t i = (uint64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
      unsigned long long v = i < n ? in[i] : 0;
      v = __reduce_add_sync(0xffffffffu, (unsigned)v);
      if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
      __syncthreads();
      if (threadIdx.x == 0)
      {
        unsigned long long t = 0;
        for (int w = 0; w < SCAN_BLOCK / 32; ++w) t += s[w];
        sums[blockIdx.x] = t;
      }
    }

    __global__ void scan_sums_kernel(uint64_t* sums, uint64_t nb)
    {
      // one thread: the number of blocks is small (n / 1024)
      if (threadIdx.x != 0 || blockIdx.x != 0) return;
      uint64_t run = 0;
      for (uint64_t b = 0; b < nb; ++b)
      {
        const uint64_t v = sums[b];
        sums[b] = run;
        run += v;
      }
    }

    __global__ void scan_finish_kernel(const uint32_t* __restrict__ in, uint64_t n, const uint64_t* __restrict__ sums,
                                       uint64_t* __restrict__ out)
    {
      __shared__ unsigned long long s[SCAN_BLOCK / 32];
      const uint64_t i = (uint64_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      unsigned long long v = i < n ? in[i] : 0, x = v;
      for (int o = 1; o < 32; o <<= 1)
      {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) s[warp] = x;
      __syncthreads();
      if (warp == 0)
      {
        unsigned long long w = s[lane];
        for (int o = 1; o < 32; o <<= 1)
        {
          const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
          if (lane >= o) w += y;
        }
        s[lane] = w;
      }
      __syncthreads();
      const unsigned long long incl = x + (warp ? s[warp - 1] : 0) + sums[blockIdx.x];
      if (i < n) out[i + 1] = incl;
      if (i == 0) out[0] = 0;
    }

    template <typename T, int KIND>
    __global__ void pack_points_kernel(const T* __restrict__ padded, const uint64_t* __restrict__ boff, uint64_t n,
                                       const uint64_t* __restrict__ ooff, T* __restrict__ out, uint64_t cap)
    {
      for (uint64_t bi = blockIdx.x; bi < n; bi += gridDim.x)
      {
        const uint64_t b0 = boff[bi];
        const T* P = padded + 2 * (KIND == 0 ? b0 + bi : 2 * b0 + bi);
        const uint64_t o0 = ooff[bi], cnt = ooff[bi + 1] - o0;
        for (uint64_t k = threadIdx.x; k < 2 * cnt; k += blockDim.x)
          if (2 * o0 + k < 2 * cap) out[2 * o0 + k] = P[k];
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

    struct AsyncMem
    {
      StreamBuffer buf;
      void* p;
      AsyncMem(size_t bytes, cudaStream_t st) : buf(bytes, st), p(buf.get()) { }
    };

    template <typename T, int KIND>
    void barcodes_to_pcfs(const T* bars, const uint64_t* boff, uint64_t n, uint64_t n_bars, T* out,
                          uint64_t out_capacity, uint64_t* out_off, cudaStream_t st)
    {
      const DeviceInfo dev = device_info();
      const uint64_t bound = (KIND == 0 ? n_bars : 2 * n_bars) + n;
      AsyncMem padded(2 * sizeof(T) * bound, st);
      AsyncMem scratch(sizeof(PKey<T>) * 4 * std::max<uint64_t>(n_bars, 1), st);
      AsyncMem counts(sizeof(uint32_t) * n, st);
      const uint64_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
      AsyncMem sums(sizeof(uint64_t) * nb, st);
      const unsigned grid = (unsigned)std::min<uint64_t>(n, (uint64_t)dev.sms * 8);
      barcode_summary_kernel<T, KIND><<<grid, PB_THREADS, 0, st>>>(bars, boff, n, (PKey<T>*)scratch.p, (T*)padded.p,
                                                                   (uint32_t*)counts.p);
      SBG_CUDA(launched());
      scan_block_sums_kernel<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>((const uint32_t*)counts.p, n, (uint64_t*)sums.p);
      SBG_CUDA(launched());
      scan_sums_kernel<<<1, 32, 0, st>>>((uint64_t*)sums.p, nb);
      SBG_CUDA(launched());
      scan_finish_kernel<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>((const uint32_t*)counts.p, n, (const uint64_t*)sums.p,
                                                              out_off);
      SBG_CUDA(launched());
      pack_points_kernel<T, KIND><<<grid, 128, 0, st>>>((const T*)padded.p, boff, n, out_off, out, out_capacity);
      SBG_CUDA(launched());
    }

    void check_summary_args(int kind, int dtype)
    {
      if (kind != SBG_STABLE_RANK && kind != SBG_BETTI_CURVE)
        throw Error(ST_INVALID_ARGUMENT, "kind must be SBG_STABLE_RANK or SBG_BETTI_CURVE");
      if (dtype != SBG_F32 && dtype != SBG_F64) throw Error(ST_INVALID_ARGUMENT, "dtype must be SBG_F32 or SBG_F64");
    }

    void run_summary(int kind, int dtype, const void* bars, const uint64_t* boff, uint64_t n, uint64_t n_bars,
                     void* out, uint64_t cap, uint64_t* out_off, cudaStream_t st)
    {
      if (dtype == SBG_F32)
      {
        if (kind == SBG_STABLE_RANK)
          barcodes_to_pcfs<float, 0>((const float*)bars, boff, n, n_bars, (float*)out, cap, out_off, st);
        else barcodes_to_pcfs<float, 1>((const float*)bars, boff, n, n_bars, (float*)out, cap, out_off, st);
      }
      else
      {
        if (kind == SBG_STABLE_RANK)
          barcodes_to_pcfs<double, 0>((const double*)bars, boff, n, n_bars, (double*)out, cap, out_off, st);
        else barcodes_to_pcfs<double, 1>((const double*)bars, boff, n, n_bars, (double*)out, cap, out_off, st);
      }
    }
  }
}

using namespace sbg;

extern "C"
{
  uint64_t sbg_barcode_pcf_capacity(int kind, uint64_t n_barcodes, uint64_t n_bars)
  {
    return (kind == SBG_BETTI_CURVE ? 2 * n_bars : n_bars) + n_barcodes;
  }

  int sbg_barcodes_to_pcfs_device(int kind, int dtype, const void* bars, const uint64_t* bar_offsets,
                                  uint64_t n_barcodes, uint64_t n_bars, void* out_points, uint64_t out_capacity,
                                  uint64_t* out_offsets, void* stream)
  {
    return abi_call([&] {
      check_summary_args(kind, dtype);
      if (!out_offsets) throw Error(ST_INVALID_ARGUMENT, "null out_offsets");
      cudaStream_t st = (cudaStream_t)stream;
      if (n_barcodes == 0)
      {
        SBG_CUDA(cudaMemsetAsync(out_offsets, 0, sizeof(uint64_t), st));
        return;
      }
      if (!bar_offsets || !out_points || (n_bars && !bars)) throw Error(ST_INVALID_ARGUMENT, "null pointer");
      if (out_capacity < sbg_barcode_pcf_capacity(kind, n_barcodes, n_bars))
        throw Error(ST_INVALID_ARGUMENT, "out_capacity is below sbg_barcode_pcf_capacity");
      run_summary(kind, dtype, bars, bar_offsets, n_barcodes, n_bars, out_points, out_capacity, out_offsets, st);
    });
  }

  int sbg_barcodes_to_pcfs_host(int kind, int dtype, const void* bars, const uint64_t* bar_offsets,
                                uint64_t n_barcodes, void* out_points, uint64_t out_capacity, uint64_t* out_offsets)
  {
    return abi_call([&] {
      check_summary_args(kind, dtype);
      if (!out_offsets) throw Error(ST_INVALID_ARGUMENT, "null out_offsets");
      if (n_barcodes == 0) { out_offsets[0] = 0; return; }
      if (!bar_offsets || !out_points) throw Error(ST_INVALID_ARGUMENT, "null pointer");
      if (bar_offsets[0] != 0) throw Error(ST_INVALID_INPUT, "bar offsets must start at 0");
      for (uint64_t i = 0; i < n_barcodes; ++i)
        if (bar_offsets[i + 1] < bar_offsets[i]) throw Error(ST_INVALID_INPUT, "bar offsets must not decrease");
      const uint64_t n_bars = bar_offsets[n_barcodes];
      if (n_bars && !bars) throw Error(ST_INVALID_ARGUMENT, "null bars");
      const uint64_t need = sbg_barcode_pcf_capacity(kind, n_barcodes, n_bars);
      if (out_capacity < need) throw Error(ST_INVALID_ARGUMENT, "out_capacity is below sbg_barcode_pcf_capacity");
      const size_t es = dtype == SBG_F32 ? 4 : 8;
      cudaStream_t st;
      SBG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{st};
      DeviceBuffer dbars(std::max<uint64_t>(n_bars, 1) * 2 * es), doff((n_barcodes + 1) * sizeof(uint64_t));
      DeviceBuffer dout(need * 2 * es), dooff((n_barcodes + 1) * sizeof(uint64_t));
      if (n_bars) SBG_CUDA(cudaMemcpyAsync(dbars.get(), bars, n_bars * 2 * es, cudaMemcpyHostToDevice, st));
      SBG_CUDA(cudaMemcpyAsync(doff.get(), bar_offsets, (n_barcodes + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice,
                               st));
      run_summary(kind, dtype, dbars.get(), (const uint64_t*)doff.get(), n_barcodes, n_bars, dout.get(), need,
                  (uint64_t*)dooff.get(), st);
      SBG_CUDA(cudaMemcpyAsync(out_offsets, dooff.get(), (n_barcodes + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                               st));
      SBG_CUDA(cudaStreamSynchronize(st));
      const uint64_t total = out_offsets[n_barcodes];
      if (total) SBG_CUDA(cudaMemcpyAsync(out_points, dout.get(), total * 2 * es, cudaMemcpyDeviceToHost, st));
      SBG_CUDA(cudaStreamSynchronize(st));
    });
  }
}
