// Two alternative designs of the float32 pair kernel, kept as selectable
// variants (sbg_set_tuning variant 7 and 8) so that each can be timed and
// profiled against the default (variant 5, pair_kernels.cu) on the same
// inputs.  The planner never picks them: both measured slower on GB300.
//
// Variant 7: one unified 8-byte shared-memory load per lane per step.
//   The default kernel brings a step's new (v, t) element in with three
//   predicated loads (row time, row value: one wavefront each; the column's
//   8-byte element: two), four wavefronts per warp-step whichever side
//   advances.  Here every lane's next element, row or column, lies in the
//   lane's own bank pair, so one 64-bit load serves the whole warp in two
//   wavefronts: the item's columns are staged as two blocks of 16 (lane l's
//   column at bank pair l % 16, 128 bytes between its elements) and each
//   warp's row is replicated 16 times (copy c at bank pair c, also 128 bytes
//   between elements).  The loaded element is routed by tracking the sides
//   as "the side that advanced last" and "the other side" instead of row and
//   column: the integrand is symmetric in the two values, so only the other
//   side's value, time and address need a select.  Rectangles, their order
//   and their grouping into Kahan blocks are those of the default walk, so
//   for finite values the sums are equal bit for bit; a zero-width rectangle
//   is not skipped, so an infinite value next to a shared breakpoint gives
//   NaN here where the default gives inf (finite inputs only).  The
//   replicated row costs 128 bytes per element per warp, which caps the
//   warps per CTA for all but short PCFs.
//
// Variant 8: merge path, one pair per warp (Green, McColl and Bader 2012).
//   The 32 lanes split the S = L_i + L_j - 1 steps of one pair: lane l
//   finds where step l S / 32 falls in the two breakpoint lists by a binary
//   search over the merge-path diagonal (ties go to the row, as in the
//   reference's walk), walks its share, and the partial sums are added by a
//   warp shuffle reduction.  Row and column are staged with one pad word
//   every 32 so lanes about S / 32 steps apart rarely share a bank.
#include "pair_kernels.cuh"
#include "sbg_internal.hpp"

#include <climits>

namespace sbg
{
  namespace
  {
    constexpr unsigned FULLMASK = 0xffffffffu;

    __device__ __forceinline__ void kahan_step(float& acc, float& comp, float x)
    {
      const float y = x - comp;
      const float s = acc + y;
      comp = isfinite(s) ? (s - acc) - y : 0.f;
      acc = s;
    }

    // The item of a persistent CTA: rows [row_lo, row_hi) against the 32
    // columns starting at col0 (same decoding as the default kernel).
    __device__ __forceinline__ void decode_item(const ProblemDesc<float>& P, unsigned long long item,
                                                uint64_t& row_lo, uint64_t& row_hi, uint64_t& col0)
    {
      const uint64_t G = ceil_div_u64(P.nc, 32);
      uint64_t c, g;
      if (P.mode == MODE_CROSS) { c = item / G; g = item % G; }
      else tri_decode(item, P.row_begin, P.row_end, P.q, G, &c, &g);
      row_lo = P.row_begin + c * 32ull * P.q;
      row_hi = row_lo + 32ull * P.q;
      if (row_hi > P.row_end) row_hi = P.row_end;
      col0 = 32ull * g;
      if (P.mode != MODE_CROSS)
      {
        const uint64_t first = col0 + (P.mode == MODE_PDIST ? 1 : 0);
        if (row_lo < first) row_lo = first;
      }
    }

    __device__ __forceinline__ void store_result(const ProblemDesc<float>& P, uint64_t iorig, uint64_t corig, float v)
    {
      const uint64_t idx = P.mode == MODE_CROSS ? iorig * P.ld + corig : condensed_index(P.mode, iorig, corig);
      const uint64_t rel = idx - P.out_base;  // wraps for idx < out_base
      if (rel < P.out_count) P.out[rel] = v;
    }

    __device__ __forceinline__ int padded(int k) { return k + (k >> 5); }
  }

  // ---- variant 7: replicated row, unified loads -------------------------------

  template <int K, int U>
  __global__ void __launch_bounds__(1024, 1) pairs_reprow_kernel(const __grid_constant__ LaunchParams<float> L)
  {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // columns: half h = lane / 16 at [h * lmax_c * 16 + k * 16 + lane % 16]
    float2* cols = reinterpret_cast<float2*>(smem_raw);
    // rows: per warp row_cap elements x 16 copies, copy c of element k at [k * 16 + c]
    float2* rows = cols + (size_t)L.lmax_c * 32;
    __shared__ unsigned long long s_item;
    __shared__ unsigned int s_next_row;
    const ProblemDesc<float>& P = L.one;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int cl = lane & 15;
    float2* rep = rows + (size_t)warp * L.row_cap * 16;
    float2* mycol = cols + (size_t)(lane >> 4) * L.lmax_c * 16 + cl;
    const float INF = __int_as_float(0x7f800000);

    for (;;)
    {
      if (threadIdx.x == 0)
      {
        s_item = atomicAdd(L.queue, 1ull);
        s_next_row = 0;
      }
      __syncthreads();
      const unsigned long long item = s_item;
      if (item >= L.total_items) break;
      uint64_t row_lo, row_hi, col0;
      decode_item(P, item, row_lo, row_hi, col0);
      const uint64_t cj = col0 + lane;
      const bool cvalid = cj < P.nc;
      uint64_t corig = P.cperm ? P.cperm[cvalid ? cj : col0] : (cvalid ? cj : col0);
      const bool pgood = corig < P.nc;
      if (!pgood) corig = 0;
      const uint64_t coff = P.coff[corig];
      const uint32_t clen = (uint32_t)(P.coff[corig + 1] - coff);
      const uint32_t maxlc = __reduce_max_sync(FULLMASK, clen);
      const bool item_ok = !(maxlc > L.lmax_c || __any_sync(FULLMASK, clen == 0));  // CTA-uniform
      if (item_ok)
      {
        // the column's last element ends at +inf, above every row time, so a
        // column never advances past its end whichever side wins a tie
        const float* cp = P.cpts + 2 * coff;
        for (uint32_t k = warp; k < maxlc; k += nwarps)
          if (k < clen)
          {
            const float v = cp[2 * k + 1];
            const float tn = (k + 1 < clen) ? fminf(cp[2 * k + 2], FLT_MAX) : INF;
            mycol[(size_t)k * 16] = make_float2(v, tn);
          }
      }
      __syncthreads();
      if (item_ok)
      {
        for (;;)
        {
          unsigned r = 0;
          if (lane == 0) r = atomicAdd(&s_next_row, 1u);
          r = __shfl_sync(FULLMASK, r, 0);
          const uint64_t i = row_lo + r;
          if (i >= row_hi) break;
          const uint64_t iorig = P.rperm ? P.rperm[i] : i;
          if (iorig >= P.nr) continue;
          const uint64_t roff = P.roff[iorig];
          const uint32_t rlen = (uint32_t)(P.roff[iorig + 1] - roff);
          const bool ok = cvalid && pgood && (P.mode == MODE_CROSS || (P.mode == MODE_PDIST ? cj < i : cj <= i));
          if (!__any_sync(FULLMASK, ok) || rlen == 0 || rlen + U > L.row_cap) continue;
          // the row, 16 copies per element, then U sentinel elements: each lane
          // loads one element and writes its copies rotated by lane, so a
          // half-warp's 16 stores hit 16 bank pairs
          const float* rp = P.rpts + 2 * roff;
          const float vlast = rp[2 * (rlen - 1) + 1];
          for (uint32_t base = 0; base < rlen + U; base += 32)
          {
            const uint32_t k = base + lane;
            float v = vlast, tn = FLT_MAX;
            if (k + 1 < rlen) { v = rp[2 * k + 1]; tn = fminf(rp[2 * k + 2], FLT_MAX); }
            else if (k + 1 == rlen) v = rp[2 * k + 1];
            if (k < rlen + U)
            {
#pragma unroll
              for (int c = 0; c < 16; ++c) rep[(size_t)k * 16 + ((c + lane) & 15)] = make_float2(v, tn);
            }
          }
          __syncwarp();
          const float2 R0 = rep[cl], C0 = mycol[0];
          // "last": the side that advanced last (the row to start with); "other": the other side
          float lv = R0.x, lt = R0.y, ov = C0.x, ot = C0.y;
          uint32_t la = (uint32_t)__cvta_generic_to_shared(rep + cl);
          uint32_t oa = (uint32_t)__cvta_generic_to_shared(mycol);
          // the row's last element (the columns lie below the rows in shared
          // memory, so a min with it leaves a column address alone)
          const uint32_t rep_last = la + (rlen - 1) * 128u;
          float t = 0.f, acc = 0.f, comp = 0.f;
          const float p = P.p;
          const uint32_t steps = rlen + maxlc - 1;
          const uint32_t nblk = (steps + U - 1) / U;
          for (uint32_t b = 0; b < nblk; ++b)
          {
            la = min(la, rep_last);
            oa = min(oa, rep_last);
            float blk = 0.f;
#pragma unroll
            for (int u = 0; u < U; ++u)
            {
              const bool q = lt <= ot;  // the last side advances again (also on a tie)
              const float tn = fminf(lt, ot);
              blk = PairOp<K>::acc(blk, tn - t, lv, ov, p);
              t = tn;
              const uint32_t a = q ? la : oa;
              const float nov = q ? ov : lv;
              const float nott = fmaxf(lt, ot);
              const uint32_t noa = q ? oa : la;
              la = a + 128u;
              asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(lv), "=f"(lt) : "r"(la));
              ov = nov;
              ot = nott;
              oa = noa;
            }
            kahan_step(acc, comp, blk);
          }
          __syncwarp();
          if (ok) store_result(P, iorig, corig, PairOp<K>::fin(acc - comp, p));
        }
      }
      __syncthreads();
    }
  }

  // ---- variant 8: merge path, one pair per warp --------------------------------

  template <int K>
  __global__ void __launch_bounds__(1024, 1) pairs_mergepath_kernel(const __grid_constant__ LaunchParams<float> L)
  {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // columns: times then values, column j at [j * CSP + padded(k)]; rows per warp likewise
    const int CSP = (int)L.lmax_c, RSP = (int)L.row_cap;  // padded strides (host-sized)
    float* ct = reinterpret_cast<float*>(smem_raw);
    float* cv = ct + 32 * CSP;
    __shared__ unsigned long long s_item;
    __shared__ unsigned int s_next_row;
    __shared__ uint32_t s_clen[32];
    __shared__ uint64_t s_corig[32];
    const ProblemDesc<float>& P = L.one;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    float* rt = cv + 32 * CSP + (size_t)warp * 2 * RSP;
    float* rv = rt + RSP;

    for (;;)
    {
      if (threadIdx.x == 0)
      {
        s_item = atomicAdd(L.queue, 1ull);
        s_next_row = 0;
      }
      __syncthreads();
      const unsigned long long item = s_item;
      if (item >= L.total_items) break;
      uint64_t row_lo, row_hi, col0;
      decode_item(P, item, row_lo, row_hi, col0);
      // column j of the item, staged by warp j % nwarps
      for (int j = warp; j < 32; j += nwarps)
      {
        const uint64_t cj = col0 + j;
        uint64_t corig = cj < P.nc ? (P.cperm ? P.cperm[cj] : cj) : P.nc;
        uint32_t clen = 0;
        if (corig < P.nc)
        {
          const uint64_t coff = P.coff[corig];
          clen = (uint32_t)(P.coff[corig + 1] - coff);
          if (clen == 0 || padded((int)clen - 1) >= CSP) clen = 0;  // host sized CSP; never expected
          const float* cp = P.cpts + 2 * coff;
          for (uint32_t k = lane; k < clen; k += 32)
          {
            cv[j * CSP + padded(k)] = cp[2 * k + 1];
            ct[j * CSP + padded(k)] = (k + 1 < clen) ? fminf(cp[2 * k + 2], FLT_MAX) : FLT_MAX;
          }
        }
        if (lane == 0)
        {
          s_clen[j] = clen;
          s_corig[j] = corig;
        }
      }
      __syncthreads();
      for (;;)
      {
        unsigned r = 0;
        if (lane == 0) r = atomicAdd(&s_next_row, 1u);
        r = __shfl_sync(FULLMASK, r, 0);
        const uint64_t i = row_lo + r;
        if (i >= row_hi) break;
        const uint64_t iorig = P.rperm ? P.rperm[i] : i;
        if (iorig >= P.nr) continue;
        const uint64_t roff = P.roff[iorig];
        const int rlen = (int)(P.roff[iorig + 1] - roff);
        if (rlen == 0 || padded(rlen - 1) >= RSP) continue;
        const float* rp = P.rpts + 2 * roff;
        for (int k = lane; k < rlen; k += 32)
        {
          rv[padded(k)] = rp[2 * k + 1];
          rt[padded(k)] = (k + 1 < rlen) ? fminf(rp[2 * k + 2], FLT_MAX) : FLT_MAX;
        }
        __syncwarp();
        const float p = P.p;
        for (int j = 0; j < 32; ++j)
        {
          const uint64_t cj = col0 + j;
          const int clen = (int)s_clen[j];
          const bool ok = clen > 0 && cj < P.nc && (P.mode == MODE_CROSS || (P.mode == MODE_PDIST ? cj < i : cj <= i));
          if (!ok) continue;  // warp-uniform
          const float* gt_ = ct + j * CSP;
          const float* gv_ = cv + j * CSP;
          const int S = rlen + clen - 1;
          const int s0 = (int)(((long long)S * lane) >> 5), s1 = (int)(((long long)S * (lane + 1)) >> 5);
          // the first e = s0 events of the merge of the finite breakpoints
          // A = rt[0 .. rlen - 2] and B = gt[0 .. clen - 2] (ties: A first)
          const int na = rlen - 1, nb = clen - 1;
          const int e = min(s0, na + nb);
          int lo = max(0, e - nb), hi = min(e, na);
          while (lo < hi)
          {
            const int a = (lo + hi + 1) >> 1;  // a >= 1, e - a <= nb
            if (rt[padded(a - 1)] <= gt_[padded(e - a)]) lo = a; else hi = a - 1;
          }
          int a = lo, b = e - lo;
          float t = 0.f;
          if (a > 0) t = rt[padded(a - 1)];
          if (b > 0) t = fmaxf(t, gt_[padded(b - 1)]);
          float fv = rv[padded(a)], ft = rt[padded(a)], gv = gv_[padded(b)], gtt = gt_[padded(b)];
          float sum = 0.f;
          for (int s = s0; s < s1; ++s)
          {
            const float tn = fminf(ft, gtt);
            sum = PairOp<K>::acc(sum, tn - t, fv, gv, p);
            t = tn;
            if (ft <= gtt)
            {
              if (a < na)
              {
                ++a;
                fv = rv[padded(a)];
                ft = rt[padded(a)];
              }
            }
            else
            {
              ++b;  // gtt < ft <= FLT_MAX: the column is not on its last element
              gv = gv_[padded(b)];
              gtt = gt_[padded(b)];
            }
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULLMASK, sum, o);
          if (lane == 0) store_result(P, iorig, s_corig[j], PairOp<K>::fin(sum, p));
        }
        __syncwarp();
      }
      __syncthreads();
    }
  }

  // ---- launchers -----------------------------------------------------------------

  template <typename KernelFn>
  static cudaError_t launch_fn(KernelFn fn, dim3 g, dim3 b, size_t smem, cudaStream_t s, const LaunchParams<float>& L)
  {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<g, b, smem, s>>>(L);
    return launched();
  }

  cudaError_t launch_pair_variant(const LaunchParams<float>& L, int opk, int variant, int warps, int grid,
                                  size_t smem, cudaStream_t s)
  {
    if (L.probs) return cudaErrorInvalidValue;  // single problems only
    constexpr int U = 8;  // the default float kernel's Kahan block
    dim3 g((unsigned)grid), b((unsigned)(warps * 32));
    if (variant == 7)
    {
      switch (opk)
      {
        case OPK_L1: return launch_fn(pairs_reprow_kernel<OPK_L1, U>, g, b, smem, s, L);
        case OPK_L2DIST: return launch_fn(pairs_reprow_kernel<OPK_L2DIST, U>, g, b, smem, s, L);
        case OPK_LP: return launch_fn(pairs_reprow_kernel<OPK_LP, U>, g, b, smem, s, L);
        case OPK_INNER: return launch_fn(pairs_reprow_kernel<OPK_INNER, U>, g, b, smem, s, L);
      }
    }
    else if (variant == 8)
    {
      switch (opk)
      {
        case OPK_L1: return launch_fn(pairs_mergepath_kernel<OPK_L1>, g, b, smem, s, L);
        case OPK_L2DIST: return launch_fn(pairs_mergepath_kernel<OPK_L2DIST>, g, b, smem, s, L);
        case OPK_LP: return launch_fn(pairs_mergepath_kernel<OPK_LP>, g, b, smem, s, L);
        case OPK_INNER: return launch_fn(pairs_mergepath_kernel<OPK_INNER>, g, b, smem, s, L);
      }
    }
    return cudaErrorInvalidValue;
  }

  int padded_words(int k) { return k + (k >> 5); }
}
