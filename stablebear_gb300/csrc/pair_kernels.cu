// Pairwise PCF integration kernels (sm_103a).  Design notes are in
// pair_kernels.cuh; this file holds the device code and its launchers.
#include "pair_kernels.cuh"
#include "sbg_internal.hpp"

#include <climits>

namespace sbg
{
  // Rectangles per naive block sum (blocks are combined with Kahan
  // compensation): 8 for float; 64 for double, whose kernels are bound by the
  // FP64 pipe, so the compensation's four FP64 operations per block cost a
  // share of the time that a longer block cuts (a naive block of 64 doubles
  // errs by at most 63 ulp, far below the 1e-12 target).
  template <typename T> struct Unroll;
#ifndef SBG_F32_UNROLL
#define SBG_F32_UNROLL 8
#endif
  template <> struct Unroll<float> { static constexpr int value = SBG_F32_UNROLL; };
#ifndef SBG_F64_UNROLL
#define SBG_F64_UNROLL 64
#endif
  template <> struct Unroll<double> { static constexpr int value = SBG_F64_UNROLL; };

  namespace
  {
    constexpr unsigned FULL = 0xffffffffu;

    __device__ __forceinline__ uint32_t warp_max_u32(uint32_t x)
    {
      return __reduce_max_sync(FULL, x);
    }
    __device__ __forceinline__ uint32_t warp_min_u32(uint32_t x)
    {
      return __reduce_min_sync(FULL, x);
    }

    // Clamp a breakpoint time into [.., TMAX]; NaN and +inf become TMAX.  This
    // keeps every time the merge compares <= TMAX, so a column can never be
    // advanced past its sentinel, whatever the input holds.
    template <typename T>
    __device__ __forceinline__ T clamp_time(T t) { return fmin(t, tmax_of<T>()); }

    template <typename T>
    __device__ __forceinline__ int find_problem(const ProblemDesc<T>* probs, int n, uint64_t item)
    {
      int lo = 0, hi = n - 1;
      while (lo < hi)
      {
        int mid = (lo + hi + 1) >> 1;
        if (probs[mid].item_begin <= item) lo = mid; else hi = mid - 1;
      }
      return lo;
    }

    // Kahan step adding a block sum; a non-finite running sum (the last
    // rectangle of a pair whose tails are non-zero runs to TMAX) keeps a zero
    // compensation so it cannot turn into NaN.
    template <typename T>
    __device__ __forceinline__ void kahan_add(T& acc, T& comp, T x)
    {
      const T y = x - comp;
      const T s = acc + y;
      comp = isfinite(s) ? (s - acc) - y : T(0);
      acc = s;
    }
  }

  // blk + (tn - t) * op(f, g) for a rectangle of positive width; a
  // zero-width rectangle (the row advancing alone on a tie) adds nothing, as
  // in the reference, whose merge advances both sides on a tie and never
  // forms one (so an infinite value there gives inf, not inf * 0 = NaN).
  // Times never decrease along the merge, so tn == t means width zero; for
  // double the test runs on the bit patterns (integer pipe).
  template <int K>
  __device__ __forceinline__ float accumulate(float blk, float t, float tn, float f, float g, float p)
  {
    return tn == t ? blk : PairOp<K>::acc(blk, tn - t, f, g, p);
  }
  template <int K>
  __device__ __forceinline__ double accumulate(double blk, double t, double tn, double f, double g, double p)
  {
    return __double_as_longlong(tn) == __double_as_longlong(t) ? blk : PairOp<K>::acc(blk, tn - t, f, g, p);
  }

  // The merge of one row (warp-shared, segment layout at pf) against one
  // column per lane (segment layout at pg, stride GS elements between
  // consecutive elements of the same column).  `steps` is warp-uniform.
  // FCLAMP: the row pointer stops at its last element (global-memory variant,
  // no padding); otherwise the row buffer is padded with sentinel copies.
  template <typename T, int K, int U, int GS, bool FCLAMP>
  __device__ __forceinline__ T merge_pair(const Elem<T>* __restrict__ pf, const Elem<T>* __restrict__ pg,
                                          uint32_t steps, uint32_t rlen, T p)
  {
    Elem<T> F = pf[0];
    Elem<T> G = pg[0];
    uint32_t fi = 0;
    T t = T(0), acc = T(0), comp = T(0);
    const uint32_t nblk = (steps + U - 1) / U;
    for (uint32_t b = 0; b < nblk; ++b)
    {
      T blk = T(0);
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
        const bool takeF = row_first(F.tn, G.tn);
        const T tn = takeF ? F.tn : G.tn;
        blk = accumulate<K>(blk, t, tn, F.v, G.v, p);
        t = tn;
        if (FCLAMP)
        {
          fi = min(fi + (takeF ? 1u : 0u), rlen - 1);
          pg += takeF ? 0 : GS;
          F = pf[fi];
        }
        else
        {
          pf += takeF ? 1 : 0;
          pg += takeF ? 0 : GS;
          F = *pf;
        }
        G = *pg;
      }
      kahan_add(acc, comp, blk);
    }
    return PairOp<K>::fin(acc - comp, p);
  }

  // Advance exactly one side of the merge with predicated shared-memory
  // loads: only the side whose next breakpoint comes first (the row on a
  // tie) moves its 32-bit shared address and reloads its element; the other
  // side issues no load.  This halves the shared-memory bytes per step of the
  // plain two-load walk, which is what bounds the kernel (one new 8-byte
  // element per lane per step is the floor).
  __device__ __forceinline__ void advance_shared(float& fv, float& ft, float& gv, float& gt, uint32_t& af,
                                                 uint32_t& ag)
  {
    asm("{\n\t.reg .pred p;\n\t"
        "setp.le.f32 p, %1, %3;\n\t"
        "@p add.u32 %4, %4, 8;\n\t"
        "@!p add.u32 %5, %5, 256;\n\t"
        "@p ld.shared.v2.f32 {%0, %1}, [%4];\n\t"
        "@!p ld.shared.v2.f32 {%2, %3}, [%5];\n\t}"
        : "+f"(fv), "+f"(ft), "+f"(gv), "+f"(gt), "+r"(af), "+r"(ag));
  }

  __device__ __forceinline__ void advance_shared(double& fv, double& ft, double& gv, double& gt, uint32_t& af,
                                                 uint32_t& ag)
  {
    asm("{\n\t.reg .pred p;\n\t.reg .s64 fa, ga;\n\t"
        "mov.b64 fa, %1;\n\t"
        "mov.b64 ga, %3;\n\t"
        "setp.le.s64 p, fa, ga;\n\t"
        "@p add.u32 %4, %4, 16;\n\t"
        "@!p add.u32 %5, %5, 512;\n\t"
        "@p ld.shared.v2.f64 {%0, %1}, [%4];\n\t"
        "@!p ld.shared.v2.f64 {%2, %3}, [%5];\n\t}"
        : "+d"(fv), "+d"(ft), "+d"(gv), "+d"(gt), "+r"(af), "+r"(ag));
  }

  // Rows as two arrays (times, then values, `voff` bytes apart) instead of
  // (v, tn) pairs.  All lanes of a warp read the same row at nearby
  // positions; with 8-byte elements two lanes of a half-warp whose positions
  // differ by a multiple of 16 hit the same bank pair, while with 4-byte
  // words two positions collide only at a distance of 32 or more, so the two
  // row loads are conflict-free in practice.  The column side keeps its
  // 8-byte interleaved elements (lane j owns bank pair j mod 16).
  __device__ __forceinline__ void advance_shared_soa(float& fv, float& ft, float& gv, float& gt, uint32_t& af,
                                                     uint32_t voff, uint32_t& ag)
  {
    asm("{\n\t.reg .pred p;\n\t.reg .b32 va;\n\t"
        "setp.le.f32 p, %1, %3;\n\t"
        "@p add.u32 %4, %4, 4;\n\t"
        "@!p add.u32 %5, %5, 256;\n\t"
        "add.u32 va, %4, %6;\n\t"
        "@p ld.shared.f32 %1, [%4];\n\t"
        "@p ld.shared.f32 %0, [va];\n\t"
        "@!p ld.shared.v2.f32 {%2, %3}, [%5];\n\t}"
        : "+f"(fv), "+f"(ft), "+f"(gv), "+f"(gt), "+r"(af), "+r"(ag)
        : "r"(voff));
  }

  __device__ __forceinline__ void advance_shared_soa(double& fv, double& ft, double& gv, double& gt, uint32_t& af,
                                                     uint32_t voff, uint32_t& ag)
  {
    asm("{\n\t.reg .pred p;\n\t.reg .b32 va;\n\t.reg .s64 fa, ga;\n\t"
        "mov.b64 fa, %1;\n\t"
        "mov.b64 ga, %3;\n\t"
        "setp.le.s64 p, fa, ga;\n\t"
        "@p add.u32 %4, %4, 8;\n\t"
        "@!p add.u32 %5, %5, 512;\n\t"
        "add.u32 va, %4, %6;\n\t"
        "@p ld.shared.f64 %1, [%4];\n\t"
        "@p ld.shared.f64 %0, [va];\n\t"
        "@!p ld.shared.v2.f64 {%2, %3}, [%5];\n\t}"
        : "+d"(fv), "+d"(ft), "+d"(gv), "+d"(gt), "+r"(af), "+r"(ag)
        : "r"(voff));
  }

  // ft0: the warp's row times; the values follow `voff` bytes later.
  // rlen: the row's elements.  Once a lane's pair is done both sides sit on
  // their sentinels and the row advances on every step; at each block start
  // the row address is pulled back to the row's last element (the sentinel
  // itself, equal to every padding copy), so within a block it runs at most
  // U elements past it and the row buffer needs only U padding copies, not
  // one per step the longest column of the warp may still take.
  template <typename T, int K, int U>
  __device__ __forceinline__ T merge_smem_soa(const T* ft0, uint32_t voff, const Elem<T>* pg, uint32_t steps,
                                              uint32_t rlen, T p)
  {
    T fv = *reinterpret_cast<const T*>(reinterpret_cast<const unsigned char*>(ft0) + voff);
    T ft = *ft0;
    Elem<T> G = *pg;
    uint32_t af = (uint32_t)__cvta_generic_to_shared(ft0);
    const uint32_t af_last = af + (rlen - 1) * (uint32_t)sizeof(T);
    uint32_t ag = (uint32_t)__cvta_generic_to_shared(pg);
    T t = T(0), acc = T(0), comp = T(0);
    const uint32_t nblk = (steps + U - 1) / U;
    for (uint32_t b = 0; b < nblk; ++b)
    {
#ifndef SBG_ROW_PAD_FULL
      af = min(af, af_last);
#endif
      T blk = T(0);
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
        const T tn = earlier(ft, G.tn);
        blk = accumulate<K>(blk, t, tn, fv, G.v, p);
        t = tn;
        advance_shared_soa(fv, ft, G.v, G.tn, af, voff, ag);
      }
      kahan_add(acc, comp, blk);
    }
    return PairOp<K>::fin(acc - comp, p);
  }

  // Shared-memory merge with predicated loads.  pf: the warp's row buffer,
  // pg: this lane's column in the interleaved column block (stride 32).
  template <typename T, int K, int U>
  __device__ __forceinline__ T merge_smem_pred(const Elem<T>* pf, const Elem<T>* pg, uint32_t steps, T p)
  {
    Elem<T> F = *pf;
    Elem<T> G = *pg;
    uint32_t af = (uint32_t)__cvta_generic_to_shared(pf);
    uint32_t ag = (uint32_t)__cvta_generic_to_shared(pg);
    T t = T(0), acc = T(0), comp = T(0);
    const uint32_t nblk = (steps + U - 1) / U;
    for (uint32_t b = 0; b < nblk; ++b)
    {
      T blk = T(0);
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
        const T tn = earlier(F.tn, G.tn);
        blk = accumulate<K>(blk, t, tn, F.v, G.v, p);
        t = tn;
        advance_shared(F.v, F.tn, G.v, G.tn, af, ag);
      }
      kahan_add(acc, comp, blk);
    }
    return PairOp<K>::fin(acc - comp, p);
  }

  // Persistent kernel.  SMEM = true stages the item's 32 columns and each
  // warp's row in shared memory; SMEM = false reads the packed segment layout
  // (pack_segments_kernel) from global memory through L1.
  // VAR: 0 global-memory variant, 1 shared memory with a two-load pointer
  // walk, 2 shared memory with predicated one-side loads (the default),
  // 5 as 2 with the row held as separate time and value arrays.
  template <typename T, int K, int U, int VAR>
  __global__ void __launch_bounds__(1024, 1) pairs_kernel(const __grid_constant__ LaunchParams<T> L)
  {
    constexpr bool SMEM = VAR != 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Elem<T>* cols = reinterpret_cast<Elem<T>*>(smem_raw);
    Elem<T>* rows = cols + (size_t)L.lmax_c * 32;
    __shared__ unsigned long long s_item;
    __shared__ unsigned int s_next_row;

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    Elem<T>* rbuf = rows + (size_t)warp * L.row_cap;
    const T TM = tmax_of<T>();

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

      const ProblemDesc<T>* Pp = L.probs ? L.probs + find_problem(L.probs, L.n_probs, item) : &L.one;
      const int mode = Pp->mode;
      const uint64_t nc = Pp->nc;
      const uint64_t G = ceil_div_u64(nc, 32);
      const uint64_t local = item - Pp->item_begin;
      uint64_t c, g;
      if (mode == MODE_CROSS) { c = local / G; g = local % G; }
      else tri_decode(local, Pp->row_begin, Pp->row_end, Pp->q, G, &c, &g);
      uint64_t row_lo = Pp->row_begin + c * 32ull * Pp->q;
      uint64_t row_hi = row_lo + 32ull * Pp->q;
      if (row_hi > Pp->row_end) row_hi = Pp->row_end;
      const uint64_t col0 = 32ull * g;
      if (mode != MODE_CROSS)
      {
        const uint64_t first = col0 + (mode == MODE_PDIST ? 1 : 0);
        if (row_lo < first) row_lo = first;
      }

      // This lane's column.  Lanes past the last column mirror lane 0's
      // column (their results are discarded) so the warp-uniform step count
      // and the row padding stay valid for them.
      const uint64_t cj = col0 + lane;
      const bool cvalid = cj < nc;
      const uint64_t cj_eff = cvalid ? cj : col0;
      uint64_t corig = Pp->cperm ? Pp->cperm[cj_eff] : cj_eff;
      const bool pgood = corig < nc;  // a permutation entry out of range reads column 0, result dropped
      if (!pgood) corig = 0;
      const uint64_t coff = Pp->coff[corig];
      const uint32_t clen = (uint32_t)(Pp->coff[corig + 1] - coff);
      const uint32_t maxlc = warp_max_u32(clen);
      const T p = Pp->p;

      bool item_ok = true;
      if (!SMEM && __any_sync(FULL, coff + clen > Pp->ccap)) item_ok = false;  // offsets past the packed columns
      if (SMEM)
      {
        if (maxlc > L.lmax_c || __any_sync(FULL, clen == 0)) item_ok = false;  // host sized lmax_c; never expected
        else
        {
          const T* cp = Pp->cpts + 2 * coff;
          for (uint32_t k = warp; k < maxlc; k += nwarps)
          {
            if (k < clen)
            {
              const T tk = cp[2 * k], vk = cp[2 * k + 1];
              cols[(size_t)k * 32 + lane].v = vk;
              if (k > 0) cols[(size_t)(k - 1) * 32 + lane].tn = clamp_time(tk);
              if (k + 1 == clen) cols[(size_t)k * 32 + lane].tn = TM;
            }
          }
        }
        __syncthreads();
      }

      if (item_ok)
      {
        for (;;)
        {
          unsigned r = 0;
          if (lane == 0) r = atomicAdd(&s_next_row, 1u);
          r = __shfl_sync(FULL, r, 0);
          const uint64_t i = row_lo + r;
          if (i >= row_hi) break;

          const uint64_t iorig = Pp->rperm ? Pp->rperm[i] : i;
          if (iorig >= Pp->nr) continue;  // a permutation entry out of range: skip the row
          const uint64_t roff = Pp->roff[iorig];
          const uint32_t rlen = (uint32_t)(Pp->roff[iorig + 1] - roff);
          const bool ok = cvalid && pgood && (mode == MODE_CROSS || (mode == MODE_PDIST ? cj < i : cj <= i));
          if (!__any_sync(FULL, ok) || rlen == 0) continue;
          if (!SMEM && roff + rlen > Pp->rcap) continue;  // offsets past the packed rows
          const uint32_t steps = rlen + maxlc - 1;

          T res;
          if (SMEM)
          {
            // Row in segment layout plus sentinel padding: at most
            // steps + U - 1 advances can reach the row side, or, with the
            // row address pulled back at every block start (VAR 5), U past
            // the last element.
#ifndef SBG_ROW_PAD_FULL
            const uint32_t pad_end = VAR == 5 ? rlen + U : rlen + maxlc + U;
#else
            const uint32_t pad_end = rlen + maxlc + U;
#endif
            if (pad_end > L.row_cap) continue;  // host sized row_cap; never expected
            const T* rp = Pp->rpts + 2 * roff;
            const T vlast = rp[2 * (rlen - 1) + 1];
            if (VAR == 5)
            {
              // times in [0, row_cap), values in [row_cap, 2 row_cap) of
              // the warp's buffer (the same bytes as row_cap elements)
              T* rt = reinterpret_cast<T*>(rbuf);
              T* rv = rt + L.row_cap;
              for (uint32_t k = lane; k < rlen; k += 32)
              {
                const T tk = rp[2 * k], vk = rp[2 * k + 1];
                rv[k] = vk;
                if (k > 0) rt[k - 1] = clamp_time(tk);
              }
              for (uint32_t k = rlen - 1 + lane; k < pad_end; k += 32)
              {
                rv[k] = vlast;
                rt[k] = TM;
              }
            }
            else
            {
              for (uint32_t k = lane; k < rlen; k += 32)
              {
                const T tk = rp[2 * k], vk = rp[2 * k + 1];
                rbuf[k].v = vk;
                if (k > 0) rbuf[k - 1].tn = clamp_time(tk);
              }
              for (uint32_t k = rlen - 1 + lane; k < pad_end; k += 32)
              {
                rbuf[k].v = vlast;
                rbuf[k].tn = TM;
              }
            }
            __syncwarp();
            if (VAR == 1) res = merge_pair<T, K, U, 32, false>(rbuf, cols + lane, steps, rlen, p);
            else if (VAR == 5)
              res = merge_smem_soa<T, K, U>(reinterpret_cast<const T*>(rbuf), L.row_cap * (uint32_t)sizeof(T),
                                            cols + lane, steps, rlen, p);
            else res = merge_smem_pred<T, K, U>(rbuf, cols + lane, steps, p);
            __syncwarp();
          }
          else
          {
            const Elem<T>* pk = reinterpret_cast<const Elem<T>*>(Pp->rpts);  // packed rows
            const Elem<T>* ck = reinterpret_cast<const Elem<T>*>(Pp->cpts);  // packed columns
            res = merge_pair<T, K, U, 1, true>(pk + roff, ck + coff, steps, rlen, p);
          }

          if (ok)
          {
            const uint64_t jorig = corig;
            uint64_t idx;
            if (mode == MODE_CROSS) idx = iorig * Pp->ld + jorig;
            else idx = condensed_index(mode, iorig, jorig);
            const uint64_t rel = idx - Pp->out_base;  // wraps for idx < out_base
            if (rel < Pp->out_count) Pp->out[rel] = res;
          }
        }
      }
      __syncthreads();
    }
  }

  // ---- time-windowed variant: long PCFs in shared memory, window by window ----
  //
  // For PCFs too long for a 32-column block plus per-warp row buffers.  A
  // work item walks consecutive time windows [A, B).  B is the earliest,
  // over the item's 32 columns, end time of a column's lmax_c-th element
  // counted from its first element ending after A, so no column slice holds
  // more than lmax_c elements.  A row holding more than win_r elements in
  // [A, B) is walked in pieces of at most win_r elements, each a sub-window
  // [Ap, Bp) (Bp the end of the piece's last element) in which every lane
  // starts its column at the first element ending after Ap.  Window ends
  // thus depend on the column group alone, and a pair's rounding on neither
  // the rows per item nor the warps per CTA.  Slices are staged like whole
  // PCFs in the shared-memory variant, with the last element's end set to
  // TMAX, and every rectangle is clipped to end at the (sub-)window end: the
  // warp-uniform steps past a lane's end add zero-width rectangles only, and
  // no side ever steps past its slice.  Integrals over [0, inf) split into
  // the window integrals exactly (the rectangles meeting a window are those
  // of the whole merge, cut at its ends).  Sums carry from piece to piece in
  // registers and from window to window through the output element (raw
  // sums, the finalizer after the last window), which the same CTA reads
  // back after a block barrier.

  __device__ __forceinline__ float earlier3(float a, float b, float c)
  {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
  }
  __device__ __forceinline__ double earlier3(double a, double b, double c) { return earlier(earlier(a, b), c); }

  // Times >= 0 (and TMAX) order as their bit patterns read as unsigned
  // integers, which shared-memory atomicMin handles for both widths.
  template <typename T> struct TimeBits;
  template <> struct TimeBits<float>
  {
    using U = unsigned int;
    __device__ static __forceinline__ U of(float x) { return __float_as_uint(x); }
    __device__ static __forceinline__ float val(U u) { return __uint_as_float(u); }
    __device__ static __forceinline__ U warp_min(U x) { return __reduce_min_sync(0xffffffffu, x); }
  };
  template <> struct TimeBits<double>
  {
    using U = unsigned long long;
    __device__ static __forceinline__ U of(double x) { return (U)__double_as_longlong(x); }
    __device__ static __forceinline__ double val(U u) { return __longlong_as_double((long long)u); }
    __device__ static __forceinline__ U warp_min(U x)
    {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        const U y = __shfl_xor_sync(0xffffffffu, x, o);
        x = y < x ? y : x;
      }
      return x;
    }
  };

  // Moves k0 past the elements of a PCF (CSR points pts, len elements) that
  // end at or before A; the last element ends at TMAX > A.  Returns whether
  // k0 moved.
  template <typename T>
  __device__ __forceinline__ bool slice_start(const T* pts, uint32_t len, uint32_t& k0, T A)
  {
    bool moved = false;
    while (k0 + 1 < len && clamp_time(pts[2 * ((uint64_t)k0 + 1)]) <= A)
    {
      ++k0;
      moved = true;
    }
    return moved;
  }

  // merge_smem_soa over one window: starts at t0 with the running sum acc0,
  // clips every rectangle to end at tend, returns the raw compensated sum.
  template <typename T, int K, int U>
  __device__ __forceinline__ T merge_window(const T* ft0, uint32_t voff, const Elem<T>* pg, uint32_t steps, T t0,
                                            T tend, T acc0, T p)
  {
    T fv = *reinterpret_cast<const T*>(reinterpret_cast<const unsigned char*>(ft0) + voff);
    T ft = *ft0;
    Elem<T> G = *pg;
    uint32_t af = (uint32_t)__cvta_generic_to_shared(ft0);
    uint32_t ag = (uint32_t)__cvta_generic_to_shared(pg);
    T t = t0, acc = acc0, comp = T(0);
    const uint32_t nblk = (steps + U - 1) / U;
    for (uint32_t b = 0; b < nblk; ++b)
    {
      T blk = T(0);
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
        const T tn = earlier3(ft, G.tn, tend);
        blk = accumulate<K>(blk, t, tn, fv, G.v, p);
        t = tn;
        advance_shared_soa(fv, ft, G.v, G.tn, af, voff, ag);
      }
      kahan_add(acc, comp, blk);
    }
    return acc - comp;
  }

  // First k in [lo, hi] whose element of this lane's staged column ends
  // after x (STRICT) or at or after x; element hi (a slice's last, ending at
  // TMAX, or one already known to qualify) always does.
  template <typename T, bool STRICT>
  __device__ __forceinline__ uint32_t column_search(const Elem<T>* cols, int lane, uint32_t lo, uint32_t hi, T x)
  {
    while (lo < hi)
    {
      const uint32_t mid = (lo + hi) >> 1;
      const T tn = cols[(size_t)mid * 32 + lane].tn;
      if (STRICT ? tn > x : tn >= x) hi = mid; else lo = mid + 1;
    }
    return lo;
  }

  // Shared memory: the column block (lmax_c x 32 elements, interleaved), one
  // row buffer per warp (row_cap elements' bytes: times, then values), and the
  // saved slice start of each row of the item (row_slots words).
  template <typename T, int K, int U>
  __global__ void __launch_bounds__(1024, 1) pairs_window_kernel(const __grid_constant__ LaunchParams<T> L)
  {
    using TB = TimeBits<T>;
    using UB = typename TB::U;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const uint32_t CW = L.lmax_c, RW = L.win_r;
    Elem<T>* cols = reinterpret_cast<Elem<T>*>(smem_raw);
    Elem<T>* rows = cols + (size_t)CW * 32;
    uint32_t* rk0 = reinterpret_cast<uint32_t*>(rows + (size_t)nwarps * L.row_cap);
    T* rt = reinterpret_cast<T*>(rows + (size_t)warp * L.row_cap);
    T* rv = rt + L.row_cap;
    const uint32_t voff = L.row_cap * (uint32_t)sizeof(T);
    __shared__ unsigned long long s_item;
    __shared__ unsigned int s_next_row;
    __shared__ UB s_bend;
    __shared__ uint32_t s_ck0[32], s_cnt[32], s_cm[32];
    const T TM = tmax_of<T>();
    const UB TMB = TB::of(TM);

    for (;;)
    {
      if (threadIdx.x == 0) s_item = atomicAdd(L.queue, 1ull);
      __syncthreads();
      const unsigned long long item = s_item;
      if (item >= L.total_items) break;

      const ProblemDesc<T>* Pp = L.probs ? L.probs + find_problem(L.probs, L.n_probs, item) : &L.one;
      const int mode = Pp->mode;
      const uint64_t nc = Pp->nc;
      const uint64_t G = ceil_div_u64(nc, 32);
      const uint64_t local = item - Pp->item_begin;
      uint64_t c, g;
      if (mode == MODE_CROSS) { c = local / G; g = local % G; }
      else tri_decode(local, Pp->row_begin, Pp->row_end, Pp->q, G, &c, &g);
      uint64_t row_lo = Pp->row_begin + c * 32ull * Pp->q;
      uint64_t row_hi = row_lo + 32ull * Pp->q;
      if (row_hi > Pp->row_end) row_hi = Pp->row_end;
      const uint64_t col0 = 32ull * g;
      if (mode != MODE_CROSS)
      {
        const uint64_t first = col0 + (mode == MODE_PDIST ? 1 : 0);
        if (row_lo < first) row_lo = first;
      }
      const uint32_t nrows = row_hi > row_lo ? (uint32_t)(row_hi - row_lo) : 0u;

      // This lane's column (lanes past the last column mirror lane 0's).
      const uint64_t cj = col0 + lane;
      const bool cvalid = cj < nc;
      const uint64_t cj_eff = cvalid ? cj : col0;
      uint64_t corig = Pp->cperm ? Pp->cperm[cj_eff] : cj_eff;
      const bool pgood = corig < nc;
      if (!pgood) corig = 0;
      const uint64_t coff = Pp->coff[corig];
      const uint32_t clen = (uint32_t)(Pp->coff[corig + 1] - coff);
      const T p = Pp->p;
      const T* cp = Pp->cpts + 2 * coff;

      // CTA-uniform: every warp holds the same 32 columns.
      if (!__any_sync(FULL, clen == 0) && nrows > 0 && nrows <= L.row_slots)
      {
        for (uint32_t r = threadIdx.x; r < nrows; r += blockDim.x) rk0[r] = 0;
        if (threadIdx.x < 32) s_ck0[threadIdx.x] = 0;
        T A = T(0);
        bool first = true;
        for (;;)
        {
          if (threadIdx.x < 32) s_cnt[threadIdx.x] = 0;
          if (threadIdx.x == 0) s_next_row = 0;

          // Window end: the earliest, over the 32 columns, end of the CW-th
          // element counted from the column's first element ending after A
          // (the start moves past elements ending at A, zero-width ones).
          if (warp == 0)
          {
            uint32_t k0 = s_ck0[lane];
            if (slice_start(cp, clen, k0, A)) s_ck0[lane] = k0;
            const uint32_t k = k0 + CW - 1;
            UB bmin = TMB;
            if (k + 1 < clen) bmin = TB::of(clamp_time(cp[2 * ((uint64_t)k + 1)]));
            bmin = TB::warp_min(bmin);
            if (lane == 0) s_bend = bmin;
          }
          __syncthreads();
          T B = TB::val(s_bend);
          if (!(B > A)) B = TM;  // times out of order: one last window ends the walk
          const bool last = TB::of(B) == TMB;

          // Column slices: up to CW elements from each column's start; the
          // slice ends at the first element ending at or after B.
          {
            const uint32_t k0c = s_ck0[lane];
            const uint32_t availc = min(CW, clen - k0c);
            uint32_t cnt = 0;
            for (uint32_t k = warp; k < availc; k += nwarps)
            {
              const uint32_t kk = k0c + k;
              Elem<T> el;
              el.v = cp[2 * (uint64_t)kk + 1];
              el.tn = (kk + 1 < clen) ? clamp_time(cp[2 * ((uint64_t)kk + 1)]) : TM;
              cols[(size_t)k * 32 + lane] = el;
              cnt += el.tn < B ? 1u : 0u;
            }
            if (cnt) atomicAdd(&s_cnt[lane], cnt);
          }
          __syncthreads();
          if (warp == 0)
          {
            const uint32_t k0c = s_ck0[lane];
            const uint32_t availc = min(CW, clen - k0c);
            const uint32_t m = min(s_cnt[lane] + 1u, availc);
            Elem<T>& el = cols[(size_t)(m - 1) * 32 + lane];
            uint32_t nxt = k0c + m - (el.tn > B ? 1u : 0u);  // first element ending after B
            if (nxt > clen - 1) nxt = clen - 1;
            el.tn = TM;
            s_cm[lane] = m;
            s_ck0[lane] = nxt;
          }
          __syncthreads();
          const uint32_t maxmc = warp_max_u32(s_cm[lane]);

          for (;;)
          {
            unsigned r = 0;
            if (lane == 0) r = atomicAdd(&s_next_row, 1u);
            r = __shfl_sync(FULL, r, 0);
            if (r >= nrows) break;
            const uint64_t i = row_lo + r;
            const uint64_t iorig = Pp->rperm ? Pp->rperm[i] : i;
            if (iorig >= Pp->nr) continue;  // skipped alike by the window-end pass
            const uint64_t roff = Pp->roff[iorig];
            const uint32_t rlen = (uint32_t)(Pp->roff[iorig + 1] - roff);
            if (rlen == 0) continue;

            const bool ok = cvalid && pgood && (mode == MODE_CROSS || (mode == MODE_PDIST ? cj < i : cj <= i));
            if (!__any_sync(FULL, ok)) continue;  // alike in every window
            uint64_t idx;
            if (mode == MODE_CROSS) idx = iorig * Pp->ld + corig;
            else idx = condensed_index(mode, iorig, corig);
            const uint64_t rel = idx - Pp->out_base;  // wraps for idx < out_base
            const bool store = ok && rel < Pp->out_count;
            T acc = (!first && store) ? Pp->out[rel] : T(0);

            // The row's elements meeting [A, B), at most RW at a time: a row
            // denser than the item's columns takes several pieces, each a
            // sub-window [Ap, Bp) for which every lane starts its column at
            // the first element ending after Ap.  A piece is staged like the
            // column slices, plus sentinel padding for the warp-uniform steps.
            uint32_t k0 = rk0[r], z, m;
            T Ap = A;
            bool first_piece = true;
            for (;;)
            {
              uint32_t avail, c2;
              for (;;)
              {
                avail = min(RW, rlen - k0);
                const T* rp = Pp->rpts + 2 * (roff + k0);
                uint32_t zl = 0, cl = 0;
                for (uint32_t k = lane; k < avail; k += 32)
                {
                  const T e = (k0 + k + 1 < rlen) ? clamp_time(rp[2 * ((uint64_t)k + 1)]) : TM;
                  rv[k] = rp[2 * (uint64_t)k + 1];
                  rt[k] = e;
                  zl += e <= Ap ? 1u : 0u;
                  cl += e < B ? 1u : 0u;
                }
                z = __reduce_add_sync(FULL, zl);   // elements ending by Ap (skipped)
                c2 = __reduce_add_sync(FULL, cl);  // elements ending before B
                if (z < avail) break;
                k0 += avail;  // all of them end by Ap; the last element ends at TMAX
                __syncwarp();
              }
              const bool full = c2 + 1 <= avail;  // the piece reaches B
              m = full ? (c2 + 1 > z ? c2 + 1 - z : 1u) : avail - z;
              __syncwarp();
              const T Bp = full ? B : rt[avail - 1];
              const T vlast = rv[z + m - 1];
              __syncwarp();
              const uint32_t pad_end = z + m + maxmc + U;  // <= RW + CW + U < row_cap
              for (uint32_t k = z + m - 1 + lane; k < pad_end; k += 32)
              {
                rv[k] = vlast;
                rt[k] = TM;
              }
              __syncwarp();
              // This lane's column elements meeting [Ap, Bp): from the first
              // ending after Ap to the first ending at or after Bp; the warp
              // steps through the most of them (the whole slices for a piece
              // that is the row's whole window).
              uint32_t g0 = 0, g1 = s_cm[lane] - 1;
              if (!first_piece) g0 = column_search<T, true>(cols, lane, 0, g1, Ap);
              if (!full) g1 = column_search<T, false>(cols, lane, g0, g1, Bp);
              const uint32_t ncol = (first_piece && full) ? maxmc : warp_max_u32(g1 - g0 + 1);
              acc = merge_window<T, K, U>(rt + z, voff, cols + (size_t)g0 * 32 + lane, m + ncol - 1, Ap, Bp, acc, p);
              __syncwarp();
              if (full) break;
              k0 += z + m;
              Ap = Bp;
              first_piece = false;
            }
            // the element reaching B starts the next window (skipped there if
            // it ends at B)
            if (lane == 0) rk0[r] = k0 + z + m - 1;
            if (store) Pp->out[rel] = last ? PairOp<K>::fin(acc, p) : acc;
          }
          __syncthreads();
          if (last) break;
          A = B;
          first = false;
        }
      }
      __syncthreads();
    }
  }

  // ---- hybrid variant: columns in shared memory, rows through L1 -------------
  //
  // Rows are read from the packed segment layout in global memory (all lanes
  // of a warp read the same row at nearby positions, so the reads hit L1);
  // the row index stops at the row's last element.  No per-warp row buffers:
  // all shared memory holds columns, so longer PCFs fit and more warps run.
  // A column group longer than the shared-memory block falls back to reading
  // its columns from global memory too.

  __device__ __forceinline__ void advance_hybrid(float& fv, float& ft, float& gv, float& gt, const Elem<float>* row,
                                                 uint32_t& fi, uint32_t flast, uint32_t& ag)
  {
    asm("{\n\t.reg .pred p;\n\t.reg .u64 a;\n\t"
        "setp.le.f32 p, %1, %3;\n\t"
        "@p add.u32 %4, %4, 1;\n\t"
        "min.u32 %4, %4, %7;\n\t"
        "@!p add.u32 %5, %5, 256;\n\t"
        "mad.wide.u32 a, %4, 8, %6;\n\t"
        "@p ld.global.nc.v2.f32 {%0, %1}, [a];\n\t"
        "@!p ld.shared.v2.f32 {%2, %3}, [%5];\n\t}"
        : "+f"(fv), "+f"(ft), "+f"(gv), "+f"(gt), "+r"(fi), "+r"(ag)
        : "l"(row), "r"(flast));
  }

  __device__ __forceinline__ void advance_hybrid(double& fv, double& ft, double& gv, double& gt,
                                                 const Elem<double>* row, uint32_t& fi, uint32_t flast, uint32_t& ag)
  {
    asm("{\n\t.reg .pred p;\n\t.reg .u64 a;\n\t.reg .s64 fa, ga;\n\t"
        "mov.b64 fa, %1;\n\t"
        "mov.b64 ga, %3;\n\t"
        "setp.le.s64 p, fa, ga;\n\t"
        "@p add.u32 %4, %4, 1;\n\t"
        "min.u32 %4, %4, %7;\n\t"
        "@!p add.u32 %5, %5, 512;\n\t"
        "mad.wide.u32 a, %4, 16, %6;\n\t"
        "@p ld.global.nc.v2.f64 {%0, %1}, [a];\n\t"
        "@!p ld.shared.v2.f64 {%2, %3}, [%5];\n\t}"
        : "+d"(fv), "+d"(ft), "+d"(gv), "+d"(gt), "+r"(fi), "+r"(ag)
        : "l"(row), "r"(flast));
  }

  template <typename T, int K, int U>
  __device__ __forceinline__ T merge_hybrid(const Elem<T>* row, uint32_t rlen, const Elem<T>* pg, uint32_t steps, T p)
  {
    Elem<T> F = row[0];
    Elem<T> G = *pg;
    uint32_t fi = 0;
    const uint32_t flast = rlen - 1;
    uint32_t ag = (uint32_t)__cvta_generic_to_shared(pg);
    T t = T(0), acc = T(0), comp = T(0);
    const uint32_t nblk = (steps + U - 1) / U;
    for (uint32_t b = 0; b < nblk; ++b)
    {
      T blk = T(0);
#pragma unroll
      for (int u = 0; u < U; ++u)
      {
        const T tn = earlier(F.tn, G.tn);
        blk = accumulate<K>(blk, t, tn, F.v, G.v, p);
        t = tn;
        advance_hybrid(F.v, F.tn, G.v, G.tn, row, fi, flast, ag);
      }
      kahan_add(acc, comp, blk);
    }
    return PairOp<K>::fin(acc - comp, p);
  }

  // Rows and columns come from the packed segment layout (rpts / cpts of the
  // descriptors point at Elem<T> arrays at the CSR offsets).
  template <typename T, int K, int U>
  __global__ void __launch_bounds__(1024, 1) pairs_hybrid_kernel(const __grid_constant__ LaunchParams<T> L)
  {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Elem<T>* cols = reinterpret_cast<Elem<T>*>(smem_raw);
    __shared__ unsigned long long s_item;
    __shared__ unsigned int s_next_row;

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;

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

      const ProblemDesc<T>* Pp = L.probs ? L.probs + find_problem(L.probs, L.n_probs, item) : &L.one;
      const int mode = Pp->mode;
      const uint64_t nc = Pp->nc;
      const uint64_t G = ceil_div_u64(nc, 32);
      const uint64_t local = item - Pp->item_begin;
      uint64_t c, g;
      if (mode == MODE_CROSS) { c = local / G; g = local % G; }
      else tri_decode(local, Pp->row_begin, Pp->row_end, Pp->q, G, &c, &g);
      uint64_t row_lo = Pp->row_begin + c * 32ull * Pp->q;
      uint64_t row_hi = row_lo + 32ull * Pp->q;
      if (row_hi > Pp->row_end) row_hi = Pp->row_end;
      const uint64_t col0 = 32ull * g;
      if (mode != MODE_CROSS)
      {
        const uint64_t first = col0 + (mode == MODE_PDIST ? 1 : 0);
        if (row_lo < first) row_lo = first;
      }

      const uint64_t cj = col0 + lane;
      const bool cvalid = cj < nc;
      const uint64_t cj_eff = cvalid ? cj : col0;
      uint64_t corig = Pp->cperm ? Pp->cperm[cj_eff] : cj_eff;
      const bool pgood = corig < nc;  // a permutation entry out of range reads column 0, result dropped
      if (!pgood) corig = 0;
      const uint64_t coff = Pp->coff[corig];
      const uint32_t clen = (uint32_t)(Pp->coff[corig + 1] - coff);
      const uint32_t maxlc = warp_max_u32(clen);
      const T p = Pp->p;
      const Elem<T>* ck = reinterpret_cast<const Elem<T>*>(Pp->cpts);
      const Elem<T>* rk = reinterpret_cast<const Elem<T>*>(Pp->rpts);

      const bool item_ok = !__any_sync(FULL, clen == 0 || coff + clen > Pp->ccap);
      const bool staged = item_ok && maxlc <= L.lmax_c;  // CTA-uniform
      if (staged)
      {
        for (uint32_t k = warp; k < maxlc; k += nwarps)
          if (k < clen) cols[(size_t)k * 32 + lane] = ck[coff + k];
        __syncthreads();
      }

      if (item_ok)
      {
        for (;;)
        {
          unsigned r = 0;
          if (lane == 0) r = atomicAdd(&s_next_row, 1u);
          r = __shfl_sync(FULL, r, 0);
          const uint64_t i = row_lo + r;
          if (i >= row_hi) break;
          const uint64_t iorig = Pp->rperm ? Pp->rperm[i] : i;
          if (iorig >= Pp->nr) continue;  // a permutation entry out of range: skip the row
          const uint64_t roff = Pp->roff[iorig];
          const uint32_t rlen = (uint32_t)(Pp->roff[iorig + 1] - roff);
          const bool ok = cvalid && pgood && (mode == MODE_CROSS || (mode == MODE_PDIST ? cj < i : cj <= i));
          if (!__any_sync(FULL, ok) || rlen == 0 || roff + rlen > Pp->rcap) continue;
          const uint32_t steps = rlen + maxlc - 1;
          T res;
          if (staged) res = merge_hybrid<T, K, U>(rk + roff, rlen, cols + lane, steps, p);
          else res = merge_pair<T, K, U, 1, true>(rk + roff, ck + coff, steps, rlen, p);
          if (ok)
          {
            uint64_t idx;
            if (mode == MODE_CROSS) idx = iorig * Pp->ld + corig;
            else idx = condensed_index(mode, iorig, corig);
            const uint64_t rel = idx - Pp->out_base;
            if (rel < Pp->out_count) Pp->out[rel] = res;
          }
        }
      }
      __syncthreads();
    }
  }

  // Segment layout in global memory: element k of PCF i (at the PCF's own
  // CSR offset) holds (v_k, t_{k+1}), the last one (v_{L-1}, TMAX).
  template <typename T>
  __global__ void pack_segments_kernel(const T* __restrict__ pts, const uint64_t* __restrict__ off, uint64_t n,
                                       Elem<T>* __restrict__ out, uint64_t cap)
  {
    const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (gridDim.x * (uint64_t)blockDim.x) >> 5;
    for (uint64_t i = w; i < n; i += nw)
    {
      const uint64_t o = off[i];
      const uint64_t len = off[i + 1] - o;
      if (o + len > cap || len > cap) continue;  // never write past the packed buffer
      for (uint64_t k = lane; k < len; k += 32)
      {
        Elem<T> e;
        e.v = pts[2 * (o + k) + 1];
        e.tn = (k + 1 < len) ? clamp_time(pts[2 * (o + k + 1)]) : tmax_of<T>();
        out[o + k] = e;
      }
    }
  }

  // ---- launchers ------------------------------------------------------------

  template <typename T, int VAR>
  static cudaError_t launch_op(int opk, dim3 grid, dim3 block, size_t smem, cudaStream_t s, const LaunchParams<T>& L)
  {
    constexpr int U = Unroll<T>::value;
    void (*fn)(const LaunchParams<T>) = nullptr;
    switch (opk)
    {
      case OPK_L1: fn = pairs_kernel<T, OPK_L1, U, VAR>; break;
      case OPK_L2DIST: fn = pairs_kernel<T, OPK_L2DIST, U, VAR>; break;
      case OPK_LP: fn = pairs_kernel<T, OPK_LP, U, VAR>; break;
      case OPK_INNER: fn = pairs_kernel<T, OPK_INNER, U, VAR>; break;
      default: return cudaErrorInvalidValue;
    }
    if (VAR != 0)
    {
      cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    fn<<<grid, block, smem, s>>>(L);
    return launched();
  }

  template <typename T>
  static cudaError_t launch_hybrid(int opk, dim3 grid, dim3 block, size_t smem, cudaStream_t s, const LaunchParams<T>& L)
  {
    constexpr int U = Unroll<T>::value;
    void (*fn)(const LaunchParams<T>) = nullptr;
    switch (opk)
    {
      case OPK_L1: fn = pairs_hybrid_kernel<T, OPK_L1, U>; break;
      case OPK_L2DIST: fn = pairs_hybrid_kernel<T, OPK_L2DIST, U>; break;
      case OPK_LP: fn = pairs_hybrid_kernel<T, OPK_LP, U>; break;
      case OPK_INNER: fn = pairs_hybrid_kernel<T, OPK_INNER, U>; break;
      default: return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, block, smem, s>>>(L);
    return launched();
  }

  template <typename T>
  static cudaError_t launch_window(int opk, dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                   const LaunchParams<T>& L)
  {
    constexpr int U = Unroll<T>::value;
    void (*fn)(const LaunchParams<T>) = nullptr;
    switch (opk)
    {
      case OPK_L1: fn = pairs_window_kernel<T, OPK_L1, U>; break;
      case OPK_L2DIST: fn = pairs_window_kernel<T, OPK_L2DIST, U>; break;
      case OPK_LP: fn = pairs_window_kernel<T, OPK_LP, U>; break;
      case OPK_INNER: fn = pairs_window_kernel<T, OPK_INNER, U>; break;
      default: return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, block, smem, s>>>(L);
    return launched();
  }

  template <typename T>
  cudaError_t launch_pairs(const LaunchParams<T>& L, int opk, int variant, int warps, int grid,
                           size_t smem_bytes, cudaStream_t s)
  {
    dim3 g((unsigned)grid), b((unsigned)(warps * 32));
    if (variant == 7 || variant == 8)
    {
      if constexpr (sizeof(T) == 4) return launch_pair_variant(L, opk, variant, warps, grid, smem_bytes, s);
      else return cudaErrorInvalidValue;  // float32 only (the planner rejects double first)
    }
    if (variant == 6) return launch_window<T>(opk, g, b, smem_bytes, s, L);
    if (variant == 1) return launch_op<T, 1>(opk, g, b, smem_bytes, s, L);
    if (variant == 2) return launch_op<T, 2>(opk, g, b, smem_bytes, s, L);
    if (variant == 5) return launch_op<T, 5>(opk, g, b, smem_bytes, s, L);
    if (variant == 3) return launch_hybrid<T>(opk, g, b, smem_bytes, s, L);
    return launch_op<T, 0>(opk, g, b, 0, s, L);
  }

  template <typename T>
  cudaError_t launch_pack(const T* pts, const uint64_t* off, uint64_t n, Elem<T>* out, uint64_t cap, int sms,
                          cudaStream_t s)
  {
    if (n == 0) return cudaSuccess;
    uint64_t blocks = (n + 7) / 8;
    const uint64_t max_blocks = (uint64_t)sms * 8;
    if (blocks > max_blocks) blocks = max_blocks;
    pack_segments_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(pts, off, n, out, cap);
    return launched();
  }

  template cudaError_t launch_pairs<float>(const LaunchParams<float>&, int, int, int, int, size_t, cudaStream_t);
  template cudaError_t launch_pairs<double>(const LaunchParams<double>&, int, int, int, int, size_t, cudaStream_t);
  template cudaError_t launch_pack<float>(const float*, const uint64_t*, uint64_t, Elem<float>*, uint64_t, int,
                                          cudaStream_t);
  template cudaError_t launch_pack<double>(const double*, const uint64_t*, uint64_t, Elem<double>*, uint64_t, int,
                                           cudaStream_t);

  int kernel_unroll(bool f64) { return f64 ? Unroll<double>::value : Unroll<float>::value; }
}
