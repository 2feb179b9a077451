// Backward pass of the pairwise integrals: given dL/dM for the condensed
// output M (L2 kernel, L2 distance or L1 distance), accumulate dL/dv and
// dL/dt for every breakpoint of every PCF.  The reference has no gradients;
// this differentiates the rectangle sum of integrate()
// (include/sbear/algorithms/functional/matrix_integrate.hpp:18-29) and
// recomputes the merge instead of storing it.
//
// For one pair with weight w = dL/dM_ij and phi(f, g) the integrand
// (f g, (f - g)^2, |f - g|):
//   d/d(value of a rectangle's side) = w s (r - l) d phi / d side
//   d/d t_k (a breakpoint of one side) = w s (phi(before t_k) - phi(after t_k))
// with s = 1 (kernel, L1) or 1 / (2 D_ij) (L2 distance, from the forward
// result; D = 0 contributes nothing).  A breakpoint that coincides with one of
// the other PCF (a tie) has no derivative and gets no time gradient.  The
// kernel's diagonal <f, f> is handled in closed form by diag_backward_kernel.
//
// Work decomposition: the forward kernel's items; a warp merges one row with
// 32 columns.  Each lane keeps running sums for the row segment and the
// column segment it is in and flushes a sum when its side advances: row
// gradients go to a per-warp shared-memory buffer (flushed to global memory
// once per row), column gradients straight to global memory.  (A per-CTA
// shared block for the column gradients measured slower on GB300: the warps
// of an item walk the same columns at similar speed and contend on the same
// shared slots, while global atomics spread over the L2 slices.)  Atomic
// adds: the summation order is not deterministic.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <algorithm>
#include <memory>

namespace sbg
{
  enum BwdOp : int { BWD_INNER = 0, BWD_L2DIST = 1, BWD_L1DIST = 2 };

  template <typename T>
  struct BwdParams
  {
    const Elem<T>* pk;      // packed segment layout at the CSR offsets
    const uint64_t* off;
    uint64_t n;
    uint64_t npts;
    int mode;               // MODE_PDIST or MODE_KERNEL
    uint32_t q;
    uint64_t total_items;
    unsigned long long* queue;
    const T* grad_out;      // condensed dL/dM
    const T* fwd;           // condensed M (distances), or null
    T* grad;                // (npts, 2): [dL/dt, dL/dv]
    uint32_t row_cap;       // per-warp shared gradient buffer (elements)
    uint32_t cols_cap;      // staged column elements per lane (0: columns read through L1)
    const uint32_t* perm;   // processing order -> PCF index (the windowed length order), or null
  };

  namespace
  {
    template <int OP, typename T>
    __device__ __forceinline__ void seg_coeffs(T f, T g, T& cf, T& cg)
    {
      if (OP == BWD_INNER) { cf = g; cg = f; }
      else if (OP == BWD_L2DIST) { cf = f - g; cg = g - f; }
      else
      {
        const T d = f - g;
        cf = d > T(0) ? T(1) : (d < T(0) ? T(-1) : T(0));
        cg = -cf;
      }
    }

    // phi(a, o) - phi(b, o): the change of the integrand when one side's value
    // steps from a to b (at that side's breakpoint), the other side being o.
    template <int OP, typename T>
    __device__ __forceinline__ T step_delta(T a, T b, T o)
    {
      if (OP == BWD_INNER) return (a - b) * o;
      if (OP == BWD_L2DIST) return T(0.5) * ((a - o) * (a - o) - (b - o) * (b - o));
      return fabs(a - o) - fabs(b - o);
    }
  }

  // SIDE 0: the lower triangle, both sides take gradients (the row side in
  // the warp's shared buffer, the column side with global atomics).
  // SIDE 1: every ordered pair (i, j), i != j, and only the warp's own row
  // side takes gradients (each PCF collects its gradients as the row of its
  // pairs); no global atomics inside the merge.
  // SIDE 2: every ordered pair, and only the column side takes gradients
  // (each PCF collects them as a column): every flush is a global vector
  // reduction to an address no other lane of the warp uses, and no shared
  // memory atomics remain.
  //
  // WARP_ITEMS: every warp takes its own items from the queue and walks the
  // item's rows itself, so the warps of a CTA work on different column
  // groups and their column atomics do not meet on the same addresses.
  // Otherwise the CTA takes an item and its warps share the rows.
  // Gradients are accumulated in a paired layout, slot k of a PCF holding
  // (dL/dv_k, dL/dt_{k+1}): a column advance adds to both halves of one
  // 8-byte slot, one vector reduction for float, and a row flush moves whole
  // slots.  pair_to_point_layout writes the (dL/dt, dL/dv) layout at the end.
  __device__ __forceinline__ void red_add2(float* p, float a, float b)
  {
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(a), "f"(b) : "memory");
  }
  __device__ __forceinline__ void red_add2(double* p, double a, double b)
  {
    atomicAdd(p, a);
    atomicAdd(p + 1, b);
  }

  template <typename T, int OP, int SIDE, bool WARP_ITEMS>
  __global__ void __launch_bounds__(1024) pairs_backward_kernel(const __grid_constant__ BwdParams<T> B)
  {
    constexpr bool SQUARE = SIDE != 0, ROWS = SIDE != 2, COLS = SIDE != 1;
    // Shared memory: the item's 32 columns, interleaved (element k of column
    // j at [k * 32 + j]) when cols_cap > 0, then the per-warp row-gradient
    // buffers.
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Elem<T>* cols = reinterpret_cast<Elem<T>*>(smem_raw);
    T* sgrad_all = reinterpret_cast<T*>(cols + (size_t)B.cols_cap * 32);
    const int nwarps = blockDim.x >> 5;
    __shared__ unsigned long long s_item;
    __shared__ unsigned int s_next_row;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    // per warp: dL/dv_k at sgv[k], dL/dt_{k+1} at sgt[k] (two arrays: lanes at
    // nearby row positions then hit distinct banks)
    T* sgv = sgrad_all + (size_t)warp * B.row_cap * 2;
    T* sgt = sgv + B.row_cap;
    const unsigned FULL = 0xffffffffu;

    for (;;)
    {
      unsigned long long item;
      if (WARP_ITEMS)
      {
        if (lane == 0) item = atomicAdd(B.queue, 1ull);
        item = __shfl_sync(FULL, item, 0);
      }
      else
      {
        if (threadIdx.x == 0)
        {
          s_item = atomicAdd(B.queue, 1ull);
          s_next_row = 0;
        }
        __syncthreads();
        item = s_item;
      }
      if (item >= B.total_items) break;
      const uint64_t G = ceil_div_u64(B.n, 32);
      uint64_t c, g;
      if (SQUARE) { c = item / G; g = item % G; }
      else tri_decode(item, 0, B.n, B.q, G, &c, &g);
      uint64_t row_lo = c * 32ull * B.q;
      uint64_t row_hi = row_lo + 32ull * B.q;
      if (row_hi > B.n) row_hi = B.n;
      const uint64_t col0 = 32ull * g;
      if (!SQUARE && row_lo < col0 + 1) row_lo = col0 + 1;  // the diagonal is not handled here

      const uint64_t cj = col0 + lane;
      const bool cvalid = cj < B.n;
      const uint64_t cj_eff = cvalid ? cj : col0;
      // the lane's column in the caller's numbering (processing order -> PCF)
      uint64_t corig = B.perm ? B.perm[cj_eff] : cj_eff;
      if (corig >= B.n) corig = 0;  // never expected: the order is a permutation
      const uint64_t coff = B.off[corig];
      const uint32_t clen = (uint32_t)(B.off[corig + 1] - coff);
      const uint32_t maxlc = __reduce_max_sync(FULL, clen);
      const bool item_ok = !__any_sync(FULL, clen == 0 || coff + clen > B.npts);
      // the same item for every warp: these are CTA-uniform
      const bool staged = !WARP_ITEMS && B.cols_cap > 0 && item_ok && maxlc <= B.cols_cap;
      if (!WARP_ITEMS && B.cols_cap > 0)
      {
        if (staged)
          for (uint32_t k = warp; k < maxlc; k += nwarps)
            if (k < clen) cols[(size_t)k * 32 + lane] = B.pk[coff + k];
        __syncthreads();
      }
      const Elem<T>* colbase = staged ? cols + lane : B.pk + coff;
      const uint32_t cstride = staged ? 32u : 1u;

      if (item_ok)
      {
        for (unsigned next = 0;; ++next)
        {
          unsigned r = next;
          if (!WARP_ITEMS)
          {
            if (lane == 0) r = atomicAdd(&s_next_row, 1u);
            r = __shfl_sync(FULL, r, 0);
          }
          const uint64_t i = row_lo + r;
          if (i >= row_hi) break;
          const uint64_t iorig = B.perm ? B.perm[i] : i;
          if (iorig >= B.n) continue;  // never expected: the order is a permutation
          const uint64_t roff = B.off[iorig];
          const uint32_t rlen = (uint32_t)(B.off[iorig + 1] - roff);
          if (rlen == 0 || rlen > B.row_cap || roff + rlen > B.npts) continue;
          const bool ok = cvalid && (SQUARE ? cj != i : cj < i);
          T w = T(0);
          if (ok)
          {
            const uint64_t idx = condensed_index(B.mode, iorig, corig);
            w = B.grad_out[idx];
            if (OP == BWD_L2DIST)
            {
              const T D = B.fwd[idx];
              w = D > T(0) ? w / D : T(0);
            }
          }
          if (!__any_sync(FULL, w != T(0))) continue;

          if (ROWS)
          {
            for (uint32_t k = lane; k < rlen; k += 32) { sgv[k] = T(0); sgt[k] = T(0); }
            __syncwarp();
          }

          const Elem<T>* row = B.pk + roff;
          Elem<T> F = row[0], Gc = colbase[0];
          uint32_t fi = 0, gi = 0;
          T t = T(0), accF = T(0), accG = T(0);
          const uint32_t steps = rlen + maxlc - 1;
          for (uint32_t s = 0; s < steps; ++s)
          {
            const bool takeF = row_first(F.tn, Gc.tn);
            const T tn = takeF ? F.tn : Gc.tn;
            const T dt = tn - t;
            T cf, cg;
            seg_coeffs<OP>(F.v, Gc.v, cf, cg);
            accF = fma(dt, cf, accF);
            accG = fma(dt, cg, accG);
            // Which side moves on; the row stays on its last element once
            // exhausted (it then runs to TMAX).  Gc.tn < F.tn <= TMAX when the
            // column moves, so the column has a next element.  The loads and
            // adds are predicated rather than branched, so the lanes of a
            // warp do not split into the two sides' paths.
            const bool advF = takeF && fi + 1 < rlen;
            const bool advG = !takeF;
            Elem<T> Fn = F, Gn = Gc;
            if (advF) Fn = row[fi + 1];
            if (advG) Gn = colbase[(size_t)(gi + 1) * cstride];
            if (w != T(0))
            {
              if (ROWS && advF) atomicAdd(&sgv[fi], w * accF);
              if (ROWS && advF && !(F.tn == Gc.tn)) atomicAdd(&sgt[fi], w * step_delta<OP>(F.v, Fn.v, Gc.v));
              // dL/dv of the column element and dL/dt of the next share a slot
              if (COLS && advG)
                red_add2(&B.grad[2 * (coff + gi)], w * accG,
                         (Gc.tn == t) ? T(0) : w * step_delta<OP>(Gc.v, Gn.v, F.v));
            }
            accF = advF ? T(0) : accF;
            accG = advG ? T(0) : accG;
            fi += advF ? 1u : 0u;
            gi += advG ? 1u : 0u;
            F = Fn;
            Gc = Gn;
            t = tn;
          }
          if (ROWS && w != T(0)) atomicAdd(&sgv[fi], w * accF);
          if (COLS && w != T(0)) atomicAdd(&B.grad[2 * (coff + gi)], w * accG);
          if (ROWS)
          {
            __syncwarp();
            for (uint32_t k = lane; k < rlen; k += 32)
            {
              const T gv = sgv[k], gt = sgt[k];
              if (gv != T(0) || gt != T(0)) red_add2(&B.grad[2 * (roff + k)], gv, gt);
            }
            __syncwarp();
          }
        }
      }
      if (!WARP_ITEMS) __syncthreads();
    }
  }

  // The default backward: row-synchronous.  The walk above is free-running:
  // each lane's row advances at its own step, so each lane adds its part of
  // a row element's gradient into the warp's shared buffer with two float
  // atomics, and lanes at the same row position contend for the same slot
  // (the bound: about 46 SM cycles per warp-step at N = 4096).  Here the
  // warp steps through the row one element at a time, all lanes together:
  // for row element k each lane first walks its column's breakpoints before
  // the row's next one (a loop that runs as long as any lane has one), then
  // all lanes take the row's breakpoint, and the 32 lanes' value-gradient
  // and time-gradient terms for element k are summed by a shuffle tree and
  // added to global memory once.  Column gradients leave as in the walk
  // above, one vector reduction per column breakpoint.  The rectangles, the
  // per-rectangle terms and the tie rules (ties go to the row; a breakpoint
  // shared by both PCFs gets no time gradient) are those of the walk; only
  // the order in which the 32 lanes' terms of a row element are added
  // changes.  No shared memory.
  template <typename T, int OP>
  __global__ void __launch_bounds__(1024) pairs_backward_rowsync_kernel(const __grid_constant__ BwdParams<T> B)
  {
    __shared__ unsigned long long s_item;
    __shared__ unsigned int s_next_row;
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;

    for (;;)
    {
      if (threadIdx.x == 0)
      {
        s_item = atomicAdd(B.queue, 1ull);
        s_next_row = 0;
      }
      __syncthreads();
      const unsigned long long item = s_item;
      if (item >= B.total_items) break;
      const uint64_t G = ceil_div_u64(B.n, 32);
      uint64_t c, g;
      tri_decode(item, 0, B.n, B.q, G, &c, &g);
      uint64_t row_lo = c * 32ull * B.q;
      uint64_t row_hi = row_lo + 32ull * B.q;
      if (row_hi > B.n) row_hi = B.n;
      const uint64_t col0 = 32ull * g;
      if (row_lo < col0 + 1) row_lo = col0 + 1;  // the diagonal is handled by diag_backward_kernel

      const uint64_t cj = col0 + lane;
      const bool cvalid = cj < B.n;
      uint64_t corig = B.perm ? B.perm[cvalid ? cj : col0] : (cvalid ? cj : col0);
      if (corig >= B.n) corig = 0;  // never expected: the order is a permutation
      const uint64_t coff = B.off[corig];
      const uint32_t clen = (uint32_t)(B.off[corig + 1] - coff);
      const bool item_ok = !__any_sync(FULL, clen == 0 || coff + clen > B.npts);
      if (item_ok)
      {
        const Elem<T>* col = B.pk + coff;
        T* cgrad = B.grad + 2 * coff;
        for (;;)
        {
          unsigned r = 0;
          if (lane == 0) r = atomicAdd(&s_next_row, 1u);
          r = __shfl_sync(FULL, r, 0);
          const uint64_t i = row_lo + r;
          if (i >= row_hi) break;
          const uint64_t iorig = B.perm ? B.perm[i] : i;
          if (iorig >= B.n) continue;  // never expected: the order is a permutation
          const uint64_t roff = B.off[iorig];
          const uint32_t rlen = (uint32_t)(B.off[iorig + 1] - roff);
          if (rlen == 0 || roff + rlen > B.npts) continue;
          T w = T(0);
          if (cvalid && cj < i)
          {
            const uint64_t idx = condensed_index(B.mode, iorig, corig);
            w = B.grad_out[idx];
            if (OP == BWD_L2DIST)
            {
              const T D = B.fwd[idx];
              w = D > T(0) ? w / D : T(0);
            }
          }
          // lanes with no weight take no part in the walk
          const bool live = w != T(0);
          if (!__any_sync(FULL, live)) continue;

          const Elem<T>* row = B.pk + roff;
          Elem<T> F = row[0];
          Elem<T> Gc = col[0];
          uint32_t gi = 0;
          T t = T(0), accG = T(0);
          for (uint32_t k = 0; k < rlen; ++k)
          {
            const Elem<T> Fn = row[min(k + 1, rlen - 1)];  // the same address in every lane
            T accF = T(0);
            // this lane's column breakpoints before the row's next one (ties
            // go to the row); Gc.tn < F.tn <= TMAX, so the column has a next
            // element
            for (;;)
            {
              const bool adv = live && Gc.tn < F.tn;
              if (!__any_sync(FULL, adv)) break;
              if (adv)
              {
                const T dt = Gc.tn - t;
                T cf, cg;
                seg_coeffs<OP>(F.v, Gc.v, cf, cg);
                accF = fma(dt, cf, accF);
                accG = fma(dt, cg, accG);
                const Elem<T> Gn = col[gi + 1];
                red_add2(&cgrad[2 * (size_t)gi], w * accG,
                         dt == T(0) ? T(0) : w * step_delta<OP>(Gc.v, Gn.v, F.v));
                accG = T(0);
                t = Gc.tn;
                Gc = Gn;
                ++gi;
              }
            }
            // the row's breakpoint (for its last element, the last rectangle to TMAX)
            T rowT = T(0);
            if (live)
            {
              const T dt = F.tn - t;
              T cf, cg;
              seg_coeffs<OP>(F.v, Gc.v, cf, cg);
              accF = fma(dt, cf, accF);
              accG = fma(dt, cg, accG);
              if (k + 1 < rlen)
              {
                if (Gc.tn == F.tn)
                {
                  // the column's breakpoint coincides: it moves too, and
                  // neither breakpoint gets a time gradient
                  const Elem<T> Gn = col[min(gi + 1, clen - 1)];
                  red_add2(&cgrad[2 * (size_t)gi], w * accG, T(0));
                  accG = T(0);
                  Gc = Gn;
                  gi = min(gi + 1, clen - 1);
                }
                else
                  rowT = w * step_delta<OP>(F.v, Fn.v, Gc.v);
              }
              t = F.tn;
            }
            T rowV = w * accF;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
            {
              rowV += __shfl_xor_sync(FULL, rowV, o);
              rowT += __shfl_xor_sync(FULL, rowT, o);
            }
            if (lane == 0 && (rowV != T(0) || rowT != T(0))) red_add2(&B.grad[2 * (roff + k)], rowV, rowT);
            F = Fn;
          }
          if (live) atomicAdd(&cgrad[2 * (size_t)gi], w * accG);
        }
      }
      __syncthreads();
    }
  }

  // The default backward: the row walked in windows of W elements.  The
  // row-synchronous walk above waits, at every row element, for the lane
  // with the most column breakpoints before the next row breakpoint (about
  // 5 for a mean of 1 on the fwd + bwd workload).  Here the lanes walk
  // freely through W row elements at a time, with the walk's own step (ties
  // go to the row; a zero-width column step gets no time gradient), and a
  // lane that leaves row element k stores its value- and time-gradient terms
  // for k in its own slot of a per-warp [W][32] shared array: a plain store,
  // no atomics, no bank conflicts (lane l's slot is at bank pair l % 16).
  // When every lane has left the window's last element, the 32 slots of each
  // element are summed (two lanes per element, a skewed read order) and
  // added to global memory once.  Lanes with no weight take no part and
  // leave zeros in their slots.  Column gradients leave as in the walks
  // above.
  //
  // STAGED: the item's 32 columns are first copied into shared memory,
  // element k of column l at [k * 32 + l] after the slots (B.cols_cap
  // elements per column), so the walk reads them with conflict-free shared
  // loads instead of one L1 request of 8 sectors per warp-step; the host
  // picks it when the columns and the slots of 32 warps fit.
  template <typename T, int OP, int W, bool STAGED>
  __global__ void __launch_bounds__(STAGED ? 1024 : 512) pairs_backward_window_kernel(
      const __grid_constant__ BwdParams<T> B)
  {
    static_assert(W >= 1 && W <= 16, "two lanes per window element");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ unsigned long long s_item;
    __shared__ unsigned int s_next_row;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const unsigned FULL = 0xffffffffu;
    // slot (element j of the window, lane l) at [j * 32 + l]: (value-gradient term, time-gradient term)
    Elem<T>* slots = reinterpret_cast<Elem<T>*>(smem_raw) + (size_t)warp * W * 32;
    Elem<T>* cols_s = reinterpret_cast<Elem<T>*>(smem_raw) + (size_t)nwarps * W * 32;

    for (;;)
    {
      if (threadIdx.x == 0)
      {
        s_item = atomicAdd(B.queue, 1ull);
        s_next_row = 0;
      }
      __syncthreads();
      const unsigned long long item = s_item;
      if (item >= B.total_items) break;
      const uint64_t G = ceil_div_u64(B.n, 32);
      uint64_t c, g;
      tri_decode(item, 0, B.n, B.q, G, &c, &g);
      uint64_t row_lo = c * 32ull * B.q;
      uint64_t row_hi = row_lo + 32ull * B.q;
      if (row_hi > B.n) row_hi = B.n;
      const uint64_t col0 = 32ull * g;
      if (row_lo < col0 + 1) row_lo = col0 + 1;  // the diagonal is handled by diag_backward_kernel

      const uint64_t cj = col0 + lane;
      const bool cvalid = cj < B.n;
      uint64_t corig = B.perm ? B.perm[cvalid ? cj : col0] : (cvalid ? cj : col0);
      if (corig >= B.n) corig = 0;  // never expected: the order is a permutation
      const uint64_t coff = B.off[corig];
      const uint32_t clen = (uint32_t)(B.off[corig + 1] - coff);
      const uint32_t maxlc = __reduce_max_sync(FULL, clen);  // warp-uniform: bounds the walk below
      // Every warp of the CTA holds the same 32 columns, so item_ok (and
      // with it the staging barrier below) is the same in all of them.  A
      // column longer than the host's max_points (never expected) skips the
      // item, as the other walks skip such rows.
      const bool item_ok =
          !__any_sync(FULL, clen == 0 || coff + clen > B.npts) && (!STAGED || maxlc <= B.cols_cap);
      if (item_ok)
      {
        const Elem<T>* col = B.pk + coff;
        T* cgrad = B.grad + 2 * coff;
        if constexpr (STAGED)
        {
          for (uint32_t k = (uint32_t)warp; k < clen; k += (uint32_t)nwarps) cols_s[(size_t)k * 32 + lane] = col[k];
          __syncthreads();
        }
        auto colat = [&](uint32_t k) -> Elem<T> {
          if constexpr (STAGED) return cols_s[(size_t)k * 32 + lane];
          else return col[k];
        };
        for (;;)
        {
          unsigned r = 0;
          if (lane == 0) r = atomicAdd(&s_next_row, 1u);
          r = __shfl_sync(FULL, r, 0);
          const uint64_t i = row_lo + r;
          if (i >= row_hi) break;
          const uint64_t iorig = B.perm ? B.perm[i] : i;
          if (iorig >= B.n) continue;  // never expected: the order is a permutation
          const uint64_t roff = B.off[iorig];
          const uint32_t rlen = (uint32_t)(B.off[iorig + 1] - roff);
          if (rlen == 0 || roff + rlen > B.npts) continue;
          T w = T(0);
          if (cvalid && cj < i)
          {
            const uint64_t idx = condensed_index(B.mode, iorig, corig);
            w = B.grad_out[idx];
            if (OP == BWD_L2DIST)
            {
              const T D = B.fwd[idx];
              w = D > T(0) ? w / D : T(0);
            }
          }
          const bool live = w != T(0);
          if (!__any_sync(FULL, live)) continue;
          if (!live)
            for (int j = 0; j < W; ++j) slots[j * 32 + lane] = Elem<T>{T(0), T(0)};

          // Next elements are read one (column) or two (row) places past a
          // PCF's end without a clamp: the packed layout has two spare
          // elements after the last PCF and the staged columns one spare
          // row, and a value read there is never used (a side's last element
          // ends at TMAX, so it is never left before the walk ends).
          const Elem<T>* row = B.pk + roff;
          Elem<T> F = row[0], F2 = row[1];
          const Elem<T>* rnext = row + 2;
          Elem<T> Gc = colat(0), G2 = colat(1);
          uint32_t fi = 0, gi = 0;
          T* cgp = cgrad;
          T t = T(0), accF = T(0), accG = T(0);
          T wF = w * F.v, wG = w * Gc.v;  // used by the L2 kernel's walk only
          for (uint32_t kb = 0; kb < rlen; kb += W)
          {
            const uint32_t ke = min(kb + (uint32_t)W, rlen);
            const uint32_t kel = live ? ke : 0u;  // lanes with no weight take no step
            Elem<T>* sp = slots + lane;           // this lane's slot for row element fi (fi == kb here)
            // One step of the walk (the lane's next rectangle).  For the L2
            // kernel the weight rides on each side's value (wF = w F.v,
            // wG = w Gc.v, renewed when a side moves), so a flush multiplies
            // by nothing more.  (The same for the L2 distance, whose step
            // term then reads (a - b)(wa + wb - 2 wo) / 2, measured slower:
            // 15.29 against 14.89 ms forward + backward at N = 4096.)
            auto step = [&]() {
              const bool takeF = row_first(F.tn, Gc.tn);
              const T tn = takeF ? F.tn : Gc.tn;
              const T dt = tn - t;
              if constexpr (OP == BWD_INNER)
              {
                accF = fma(dt, wG, accF);
                accG = fma(dt, wF, accG);
              }
              else
              {
                T cf, cg;
                seg_coeffs<OP>(F.v, Gc.v, cf, cg);
                accF = fma(dt, cf, accF);
                accG = fma(dt, cg, accG);
              }
              if (takeF)
              {
                // leave row element fi; a breakpoint shared with the
                // column, or the row's end, has no time gradient
                const bool none = F.tn == Gc.tn || fi + 1 >= rlen;
                if constexpr (OP == BWD_INNER)
                  *sp = Elem<T>{accF, none ? T(0) : (F.v - F2.v) * wG};
                else
                  *sp = Elem<T>{w * accF, none ? T(0) : w * step_delta<OP>(F.v, F2.v, Gc.v)};
                sp += 32;
                accF = T(0);
                F = F2;
                ++fi;
                F2 = *rnext++;
                if constexpr (OP == BWD_INNER) wF = w * F.v;
              }
              else
              {
                // Gc.tn < F.tn <= TMAX: the column has a next element, G2
                if constexpr (OP == BWD_INNER)
                  red_add2(cgp, accG, dt == T(0) ? T(0) : (Gc.v - G2.v) * wF);
                else
                  red_add2(cgp, w * accG, dt == T(0) ? T(0) : w * step_delta<OP>(Gc.v, G2.v, F.v));
                cgp += 2;
                accG = T(0);
                Gc = G2;
                ++gi;
                G2 = colat(gi + 1);
                if constexpr (OP == BWD_INNER) wG = w * Gc.v;
              }
              t = tn;
            };
            // Walk until this lane has left row element ke - 1 (for the last
            // element: taken the last rectangle, to TMAX).  A lane takes at
            // most W row steps and clen - 1 column steps in a window, so the
            // bound W + maxlc ends the loop whatever the data; it is the same
            // in every lane, so all 32 lanes run every iteration's vote.
            // Two steps per vote; a lane that leaves the window after the
            // first takes no second one.
            for (uint32_t guard = 0; guard <= (uint32_t)W + maxlc; ++guard)
            {
              if (!__any_sync(FULL, fi < kel)) break;
              if (fi < kel) step();
              if (fi < kel) step();
            }
            __syncwarp();
            // element j of the window: lanes j and j + 16 each sum 16 of its
            // 32 slots, in an order skewed by j so that the lanes of a
            // half-warp read 16 different bank pairs
            const uint32_t nel = ke - kb;
            const uint32_t j = lane & 15, h = lane >> 4;
            T sv = T(0), st = T(0);
            if (j < nel)
            {
#pragma unroll
              for (int m = 0; m < 16; ++m)
              {
                const Elem<T> s = slots[j * 32 + h * 16 + ((m + j) & 15)];
                sv += s.v;
                st += s.tn;
              }
            }
            sv += __shfl_xor_sync(FULL, sv, 16);
            st += __shfl_xor_sync(FULL, st, 16);
            if (h == 0 && j < nel && (sv != T(0) || st != T(0))) red_add2(&B.grad[2 * (roff + kb + j)], sv, st);
            __syncwarp();
          }
          if (live) atomicAdd(cgp, OP == BWD_INNER ? accG : w * accG);
        }
      }
      __syncthreads();
    }
  }

  // (dL/dv_k, dL/dt_{k+1}) slots to the point layout (dL/dt_k, dL/dv_k).
  // The slot of a PCF's last element holds no time gradient (there is no
  // breakpoint after it).  One warp per PCF.
  template <typename T>
  __global__ void pair_to_point_layout(const T* __restrict__ gp, const uint64_t* __restrict__ off, uint64_t n,
                                       uint64_t npts, T* __restrict__ grad)
  {
    const uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (gridDim.x * (uint64_t)blockDim.x) >> 5;
    for (uint64_t i = wid; i < n; i += nw)
    {
      const uint64_t o = off[i], len = off[i + 1] - o;
      if (o + len > npts) continue;
      for (uint64_t k = lane; k < len; k += 32)
      {
        grad[2 * (o + k)] = k == 0 ? T(0) : gp[2 * (o + k - 1) + 1];
        grad[2 * (o + k) + 1] = gp[2 * (o + k)];
      }
    }
  }

  // <f, f> = sum_k v_k^2 (t_{k+1} - t_k):  d/dv_k = 2 v_k (t_{k+1} - t_k),
  // d/dt_k = v_{k-1}^2 - v_k^2, weighted by dL/dK_ii.  One warp per PCF.
  template <typename T>
  __global__ void diag_backward_kernel(const Elem<T>* __restrict__ pk, const uint64_t* __restrict__ off, uint64_t n,
                                       uint64_t npts, const T* __restrict__ grad_out, T* __restrict__ grad)
  {
    const uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (gridDim.x * (uint64_t)blockDim.x) >> 5;
    for (uint64_t i = wid; i < n; i += nw)
    {
      const uint64_t o = off[i], len = off[i + 1] - o;
      if (len == 0 || o + len > npts) continue;
      const T w = grad_out[i * (i + 1) / 2 + i];
      if (w == T(0)) continue;
      for (uint64_t k = lane; k < len; k += 32)
      {
        const Elem<T> e = pk[o + k];
        const T tk = (k == 0) ? T(0) : pk[o + k - 1].tn;
        grad[2 * (o + k) + 1] += w * (T(2) * (e.v * (e.tn - tk)));
        if (k > 0)
        {
          const T a = pk[o + k - 1].v;
          grad[2 * (o + k)] += w * (a * a - e.v * e.v);
        }
      }
    }
  }

  constexpr bool defined_stage_columns()
  {
#if defined(SBG_BWD_STAGE_COLUMNS)
    return true;
#else
    return false;
#endif
  }

  template <typename T>
  static void backward_device(int op, double p, int mode, const T* pts, const uint64_t* off, uint64_t n,
                              uint64_t npts, uint32_t lmax, const T* grad_out, const T* fwd, T* grad, cudaStream_t st)
  {
    int bop;
    if (mode == MODE_KERNEL && op == SBG_OP_L2_INNER) bop = BWD_INNER;
    else if (mode == MODE_PDIST && op == SBG_OP_LP && p == 2.0) bop = BWD_L2DIST;
    else if (mode == MODE_PDIST && (op == SBG_OP_L1 || (op == SBG_OP_LP && p == 1.0))) bop = BWD_L1DIST;
    else throw Error(ST_INVALID_ARGUMENT, "gradients exist for the L2 kernel (SBG_SKIP_LOWER), and L2 or L1 pdist");
    if (bop == BWD_L2DIST && !fwd) throw Error(ST_INVALID_ARGUMENT, "the L2-distance gradient needs the forward result");
    if (lmax == 0) throw Error(ST_INVALID_ARGUMENT, "max_points must be given");
    const DeviceInfo dev = device_info();
    SBG_CUDA(cudaMemsetAsync(grad, 0, sizeof(T) * 2 * npts, st));
    if (n == 0) return;

    // two spare elements after the last PCF: the windowed walk reads up to
    // two places past a PCF's end (values it never uses)
    StreamBuffer packed_buf((npts + 2) * sizeof(Elem<T>), st);
    StreamBuffer queue_buf(256, st);
    StreamBuffer paired_buf(std::max<uint64_t>(1, npts) * 2 * sizeof(T), st);
    StreamBuffer order_buf(n * sizeof(uint32_t), st);
    void* packed = packed_buf.get();
    void* queue = queue_buf.get();
    void* paired = paired_buf.get();
    void* order = order_buf.get();
    // The forward's processing order (windows of 1024 PCFs by length): the
    // 32 columns of a group then have similar lengths, so the warp-uniform
    // step count wastes little.  Gradients land at the PCFs' own offsets.
    length_order_device(off, n, static_cast<uint32_t*>(order), nullptr, st);
    SBG_CUDA(cudaMemsetAsync(paired, 0, std::max<uint64_t>(1, npts) * 2 * sizeof(T), st));
    SBG_CUDA(launch_pack<T>(pts, off, n, static_cast<Elem<T>*>(packed), npts, dev.sms, st));

    BwdParams<T> B{};
    B.pk = static_cast<const Elem<T>*>(packed);
    B.off = off; B.n = n; B.npts = npts; B.mode = mode;
    B.grad_out = grad_out; B.fwd = fwd; B.grad = static_cast<T*>(paired);
    B.queue = static_cast<unsigned long long*>(queue);
    B.row_cap = lmax;
    B.perm = static_cast<const uint32_t*>(order);
    // As many warps (up to 32) as the per-warp row-gradient buffers allow:
    // the merge is latency-bound, so occupancy pays.  Columns are read
    // through L1: staging them in shared memory (behind
    // SBG_BWD_STAGE_COLUMNS) costs warps and measured slower (N = 4096, L2
    // kernel, forward + backward: 26.4 ms with 24 warps and staged columns
    // against 25.6 ms with 32 warps).
#if defined(SBG_BWD_SQUARE_COLUMNS)
    constexpr int SIDE = 2;
#elif defined(SBG_BWD_SQUARE)
    constexpr int SIDE = 1;
#else
    constexpr int SIDE = 0;
#endif
    constexpr bool SQ = SIDE != 0;
#ifdef SBG_BWD_WARP_ITEMS
    constexpr bool WI = true;
#else
    constexpr bool WI = false;
#endif
    // The walk in windows of row elements (the default), the row-synchronous
    // walk (SBG_BWD_ROWSYNC) or the free-running walk with per-warp
    // row-gradient buffers (SBG_BWD_LEGACY and the alternatives above).
#if defined(SBG_BWD_LEGACY)
    constexpr int WALK = 0;
#elif defined(SBG_BWD_ROWSYNC)
    constexpr int WALK = 1;
#else
    constexpr int WALK = 2;
#endif
    constexpr bool ROWSYNC = WALK == 1 && SIDE == 0 && !WI && !defined_stage_columns();
    constexpr bool WINDOWED = WALK == 2 && SIDE == 0 && !WI && !defined_stage_columns();
    // The windowed walk with columns read through L1 (f64, long PCFs, or
    // SBG_BWD_UNSTAGED).  Forward + backward on GB300 (N = 4096 f32,
    // L ~ U{16..512}; L2 kernel / L2 distance, ms): W = 4 21.6 / 22.4,
    // W = 8 19.5 / 20.2, W = 16 18.4 / 19.3; the row-synchronous walk
    // 18.5 / 19.6; the free-running walk with per-warp buffers 24.7 / 24.8.
    // W = 16 holds 64 KB of slots per 16-warp block in f32 and 128 KB in f64.
#ifndef SBG_BWD_WINDOW
#define SBG_BWD_WINDOW 16
#endif
    constexpr int BWD_W = SBG_BWD_WINDOW;  // row elements per window
    // per-warp row-gradient buffers (none when only columns take gradients,
    // nor in the row-synchronous and windowed walks)
    const size_t grad_per_warp = (SIDE == 2 || ROWSYNC || WINDOWED) ? 0 : (size_t)lmax * 2 * sizeof(T);
    const size_t cols_bytes = (size_t)32 * lmax * sizeof(Elem<T>);
    const size_t budget = dev.smem_optin > 2048 ? dev.smem_optin - 2048 : 0;
#if defined(SBG_BWD_STAGE_COLUMNS) && !defined(SBG_BWD_WARP_ITEMS)
    const bool stage = cols_bytes + 16 * grad_per_warp <= budget;
#else
    const bool stage = false;
#endif
    // The windowed walk with the item's columns staged in shared memory:
    // 32 warps and the widest window, 12 or 8 elements, whose slots fit
    // beside the columns (float32 PCFs up to about 515 or 640 breakpoints).
    // Forward + backward on GB300 (N = 4096 f32, L ~ U{16..512}; L2 kernel /
    // L2 distance, ms): staged W = 12 16.5 / 17.3, W = 10 16.7 / 17.6,
    // W = 8 17.0 / 17.9, W = 4 18.4 / 19.4; unstaged W = 16 18.4 / 19.3.
    // Staged W = 16 fits 24 warps only: 16.3 / 16.3 against 16.2 / 16.2 for
    // W = 12 with 32 warps (both with two steps per vote).
#if defined(SBG_BWD_UNSTAGED)
    constexpr bool ALLOW_STAGED = false;
#else
    constexpr bool ALLOW_STAGED = true;
#endif
    // the staged columns keep one spare row (the walk reads one place past a column's end)
    const size_t scols_bytes = (size_t)32 * (lmax + 1) * sizeof(Elem<T>);
    auto staged_fits = [&](int w) { return (size_t)32 * w * 32 * sizeof(Elem<T>) + scols_bytes <= budget; };
    // float32 only: the f64 walk is bound by the FP64 pipe, and its staged
    // form would spill at 32 warps.
    const int BWD_WS =
        (WINDOWED && ALLOW_STAGED && sizeof(T) == 4) ? (staged_fits(12) ? 12 : staged_fits(8) ? 8 : 0) : 0;
    const bool wstage = BWD_WS > 0;
    B.cols_cap = (stage || wstage) ? lmax : 0;
    const size_t fixed = stage ? cols_bytes : 0;
    int warps = wstage ? 32 : WINDOWED ? 16 : 32;
    while (warps > 1 && fixed + (size_t)warps * grad_per_warp > budget) warps /= 2;
    if (stage) while (warps < 32 && fixed + (size_t)(warps + 8) * grad_per_warp <= budget) warps += 8;
    // the windowed walk: one [W][32] slot array per warp (then the staged columns)
    const size_t smem = wstage     ? (size_t)warps * BWD_WS * 32 * sizeof(Elem<T>) + scols_bytes
                        : WINDOWED ? (size_t)warps * BWD_W * 32 * sizeof(Elem<T>)
                                   : fixed + (size_t)warps * grad_per_warp;
    if (smem > budget) throw Error(ST_INVALID_ARGUMENT, "PCFs too long for the backward kernel's row buffers");
    // The ordered-pairs variants measured slower on GB300 (N = 4096, L2
    // kernel): rows only, forward + backward 74 ms against 46 ms at the time
    // (twice the merges, and the lanes' shared-memory adds into one row
    // buffer contend); columns only, backward 25.7 against 20.8 ms (every
    // flush a global reduction: the L2 atomic units bound it).  They stay
    // available for measurement behind SBG_BWD_SQUARE and
    // SBG_BWD_SQUARE_COLUMNS.
    // Per-warp items measured slower (58 against 50 ms): the column atomics
    // were not colliding; they stay available behind SBG_BWD_WARP_ITEMS.
    const uint64_t G = ceil_div_u64(n, 32);
    auto items = [&](uint32_t qq) { return SQ ? ceil_div_u64(n, 32ull * qq) * G : tri_item_count(0, n, qq, G); };
    // At least 12 work items per SM, with the largest rows per item (up to
    // 256) that give them: forward + backward at N = 4096 (L2 kernel)
    // measured 15.10 ms with 6 items per SM, 14.84 with 12, 14.81 with 24
    // and 14.92 with 48.
#ifndef SBG_BWD_ITEMS_PER_SM
#define SBG_BWD_ITEMS_PER_SM 12
#endif
    const uint64_t want_items = (uint64_t)dev.sms * (WI ? warps * 4 : SBG_BWD_ITEMS_PER_SM);
    uint32_t q = 1;
    for (uint32_t cand = 8; cand >= 1; cand /= 2)
      if (items(cand) >= want_items) { q = cand; break; }
    B.q = q;
    B.total_items = items(q);
    SBG_CUDA(cudaMemsetAsync(queue, 0, 8, st));
    if (B.total_items > 0)
    {
      void (*staged_fn)(const BwdParams<T>) = nullptr;
      if constexpr (sizeof(T) == 4)
        staged_fn = BWD_WS == 12 ? (bop == BWD_INNER ? pairs_backward_window_kernel<T, BWD_INNER, 12, true>
                                    : bop == BWD_L2DIST ? pairs_backward_window_kernel<T, BWD_L2DIST, 12, true>
                                                        : pairs_backward_window_kernel<T, BWD_L1DIST, 12, true>)
                                 : (bop == BWD_INNER ? pairs_backward_window_kernel<T, BWD_INNER, 8, true>
                                    : bop == BWD_L2DIST ? pairs_backward_window_kernel<T, BWD_L2DIST, 8, true>
                                                        : pairs_backward_window_kernel<T, BWD_L1DIST, 8, true>);
      void (*fn)(const BwdParams<T>) =
          wstage ? staged_fn
          : WINDOWED ? (bop == BWD_INNER ? pairs_backward_window_kernel<T, BWD_INNER, BWD_W, false>
                      : bop == BWD_L2DIST ? pairs_backward_window_kernel<T, BWD_L2DIST, BWD_W, false>
                                          : pairs_backward_window_kernel<T, BWD_L1DIST, BWD_W, false>)
          : ROWSYNC ? (bop == BWD_INNER ? pairs_backward_rowsync_kernel<T, BWD_INNER>
                       : bop == BWD_L2DIST ? pairs_backward_rowsync_kernel<T, BWD_L2DIST>
                                           : pairs_backward_rowsync_kernel<T, BWD_L1DIST>)
                    : (bop == BWD_INNER ? pairs_backward_kernel<T, BWD_INNER, SIDE, WI>
                       : bop == BWD_L2DIST ? pairs_backward_kernel<T, BWD_L2DIST, SIDE, WI>
                                           : pairs_backward_kernel<T, BWD_L1DIST, SIDE, WI>);
      SBG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      // persistent CTAs: as many per SM as registers, threads and shared memory allow
      int per_sm = 1;
      SBG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, warps * 32, smem));
      per_sm = std::max(1, per_sm);
      const unsigned grid = (unsigned)std::min<uint64_t>(B.total_items, (uint64_t)dev.sms * per_sm);
      fn<<<grid, warps * 32, smem, st>>>(B);
      SBG_CUDA(launched());
    }
    {
      const unsigned blocks = (unsigned)std::min<uint64_t>((n + 7) / 8, (uint64_t)dev.sms * 8);
      pair_to_point_layout<T><<<blocks, 256, 0, st>>>(static_cast<const T*>(paired), off, n, npts, grad);
      SBG_CUDA(launched());
    }
    if (bop == BWD_INNER)
    {
      // after the layout pass on the same stream: plain adds are race-free
      const unsigned blocks = (unsigned)std::min<uint64_t>((n + 7) / 8, (uint64_t)dev.sms * 8);
      diag_backward_kernel<T><<<blocks, 256, 0, st>>>(B.pk, off, n, npts, grad_out, grad);
      SBG_CUDA(launched());
    }
  }
}

extern "C" int sbg_pairwise_backward_device(int dtype, int op, double p, int skip_mode, const void* points,
                                            const uint64_t* offsets, uint64_t n, uint64_t n_points,
                                            uint32_t max_points, const void* grad_out, const void* forward_out,
                                            void* grad_points, void* stream)
{
  using namespace sbg;
  try
  {
    if (dtype != SBG_F32 && dtype != SBG_F64) throw Error(ST_INVALID_ARGUMENT, "dtype must be SBG_F32 or SBG_F64");
    if (skip_mode != SBG_SKIP_LOWER && skip_mode != SBG_SKIP_LOWER_NODIAG)
      throw Error(ST_INVALID_ARGUMENT, "gradients are defined for pdist and l2 kernel outputs");
    if (n > 0 && (!points || !offsets || !grad_out || !grad_points)) throw Error(ST_INVALID_ARGUMENT, "null pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == SBG_F32)
      backward_device<float>(op, p, skip_mode, static_cast<const float*>(points), offsets, n, n_points, max_points,
                             static_cast<const float*>(grad_out), static_cast<const float*>(forward_out),
                             static_cast<float*>(grad_points), st);
    else
      backward_device<double>(op, p, skip_mode, static_cast<const double*>(points), offsets, n, n_points, max_points,
                              static_cast<const double*>(grad_out), static_cast<const double*>(forward_out),
                              static_cast<double*>(grad_points), st);
    set_last_error("");
    return SBG_OK;
  }
  catch (const Error& e)
  {
    set_last_error(e.what());
    return e.status;
  }
  catch (const std::exception& e)
  {
    set_last_error(e.what());
    return SBG_ERR_INTERNAL;
  }
}
