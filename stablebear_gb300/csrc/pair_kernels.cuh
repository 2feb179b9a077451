// Pairwise PCF integration kernels for sm_103a (GB300).
//
// One pass computes, for every requested pair (i, j), the integral
//   I(i, j) = sum over merged rectangles [l, r) of (r - l) * op(f_i, f_j)
// followed by op's finalizer, exactly as stablebear's rectangle walk does
// (include/sbear/algorithms/functional/iterate_rectangles.hpp:37-104 and
// include/sbear/algorithms/functional/matrix_integrate.hpp:18-29), with the
// last rectangle running to numeric_limits<T>::max()
// (include/sbear/functional/time_point.hpp:10-14).
//
// Work decomposition (GB300-first; the reference runs one thread per pair over
// dense tiles, cuda_pcf_kernel.cuh:95-136):
//   * a work item is (problem, chunk of 32*Q rows, group of 32 columns);
//   * persistent CTAs (one per SM) pull items from a device queue;
//   * the 32 columns of the item are staged in shared memory *interleaved*
//     (element k of column j at [k*32 + j]), so a warp whose lanes sit at
//     different merge positions still reads 32 distinct banks;
//   * each warp takes rows from a CTA-local counter; lane j merges the row
//     with column j; the row lives in a warp-private shared buffer;
//   * every lane runs the same, warp-uniform number of merge steps: each step
//     advances exactly one side (ties become zero-width rectangles), so the
//     step count of a pair is L_i + L_j - 1 including the last rectangle,
//     known up front — no data-dependent loop exit, no divergence;
//   * sums are compensated: naive sums over blocks of U rectangles, the
//     block sums combined with Kahan's algorithm;
//   * results are written straight into the reference's condensed storage
//     order (DistanceMatrix: i*(i-1)/2 + j, distance_matrix.hpp:141-146;
//     SymmetricMatrix: i*(i+1)/2 + j, symmetric_matrix.hpp:257-259) or dense
//     row-major (cdist), coalesced along j for a fixed row.
//
// Storage of one PCF in the merge buffers ("segment layout"): element k holds
// (v_k, t_{k+1}) — the value on [t_k, t_{k+1}) and the time where it ends —
// with t_L replaced by TMAX = numeric_limits<T>::max().  Both PCFs start at
// t = 0 (the input contract, pypcf_support.hpp:84-89), so the walk starts at
// t = 0 with (v_0, w_0).  When both sides reach TMAX the next step emits the
// reference's last rectangle [t_last, TMAX) and every later step has width 0.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

namespace sbg
{
  enum Mode : int { MODE_CROSS = 0, MODE_PDIST = 1, MODE_KERNEL = 2 };
  enum OpKind : int { OPK_L1 = 0, OPK_L2DIST = 1, OPK_LP = 2, OPK_INNER = 3 };

  template <typename T> struct alignas(2 * sizeof(T)) Elem { T v; T tn; };

  template <typename T> __host__ __device__ constexpr T tmax_of();
  template <> __host__ __device__ constexpr float tmax_of<float>() { return FLT_MAX; }
  template <> __host__ __device__ constexpr double tmax_of<double>() { return DBL_MAX; }

  // ---- pair operations (operations.cuh:19-65) -----------------------------
  // seg(dt, f, g) = dt * op(f, g) with the reference's association; fin(x)
  // is op's finalizer.

  template <int K> struct PairOp;

  // acc(blk, dt, f, g) = blk + dt * op(f, g), with dt * op folded into one
  // fused multiply-add (one rounding fewer than the reference's separate
  // product and sum; the sum is compensated anyway).
  template <> struct PairOp<OPK_L1>
  {
    // |dt * (f - g)| == dt * |f - g| bit for bit, since dt >= 0.
    template <typename T> __device__ static __forceinline__ T seg(T dt, T f, T g, T) { return fabs(dt * (f - g)); }
    template <typename T> __device__ static __forceinline__ T acc(T blk, T dt, T f, T g, T)
    {
      return fma(fabs(f - g), dt, blk);
    }
    template <typename T> __device__ static __forceinline__ T fin(T x, T) { return x; }
  };

  // Lp with p == 2: pow(|d|, 2) and pow(x, 1/2) evaluated as d*d and a
  // correctly rounded sqrt (the values a correctly rounded pow returns).
  template <> struct PairOp<OPK_L2DIST>
  {
    template <typename T> __device__ static __forceinline__ T seg(T dt, T f, T g, T)
    {
      T d = f - g;
      return dt * (d * d);
    }
    template <typename T> __device__ static __forceinline__ T acc(T blk, T dt, T f, T g, T)
    {
      const T d = f - g;
      return fma(d * d, dt, blk);
    }
    template <typename T> __device__ static __forceinline__ T fin(T x, T) { return sqrt(x); }
  };

  template <> struct PairOp<OPK_LP>
  {
    template <typename T> __device__ static __forceinline__ T seg(T dt, T f, T g, T p) { return dt * pow(fabs(f - g), p); }
    template <typename T> __device__ static __forceinline__ T acc(T blk, T dt, T f, T g, T p)
    {
      return fma(pow(fabs(f - g), p), dt, blk);
    }
    template <typename T> __device__ static __forceinline__ T fin(T x, T p) { return pow(x, T(1) / p); }
  };

  template <> struct PairOp<OPK_INNER>
  {
    template <typename T> __device__ static __forceinline__ T seg(T dt, T f, T g, T) { return dt * (f * g); }
    template <typename T> __device__ static __forceinline__ T acc(T blk, T dt, T f, T g, T)
    {
      return fma(f * g, dt, blk);
    }
    template <typename T> __device__ static __forceinline__ T fin(T x, T) { return x; }
  };

  // The earlier of two breakpoint times.  float: one FMNMX.  double: the
  // times are >= 0 (or clamped to TMAX), where the IEEE order equals the
  // order of the bit patterns as signed 64-bit integers, so the compare and
  // select run on the integer pipe instead of the (much narrower) FP64 pipe.
  __device__ __forceinline__ float earlier(float a, float b) { return fminf(a, b); }
  __device__ __forceinline__ double earlier(double a, double b)
  {
    return (__double_as_longlong(a) <= __double_as_longlong(b)) ? a : b;
  }
  // Whether the row side advances (its next time is not later; ties go to
  // the row), with the same integer-order trick for double.
  __device__ __forceinline__ bool row_first(float a, float b) { return a <= b; }
  __device__ __forceinline__ bool row_first(double a, double b)
  {
    return __double_as_longlong(a) <= __double_as_longlong(b);
  }

  // ---- problem descriptors ----------------------------------------------

  // One independent pairwise problem (pdist / kernel / cdist) inside a
  // launch.  Row and column sets use the reference's CSR: interleaved (t, v)
  // points, u64 offsets (offset_data_manager.hpp:42-68).  *perm maps the
  // processing order to the caller's PCF index (NULL = identity); the kernel
  // visits PCFs in processing order but always writes the caller's (i, j).
  template <typename T>
  struct ProblemDesc
  {
    const T* rpts; const uint64_t* roff; const uint32_t* rperm; uint64_t nr;
    const T* cpts; const uint64_t* coff; const uint32_t* cperm; uint64_t nc;
    T* out;            // output buffer; element index minus out_base
    uint64_t out_base;
    uint64_t out_count;  // stores outside [out_base, out_base + out_count) are dropped
    uint64_t ld;       // dense leading dimension (cross mode)
    uint64_t row_begin, row_end;  // processing-order rows of this launch (row_begin % (32*q) == 0)
    uint64_t item_begin;          // first global item of this problem
    uint64_t n_items;
    uint32_t q;        // rows per chunk = 32 * q
    int mode;
    T p;
    // Global-memory variant: elements in the packed row / column arrays.
    // Rows or column groups whose offsets reach past them are skipped.
    uint64_t rcap, ccap;
  };

  // probs == nullptr: a single problem passed inline in `one` (kernel
  // parameter space, read through a __grid_constant__ pointer), so a
  // single-problem launch needs no descriptor copy to the device.
  template <typename T>
  struct LaunchParams
  {
    ProblemDesc<T> one;
    const ProblemDesc<T>* probs;
    int n_probs;
    uint64_t total_items;
    unsigned long long* queue;   // zeroed before launch
    uint32_t lmax_c;             // max column length (shared-memory layout); time-windowed
                                 // variant: elements of a column slice
    uint32_t row_cap;            // per-warp row buffer capacity (elements)
    uint32_t win_r;              // time-windowed variant: elements of a row slice
    uint32_t row_slots;          // time-windowed variant: rows of an item with saved slice starts
  };

  // ---- item decoding ------------------------------------------------------

  __host__ __device__ inline uint64_t ceil_div_u64(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

  // Number of column groups of chunk c for the triangular modes.
  __host__ __device__ inline uint64_t tri_groups_of_chunk(uint64_t c, uint64_t rb, uint64_t re, uint64_t q, uint64_t G)
  {
    uint64_t hi = rb + (c + 1) * 32 * q;
    if (hi > re) hi = re;
    uint64_t ng = (hi - 1) / 32 + 1;
    return ng < G ? ng : G;
  }

  // Prefix P(c) = sum_{c' < c} ng(c') over whole chunks, where whole chunk c'
  // has ng(c') = min(G, B0 + (c'+1) q) groups (B0 = rb / 32).  For
  // c <= c1 = floor((G - B0) / q) every term is below the cap:
  //   P(c) = c B0 + q c (c + 1) / 2;  beyond c1 each chunk adds G.
  __host__ __device__ inline uint64_t tri_c1(uint64_t B0, uint64_t q, uint64_t G)
  {
    return G >= B0 ? (G - B0) / q : 0;
  }

  __host__ __device__ inline uint64_t tri_prefix(uint64_t c, uint64_t B0, uint64_t q, uint64_t G)
  {
    uint64_t c1 = tri_c1(B0, q, G);
    if (c <= c1) return c * B0 + q * c * (c + 1) / 2;
    return c1 * B0 + q * c1 * (c1 + 1) / 2 + (c - c1) * G;
  }

  __host__ __device__ inline uint64_t tri_item_count(uint64_t rb, uint64_t re, uint64_t q, uint64_t G)
  {
    if (re <= rb || G == 0) return 0;
    uint64_t C = ceil_div_u64(re - rb, 32 * q);
    return tri_prefix(C - 1, rb / 32, q, G) + tri_groups_of_chunk(C - 1, rb, re, q, G);
  }

  // id -> (chunk c, group g) for the triangular modes.
  __host__ __device__ inline void tri_decode(uint64_t id, uint64_t rb, uint64_t re, uint64_t q, uint64_t G,
                                             uint64_t* c_out, uint64_t* g_out)
  {
    uint64_t B0 = rb / 32;
    uint64_t C = ceil_div_u64(re - rb, 32 * q);
    uint64_t c1 = tri_c1(B0, q, G);
    uint64_t pc1 = tri_prefix(c1, B0, q, G);
    uint64_t c;
    if (id >= pc1) {
      c = c1 + (id - pc1) / G;
    } else {
      // largest c with c B0 + q c (c+1)/2 <= id, from the quadratic formula
      double a = 0.5 * (double)q, b = (double)B0 + 0.5 * (double)q;
      double cg = (-b + sqrt(b * b + 4.0 * a * (double)id)) / (2.0 * a);
      c = cg > 0 ? (uint64_t)cg : 0;
    }
    if (c > C - 1) c = C - 1;
    while (c > 0 && tri_prefix(c, B0, q, G) > id) --c;
    while (c + 1 < C && tri_prefix(c + 1, B0, q, G) <= id) ++c;
    *c_out = c;
    *g_out = id - tri_prefix(c, B0, q, G);
  }

  template <typename T>
  __host__ __device__ inline uint64_t problem_item_count(const ProblemDesc<T>& d)
  {
    uint64_t G = ceil_div_u64(d.nc, 32);
    if (d.row_end <= d.row_begin || G == 0) return 0;
    if (d.mode == MODE_CROSS) return ceil_div_u64(d.row_end - d.row_begin, 32ull * d.q) * G;
    return tri_item_count(d.row_begin, d.row_end, d.q, G);
  }

  __host__ __device__ inline uint64_t condensed_index(int mode, uint64_t i, uint64_t j)
  {
    uint64_t r = i > j ? i : j, c = i > j ? j : i;
    return mode == MODE_PDIST ? r * (r - 1) / 2 + c : r * (r + 1) / 2 + c;
  }
}
