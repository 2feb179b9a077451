/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C restatement of stablebear's CPU pairwise-integration path, used by
 * the tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, as
 * the parity reference and the CPU baseline.  Nothing in the product (stablebear_gb300/)
 * links, imports or calls this file.
 *
 * What it restates (paths relative to the stablebear source tree):
 *   - iterate_rectangles()      include/sbear/algorithms/functional/iterate_rectangles.hpp:37-104
 *   - max_time_iterator_prior_to() (the a = 0 start)  iterate_rectangles.hpp:23-35
 *   - integrate()               include/sbear/algorithms/functional/matrix_integrate.hpp:18-29
 *                               (naive in-order sum  val += (r - l) * op(f, g))
 *   - compute_row()             matrix_integrate.hpp:80-90  (j from i+1, or from i for the kernel)
 *   - CpuCrossIntegrationTask   matrix_integrate.hpp:132-143 (dense row-major cdist)
 *   - OperationL1Dist / OperationLpDist / OperationL2InnerProduct
 *                               include/sbear/functional/operations.cuh:19-65
 *   - DistanceMatrix / SymmetricMatrix storage order
 *                               include/sbear/distance_matrix.hpp:141-146,
 *                               include/sbear/symmetric_matrix.hpp:248-260
 *   - b = numeric_limits<T>::max() as the right end of the last rectangle
 *                               include/sbear/functional/time_point.hpp:10-14
 * taskflow's for_each_index over rows (matrix_integrate.hpp:69-75) is replaced
 * by a pthread pool that hands out rows through an atomic counter.
 *
 * A second, "truth" oracle accumulates the same rectangles in double-double
 * arithmetic (Dekker/Knuth TwoSum and an FMA-based TwoProd) and is used to
 * state the error of every implementation against near-exact sums.
 *
 * Build: see oracle/build_oracle.py (gcc -O2 -ffp-contract=off, so that the
 * same bits come out on x86-64 and aarch64).
 *
 * Point layout everywhere: interleaved (t, v) pairs, PCF i occupies points
 * [offsets[i], offsets[i+1]) — the reference's SimplePoint CSR
 * (include/sbear/cuda/offset_data_manager.hpp:42-68).
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SBO_OP_L1 0
#define SBO_OP_LP 1
#define SBO_OP_L2 2

/* ---------------------------------------------------------------------- */
/* Naive restatement, one instance per precision.                           */
/* ---------------------------------------------------------------------- */

#define SBO_DEFINE_NAIVE(T, SUF, ABS, POW, TMAX)                                          \
  static inline T sbo_op_##SUF(int op, T p, T f, T g)                                     \
  {                                                                                       \
    /* operations.cuh:19-65 */                                                            \
    if (op == SBO_OP_L1) return ABS(f - g);                                               \
    if (op == SBO_OP_LP) return POW(ABS(f - g), p);                                       \
    return f * g;                                                                         \
  }                                                                                       \
                                                                                          \
  T sbo_finalize_##SUF(int op, T p, T x)                                                  \
  {                                                                                       \
    if (op == SBO_OP_LP) return POW(x, (T)1 / p);                                         \
    return x;                                                                             \
  }                                                                                       \
                                                                                          \
  /* Index of the last point with t <= a, or 0 (iterate_rectangles.hpp:23-35). */         \
  static size_t sbo_prior_##SUF(const T* pts, uint64_t n, T a)                            \
  {                                                                                       \
    size_t lo = 0, hi = (size_t)n; /* upper_bound: first index with a < t */              \
    while (lo < hi) {                                                                     \
      size_t mid = lo + (hi - lo) / 2;                                                    \
      if (a < pts[2 * mid]) hi = mid; else lo = mid + 1;                                  \
    }                                                                                     \
    return lo == 0 ? 0 : lo - 1;                                                          \
  }                                                                                       \
                                                                                          \
  /* integrate() with a = 0, b = max (matrix_integrate.hpp:18-29). */                     \
  T sbo_integrate_##SUF(const T* f, uint64_t lf, const T* g, uint64_t lg, int op, T p)    \
  {                                                                                       \
    const T a = (T)0, b = TMAX;                                                           \
    size_t fi = sbo_prior_##SUF(f, lf, a);                                                \
    size_t gi = sbo_prior_##SUF(g, lg, a);                                                \
    T t = a, tprev = a, fv, gv, val = (T)0;                                               \
    while (t < b) {                                                                       \
      tprev = t;                                                                          \
      fv = f[2 * fi + 1];                                                                 \
      gv = g[2 * gi + 1];                                                                 \
      int fn = fi + 1 < lf, gn = gi + 1 < lg;                                             \
      if (fn && gn) {                                                                     \
        T delta = f[2 * (fi + 1)] - g[2 * (gi + 1)];                                      \
        if (delta <= 0) ++fi;                                                             \
        if (delta >= 0) ++gi;                                                             \
      } else if (fn) {                                                                    \
        ++fi;                                                                             \
      } else if (gn) {                                                                    \
        ++gi;                                                                             \
      } else {                                                                            \
        val += (b - tprev) * sbo_op_##SUF(op, p, fv, gv);                                 \
        return val;                                                                       \
      }                                                                                   \
      T hi_t = f[2 * fi] > g[2 * gi] ? f[2 * fi] : g[2 * gi];                             \
      t = hi_t < b ? hi_t : b;                                                            \
      val += (t - tprev) * sbo_op_##SUF(op, p, fv, gv);                                   \
    }                                                                                     \
    return val;                                                                           \
  }                                                                                       \
                                                                                          \
  /* Count of rectangles the merge emits (including the final one to b). */               \
  uint64_t sbo_count_segments_##SUF(const T* f, uint64_t lf, const T* g, uint64_t lg)     \
  {                                                                                       \
    size_t fi = 0, gi = 0;                                                                \
    uint64_t n = 0;                                                                       \
    for (;;) {                                                                            \
      int fn = fi + 1 < lf, gn = gi + 1 < lg;                                             \
      ++n;                                                                                \
      if (fn && gn) {                                                                     \
        T delta = f[2 * (fi + 1)] - g[2 * (gi + 1)];                                      \
        if (delta <= 0) ++fi;                                                             \
        if (delta >= 0) ++gi;                                                             \
      } else if (fn) ++fi;                                                                \
      else if (gn) ++gi;                                                                  \
      else return n;                                                                      \
    }                                                                                     \
  }

SBO_DEFINE_NAIVE(float, f32, fabsf, powf, FLT_MAX)
SBO_DEFINE_NAIVE(double, f64, fabs, pow, DBL_MAX)

/* ---------------------------------------------------------------------- */
/* Double-double "truth" accumulation of the same rectangles.              */
/* ---------------------------------------------------------------------- */

typedef struct { double hi, lo; } sbo_dd;

static inline sbo_dd dd_two_sum(double a, double b)
{
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  sbo_dd r = { s, e };
  return r;
}

static inline sbo_dd dd_add(sbo_dd x, sbo_dd y)
{
  sbo_dd s = dd_two_sum(x.hi, y.hi);
  sbo_dd t = dd_two_sum(x.lo, y.lo);
  s.lo += t.hi;
  s = dd_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return dd_two_sum(s.hi, s.lo);
}

static inline sbo_dd dd_from_diff(double a, double b) /* exact a - b */
{
  return dd_two_sum(a, -b);
}

static inline sbo_dd dd_mul(sbo_dd x, sbo_dd y)
{
  double p = x.hi * y.hi;
  double e = fma(x.hi, y.hi, -p);
  e += x.hi * y.lo + x.lo * y.hi;
  return dd_two_sum(p, e);
}

static inline sbo_dd dd_abs(sbo_dd x)
{
  if (x.hi < 0 || (x.hi == 0 && x.lo < 0)) { x.hi = -x.hi; x.lo = -x.lo; }
  return x;
}

/* op evaluated in double-double; Lp uses pow() on the rounded |f - g|. */
static inline sbo_dd dd_op(int op, double p, double f, double g)
{
  if (op == SBO_OP_L1) return dd_abs(dd_from_diff(f, g));
  if (op == SBO_OP_LP) {
    sbo_dd d = dd_abs(dd_from_diff(f, g));
    double base = d.hi + d.lo;
    double r = pow(base, p);
    sbo_dd out = { r, 0.0 };
    return out;
  }
  sbo_dd a = { f, 0.0 }, b = { g, 0.0 };
  return dd_mul(a, b);
}

/* Same rectangle walk as the naive restatement, but times/values widened to
 * double and the sum carried in double-double.  The right end of the last
 * rectangle is the *input* type's max, as in the reference. */
#define SBO_DEFINE_DD(T, SUF, TMAX)                                                       \
  double sbo_integrate_dd_##SUF(const T* f, uint64_t lf, const T* g, uint64_t lg,         \
                                int op, double p)                                         \
  {                                                                                       \
    const double b = (double)TMAX;                                                        \
    size_t fi = sbo_prior_##SUF(f, lf, (T)0);                                             \
    size_t gi = sbo_prior_##SUF(g, lg, (T)0);                                             \
    double t = 0.0, tprev = 0.0, fv, gv;                                                  \
    sbo_dd acc = { 0.0, 0.0 };                                                            \
    while (t < b) {                                                                       \
      tprev = t;                                                                          \
      fv = (double)f[2 * fi + 1];                                                         \
      gv = (double)g[2 * gi + 1];                                                         \
      int fn = fi + 1 < lf, gn = gi + 1 < lg;                                             \
      double right;                                                                       \
      int last = 0;                                                                       \
      if (fn && gn) {                                                                     \
        T delta = f[2 * (fi + 1)] - g[2 * (gi + 1)];                                      \
        if (delta <= 0) ++fi;                                                             \
        if (delta >= 0) ++gi;                                                             \
      } else if (fn) ++fi;                                                                \
      else if (gn) ++gi;                                                                  \
      else last = 1;                                                                      \
      if (last) right = b;                                                                \
      else {                                                                              \
        double hi_t = (double)(f[2 * fi] > g[2 * gi] ? f[2 * fi] : g[2 * gi]);            \
        right = hi_t < b ? hi_t : b;                                                      \
      }                                                                                   \
      sbo_dd w = dd_from_diff(right, tprev);                                              \
      acc = dd_add(acc, dd_mul(w, dd_op(op, p, fv, gv)));                                 \
      t = right;                                                                          \
      if (last) break;                                                                    \
    }                                                                                     \
    double s = acc.hi + acc.lo;                                                           \
    if (op == SBO_OP_LP) return pow(s, 1.0 / p);                                          \
    return s;                                                                             \
  }

SBO_DEFINE_DD(float, f32, FLT_MAX)
SBO_DEFINE_DD(double, f64, DBL_MAX)

/* ---------------------------------------------------------------------- */
/* Row-parallel drivers (the taskflow for_each_index substitute).          */
/* ---------------------------------------------------------------------- */

/* mode: 0 = cross (dense rows x cols), 1 = pdist (j < i, DistanceMatrix
 * order), 2 = kernel (j <= i, SymmetricMatrix order).  kind: 0 naive in the
 * input precision, 1 double-double truth (output always double). */
typedef struct {
  int dtype;             /* 0 = f32, 1 = f64 */
  int kind;
  int op;
  double p;
  int mode;
  const void* rpts; const uint64_t* roff; uint64_t nr;
  const void* cpts; const uint64_t* coff; uint64_t nc;
  const uint64_t* rows;  /* row list to evaluate (NULL = 0..nr-1) */
  uint64_t nrows;
  void* out;
  int compact;           /* 1: write each evaluated row's results back to back */
  const uint64_t* compact_base; /* per listed row: first output slot when compact */
  uint64_t chunk;        /* > 0: work items are pieces of at most `chunk` pairs of a row */
  const uint64_t* chunk_first; /* per listed row: its first work item (nrows + 1 entries) */
  uint64_t nitems;       /* work items handed out */
  _Atomic uint64_t next;
} sbo_job;

static inline uint64_t sbo_cond_index(int mode, uint64_t i, uint64_t j)
{
  uint64_t r = i > j ? i : j, c = i > j ? j : i;
  if (mode == 1) return r * (r - 1) / 2 + c; /* distance_matrix.hpp:141-146 */
  return r * (r + 1) / 2 + c;                /* symmetric_matrix.hpp:257-259 */
}

static uint64_t sbo_row_len(const sbo_job* job, uint64_t i)
{
  if (job->mode == 1) return i;
  if (job->mode == 2) return i + 1;
  return job->nc;
}

/* Pairs (i, j) of listed row k for j in [jlo, jhi). */
static void sbo_eval_range(sbo_job* job, uint64_t k, uint64_t jlo, uint64_t jhi)
{
  uint64_t i = job->rows ? job->rows[k] : k;
  const uint64_t jbeg = 0;
  for (uint64_t j = jlo; j < jhi; ++j) {
    uint64_t slot;
    if (job->compact) slot = job->compact_base[k] + (j - jbeg);
    else if (job->mode == 0) slot = i * job->nc + j;
    else slot = sbo_cond_index(job->mode, i, j);
    if (job->dtype == 0) {
      const float* fp = (const float*)job->rpts + 2 * job->roff[i];
      const float* gp = (const float*)job->cpts + 2 * job->coff[j];
      uint64_t lf = job->roff[i + 1] - job->roff[i], lg = job->coff[j + 1] - job->coff[j];
      if (job->kind == 0) {
        float v = sbo_integrate_f32(fp, lf, gp, lg, job->op, (float)job->p);
        ((float*)job->out)[slot] = sbo_finalize_f32(job->op, (float)job->p, v);
      } else {
        ((double*)job->out)[slot] = sbo_integrate_dd_f32(fp, lf, gp, lg, job->op, (double)(float)job->p);
      }
    } else {
      const double* fp = (const double*)job->rpts + 2 * job->roff[i];
      const double* gp = (const double*)job->cpts + 2 * job->coff[j];
      uint64_t lf = job->roff[i + 1] - job->roff[i], lg = job->coff[j + 1] - job->coff[j];
      if (job->kind == 0) {
        double v = sbo_integrate_f64(fp, lf, gp, lg, job->op, job->p);
        ((double*)job->out)[slot] = sbo_finalize_f64(job->op, job->p, v);
      } else {
        ((double*)job->out)[slot] = sbo_integrate_dd_f64(fp, lf, gp, lg, job->op, job->p);
      }
    }
  }
}

static void sbo_eval_item(sbo_job* job, uint64_t u)
{
  if (job->chunk == 0) {
    uint64_t i = job->rows ? job->rows[u] : u;
    sbo_eval_range(job, u, 0, sbo_row_len(job, i));
    return;
  }
  /* the listed row holding item u: last k with chunk_first[k] <= u */
  uint64_t lo = 0, hi = job->nrows - 1;
  while (lo < hi) {
    uint64_t mid = (lo + hi + 1) / 2;
    if (job->chunk_first[mid] <= u) lo = mid; else hi = mid - 1;
  }
  uint64_t i = job->rows ? job->rows[lo] : lo;
  uint64_t len = sbo_row_len(job, i);
  uint64_t jlo = (u - job->chunk_first[lo]) * job->chunk;
  uint64_t jhi = jlo + job->chunk < len ? jlo + job->chunk : len;
  sbo_eval_range(job, lo, jlo, jhi);
}

static void* sbo_worker(void* arg)
{
  sbo_job* job = (sbo_job*)arg;
  for (;;) {
    uint64_t u = atomic_fetch_add(&job->next, 1);
    if (u >= job->nitems) break;
    sbo_eval_item(job, u);
  }
  return NULL;
}

static int sbo_run(sbo_job* job, int nthreads)
{
  atomic_store(&job->next, 0);
  if (nthreads <= 1) { sbo_worker(job); return 0; }
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  if (!th) return -1;
  int started = 0;
  for (int t = 0; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, sbo_worker, job) != 0) break;
    ++started;
  }
  if (started == 0) sbo_worker(job);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  free(th);
  return 0;
}

/* Full pairwise / cross evaluation.  out: naive -> input type, truth -> double. */
int sbo_evaluate(int dtype, int kind, int op, double p, int mode,
                 const void* rpts, const uint64_t* roff, uint64_t nr,
                 const void* cpts, const uint64_t* coff, uint64_t nc,
                 void* out, int nthreads)
{
  sbo_job job;
  memset(&job, 0, sizeof(job));
  job.dtype = dtype; job.kind = kind; job.op = op; job.p = p; job.mode = mode;
  job.rpts = rpts; job.roff = roff; job.nr = nr;
  if (mode != 0) { cpts = rpts; coff = roff; nc = nr; }
  job.cpts = cpts; job.coff = coff; job.nc = nc;
  job.rows = NULL; job.nrows = nr; job.nitems = nr; job.out = out;
  return sbo_run(&job, nthreads);
}

/* Evaluate only the listed rows; results of row k are written back to back
 * starting at compact_base[k] (used for bounded CPU-baseline samples and for
 * sampled parity checks at full size). */
int sbo_evaluate_rows(int dtype, int kind, int op, double p, int mode,
                      const void* rpts, const uint64_t* roff, uint64_t nr,
                      const void* cpts, const uint64_t* coff, uint64_t nc,
                      const uint64_t* rows, uint64_t nrows, const uint64_t* compact_base,
                      void* out, int nthreads)
{
  sbo_job job;
  memset(&job, 0, sizeof(job));
  job.dtype = dtype; job.kind = kind; job.op = op; job.p = p; job.mode = mode;
  job.rpts = rpts; job.roff = roff; job.nr = nr;
  if (mode != 0) { cpts = rpts; coff = roff; nc = nr; }
  job.cpts = cpts; job.coff = coff; job.nc = nc;
  job.rows = rows; job.nrows = nrows; job.nitems = nrows; job.out = out;
  job.compact = 1; job.compact_base = compact_base;
  return sbo_run(&job, nthreads);
}

/* As sbo_evaluate_rows, with the threads taking pieces of at most `chunk`
 * pairs of a row instead of whole rows, so that a few long rows cannot leave
 * threads idle at the end (row i of a pdist has i pairs). */
int sbo_evaluate_rows_chunked(int dtype, int kind, int op, double p, int mode,
                              const void* rpts, const uint64_t* roff, uint64_t nr,
                              const void* cpts, const uint64_t* coff, uint64_t nc,
                              const uint64_t* rows, uint64_t nrows, const uint64_t* compact_base,
                              void* out, int nthreads, uint64_t chunk)
{
  if (chunk == 0 || nrows == 0)
    return sbo_evaluate_rows(dtype, kind, op, p, mode, rpts, roff, nr, cpts, coff, nc, rows, nrows, compact_base,
                             out, nthreads);
  sbo_job job;
  memset(&job, 0, sizeof(job));
  job.dtype = dtype; job.kind = kind; job.op = op; job.p = p; job.mode = mode;
  job.rpts = rpts; job.roff = roff; job.nr = nr;
  if (mode != 0) { cpts = rpts; coff = roff; nc = nr; }
  job.cpts = cpts; job.coff = coff; job.nc = nc;
  job.rows = rows; job.nrows = nrows; job.out = out;
  job.compact = 1; job.compact_base = compact_base;
  uint64_t* first = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(nrows + 1));
  if (!first) return -1;
  first[0] = 0;
  for (uint64_t k = 0; k < nrows; ++k) {
    uint64_t len = sbo_row_len(&job, rows[k]);
    first[k + 1] = first[k] + (len + chunk - 1) / chunk;
  }
  job.chunk = chunk; job.chunk_first = first; job.nitems = first[nrows];
  int rc = sbo_run(&job, nthreads);
  free(first);
  return rc;
}

/* Total merged rectangles (segments) of a pairwise/cross problem, the work
 * unit of the throughput metric.  Counted, not estimated. */
uint64_t sbo_count_total_segments(int dtype, int mode,
                                  const void* rpts, const uint64_t* roff, uint64_t nr,
                                  const void* cpts, const uint64_t* coff, uint64_t nc)
{
  if (mode != 0) { cpts = rpts; coff = roff; nc = nr; }
  uint64_t total = 0;
  for (uint64_t i = 0; i < nr; ++i) {
    uint64_t jend = mode == 0 ? nc : (mode == 1 ? i : i + 1);
    for (uint64_t j = 0; j < jend; ++j) {
      uint64_t lf = roff[i + 1] - roff[i], lg = coff[j + 1] - coff[j];
      if (dtype == 0)
        total += sbo_count_segments_f32((const float*)rpts + 2 * roff[i], lf, (const float*)cpts + 2 * coff[j], lg);
      else
        total += sbo_count_segments_f64((const double*)rpts + 2 * roff[i], lf, (const double*)cpts + 2 * coff[j], lg);
    }
  }
  return total;
}

/* ---------------------------------------------------------------------- */
/* FP64 reference gradient of  L = sum_pairs w_ij * M_ij  with respect to   */
/* every breakpoint's value and time, for M = L2 kernel (op 2) or L2        */
/* distance (op 1, p = 2).  The reference has no gradient; this is the      */
/* analytic derivative of the rectangle sum of integrate()                  */
/* (matrix_integrate.hpp:18-29), evaluated on the same rectangles:           */
/*   d/dv (value of a rectangle's side) = (r - l) * d phi / d side value     */
/*   d/dt_k (breakpoint k of one side, no tie) =                             */
/*          phi(value before t_k) - phi(value after t_k)                     */
/* with phi(f, g) = f g (kernel) or (f - g)^2 / (2 D) (distance, D the pair */
/* distance; D = 0 gives no gradient).  Breakpoints that coincide with one   */
/* of the other PCF (ties) get no time gradient.  Diagonal kernel entries:   */
/* d/dv_k = 2 v_k (t_{k+1} - t_k), d/dt_k = v_{k-1}^2 - v_k^2.               */
/* w: condensed weights in the output layout; grad: (M, 2) doubles           */
/* [t-grad, v-grad], accumulated.  Single-threaded (small problems).         */
/* ---------------------------------------------------------------------- */

static void sbo_grad_pair_f64(const double* f, uint64_t lf, double* gf, const double* g, uint64_t lg, double* gg,
                              int op, double w, double D, double bmax)
{
  if (w == 0.0) return;
  double scale = w;
  if (op == SBO_OP_LP) {
    if (!(D > 0.0)) return;
    scale = w / D;
  }
  size_t fi = 0, gi = 0;
  double t = 0.0;
  for (;;) {
    int fn = fi + 1 < lf, gn = gi + 1 < lg;
    double fv = f[2 * fi + 1], gv = g[2 * gi + 1];
    double right;
    int adv_f = 0, adv_g = 0;
    if (fn && gn) {
      double delta = f[2 * (fi + 1)] - g[2 * (gi + 1)];
      if (delta <= 0) adv_f = 1;
      if (delta >= 0) adv_g = 1;
    } else if (fn) adv_f = 1;
    else if (gn) adv_g = 1;
    if (!adv_f && !adv_g) right = bmax;
    else right = adv_f ? f[2 * (fi + 1)] : g[2 * (gi + 1)];
    double dt = right - t;
    /* value gradients of this rectangle */
    /* dt * coefficient first: the last rectangle's dt is the type's max and
       its coefficient usually 0 */
    if (op == SBO_OP_L2) {
      gf[2 * fi + 1] += scale * (dt * gv);
      gg[2 * gi + 1] += scale * (dt * fv);
    } else if (op == SBO_OP_L1) {
      double sg = fv > gv ? 1.0 : (fv < gv ? -1.0 : 0.0);
      gf[2 * fi + 1] += scale * (dt * sg);
      gg[2 * gi + 1] -= scale * (dt * sg);
    } else {
      gf[2 * fi + 1] += scale * (dt * (fv - gv));
      gg[2 * gi + 1] += scale * (dt * (gv - fv));
    }
    if (!adv_f && !adv_g) break;
    int tie = adv_f && adv_g;
    if (adv_f) ++fi;
    if (adv_g) ++gi;
    if (!tie) {
      if (adv_f) {
        double a = f[2 * (fi - 1) + 1], b = f[2 * fi + 1];
        double d = (op == SBO_OP_L2) ? (a - b) * gv
                 : (op == SBO_OP_L1) ? fabs(a - gv) - fabs(b - gv)
                 : 0.5 * ((a - gv) * (a - gv) - (b - gv) * (b - gv));
        gf[2 * fi] += scale * d;
      } else {
        double a = g[2 * (gi - 1) + 1], b = g[2 * gi + 1];
        double d = (op == SBO_OP_L2) ? (a - b) * fv
                 : (op == SBO_OP_L1) ? fabs(a - fv) - fabs(b - fv)
                 : 0.5 * ((a - fv) * (a - fv) - (b - fv) * (b - fv));
        gg[2 * gi] += scale * d;
      }
    }
    t = right;
  }
}

static void sbo_grad_diag_f64(const double* f, uint64_t lf, double* gf, double w, double bmax)
{
  if (w == 0.0) return;
  for (uint64_t k = 0; k < lf; ++k) {
    double right = (k + 1 < lf) ? f[2 * (k + 1)] : bmax;
    double v = f[2 * k + 1];
    gf[2 * k + 1] += w * (2.0 * (v * (right - f[2 * k])));
    if (k > 0) {
      double a = f[2 * (k - 1) + 1];
      gf[2 * k] += w * (a * a - v * v);
    }
  }
}

/* pts: (M,2) doubles; mode 1 (distance: op LP means p = 2, op L1 the L1
 * distance) or 2 (kernel, op L2). */
int sbo_gradient_f64(const double* pts, const uint64_t* off, uint64_t n, int op, int mode, const double* w,
                     const double* dist, double* grad, double bmax)
{
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t jend = (mode == 1) ? i : i + 1;
    for (uint64_t j = 0; j < jend; ++j) {
      uint64_t idx = sbo_cond_index(mode, i, j);
      const double* fp = pts + 2 * off[i];
      const double* gp = pts + 2 * off[j];
      uint64_t lf = off[i + 1] - off[i], lg = off[j + 1] - off[j];
      if (i == j) {
        sbo_grad_diag_f64(fp, lf, grad + 2 * off[i], w[idx], bmax);
      } else {
        sbo_grad_pair_f64(fp, lf, grad + 2 * off[i], gp, lg, grad + 2 * off[j], op, w[idx],
                          dist ? dist[idx] : 0.0, bmax);
      }
    }
  }
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Single-PCF Lp norms: l1_norm / lp_norm                                   */
/* (include/sbear/algorithms/functional/apply_functional.hpp:63-100) over   */
/* iterate_segments with a = 0, b = max (iterate_rectangles.hpp:106-155):   */
/* start at the last breakpoint with t <= a; segment [t_prev, min(t, b))    */
/* with the previous value; stop after a segment that reaches b; otherwise  */
/* a last segment [t_last, b).  Naive in-order sum; p == 1 uses |v|, any    */
/* other p pow(|v|, p) and a final pow(sum, 1/p).                           */
/* ---------------------------------------------------------------------- */

#define SBO_DEFINE_NORM(T, SUF, ABS, POW, TMAX)                                             \
  static T sbo_norm_one_##SUF(const T* f, uint64_t lf, T p)                                 \
  {                                                                                         \
    const T b = TMAX;                                                                       \
    uint64_t prev = 0;                                                                      \
    T out = (T)0;                                                                           \
    if (lf == 0) return (T)0;                                                               \
    while (prev + 1 < lf && f[2 * (prev + 1)] <= (T)0) ++prev;                              \
    T tprev = (T)0, vprev = f[2 * prev + 1];                                                \
    for (uint64_t k = prev + 1; k < lf; ++k) {                                              \
      T tnext = f[2 * k] < b ? f[2 * k] : b;                                                \
      out += (tnext - tprev) * (p == (T)1 ? ABS(vprev) : POW(ABS(vprev), p));               \
      if (tnext >= b) return p == (T)1 ? out : POW(out, (T)1 / p);                          \
      tprev = f[2 * k];                                                                     \
      vprev = f[2 * k + 1];                                                                 \
    }                                                                                       \
    out += (b - tprev) * (p == (T)1 ? ABS(vprev) : POW(ABS(vprev), p));                     \
    return p == (T)1 ? out : POW(out, (T)1 / p);                                            \
  }

SBO_DEFINE_NORM(float, f32, fabsf, powf, FLT_MAX)
SBO_DEFINE_NORM(double, f64, fabs, pow, DBL_MAX)

int sbo_lp_norm(int dtype, double p, const void* pts, const uint64_t* off, uint64_t n, void* out)
{
  for (uint64_t i = 0; i < n; ++i) {
    if (dtype == 0)
      ((float*)out)[i] = sbo_norm_one_f32((const float*)pts + 2 * off[i], off[i + 1] - off[i], (float)p);
    else
      ((double*)out)[i] = sbo_norm_one_f64((const double*)pts + 2 * off[i], off[i + 1] - off[i], p);
  }
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Barcodes to PCFs: the reference's loops, literally.                      */
/*   barcode_to_stable_rank  include/sbear/persistence/stable_rank.hpp:17-66 */
/*   barcode_to_betti_curve  include/sbear/persistence/betti_curve.hpp:21-84 */
/* is_infinite: +inf or max (persistence/barcode.hpp:18-21).  The sorts are */
/* qsort with the reference's orderings (lifetimes ascending; events by     */
/* time, births before deaths at equal times).                              */
/* ---------------------------------------------------------------------- */

#define SBO_DEFINE_SUMMARY(T, SUF, TMAX)                                                   \
  typedef struct { T time; int delta; } sbo_event_##SUF;                                   \
  static int sbo_cmp_t_##SUF(const void* a, const void* b)                                 \
  {                                                                                        \
    T x = *(const T*)a, y = *(const T*)b;                                                  \
    return (x < y) ? -1 : (y < x) ? 1 : 0;                                                 \
  }                                                                                        \
  static int sbo_cmp_ev_##SUF(const void* a, const void* b)                                \
  {                                                                                        \
    const sbo_event_##SUF* x = (const sbo_event_##SUF*)a;                                  \
    const sbo_event_##SUF* y = (const sbo_event_##SUF*)b;                                  \
    if (x->time < y->time || (x->time == y->time && x->delta > y->delta)) return -1;       \
    if (y->time < x->time || (x->time == y->time && y->delta > x->delta)) return 1;        \
    return 0;                                                                              \
  }                                                                                        \
  static int sbo_inf_##SUF(T v) { return v == (T)INFINITY || v == TMAX; }                  \
  /* writes (t, v) pairs at out, returns the count */                                      \
  static uint64_t sbo_stable_rank_one_##SUF(const T* bars, uint64_t m, T* out, T* tmp)     \
  {                                                                                        \
    uint64_t np = 0;                                                                       \
    if (m == 0) { out[0] = 0; out[1] = 0; return 1; }                                      \
    for (uint64_t k = 0; k < m; ++k) {                                                     \
      T birth = bars[2 * k], death = bars[2 * k + 1];                                      \
      tmp[k] = (death == TMAX) ? TMAX : death - birth;                                     \
    }                                                                                      \
    qsort(tmp, m, sizeof(T), sbo_cmp_t_##SUF);                                             \
    T nAlive = (T)m;                                                                       \
    out[2 * np] = 0; out[2 * np + 1] = nAlive; ++np;                                       \
    T last = tmp[0];                                                                       \
    for (uint64_t k = 0; k < m; ++k) {                                                     \
      if (sbo_inf_##SUF(last)) break;                                                      \
      if (tmp[k] != last) { out[2 * np] = last; out[2 * np + 1] = nAlive; ++np; last = tmp[k]; } \
      nAlive -= 1;                                                                         \
    }                                                                                      \
    if (!sbo_inf_##SUF(last)) { out[2 * np] = last; out[2 * np + 1] = nAlive; ++np; }      \
    return np;                                                                             \
  }                                                                                        \
  static uint64_t sbo_betti_one_##SUF(const T* bars, uint64_t m, T* out, sbo_event_##SUF* ev) \
  {                                                                                        \
    uint64_t ne = 0, np = 0;                                                               \
    if (m == 0) { out[0] = 0; out[1] = 0; return 1; }                                      \
    for (uint64_t k = 0; k < m; ++k) {                                                     \
      ev[ne].time = bars[2 * k]; ev[ne].delta = 1; ++ne;                                   \
      if (!sbo_inf_##SUF(bars[2 * k + 1])) { ev[ne].time = bars[2 * k + 1]; ev[ne].delta = -1; ++ne; } \
    }                                                                                      \
    qsort(ev, ne, sizeof(sbo_event_##SUF), sbo_cmp_ev_##SUF);                              \
    T count = 0, lastTime = 0;                                                             \
    for (uint64_t k = 0; k < ne; ++k) {                                                    \
      if (ev[k].time != lastTime) { out[2 * np] = lastTime; out[2 * np + 1] = count; ++np; lastTime = ev[k].time; } \
      count += (T)ev[k].delta;                                                             \
    }                                                                                      \
    out[2 * np] = lastTime; out[2 * np + 1] = count; ++np;                                 \
    return np;                                                                             \
  }

SBO_DEFINE_SUMMARY(float, f32, FLT_MAX)
SBO_DEFINE_SUMMARY(double, f64, DBL_MAX)

/* kind 0 stable rank, 1 Betti curve.  out has room for the bound (m + 1 or
 * 2 m + 1 points per barcode); out_off[n + 1] receives the PCF offsets. */
int sbo_barcodes_to_pcfs(int kind, int dtype, const void* bars, const uint64_t* boff, uint64_t n, void* out,
                         uint64_t* out_off)
{
  uint64_t mmax = 0;
  for (uint64_t i = 0; i < n; ++i) if (boff[i + 1] - boff[i] > mmax) mmax = boff[i + 1] - boff[i];
  void* tmp = malloc((2 * mmax + 1) * 16);
  if (!tmp) return -1;
  out_off[0] = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t m = boff[i + 1] - boff[i], np;
    if (dtype == 0) {
      const float* b = (const float*)bars + 2 * boff[i];
      float* o = (float*)out + 2 * out_off[i];
      np = kind == 0 ? sbo_stable_rank_one_f32(b, m, o, (float*)tmp) : sbo_betti_one_f32(b, m, o, (sbo_event_f32*)tmp);
    } else {
      const double* b = (const double*)bars + 2 * boff[i];
      double* o = (double*)out + 2 * out_off[i];
      np = kind == 0 ? sbo_stable_rank_one_f64(b, m, o, (double*)tmp) : sbo_betti_one_f64(b, m, o, (sbo_event_f64*)tmp);
    }
    out_off[i + 1] = out_off[i] + np;
  }
  free(tmp);
  return 0;
}
