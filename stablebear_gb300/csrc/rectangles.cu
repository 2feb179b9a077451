// The rectangles of one pair of PCFs: stablebear's iterate_rectangles
// (include/sbear/algorithms/functional/iterate_rectangles.hpp:37-104), as
// its Python binding returns them (src/python/functional/py_pcf.cpp:92-96).
//
// The reference walks both breakpoint lists from their last points at or
// before a, advancing the side whose next breakpoint comes first (both on a
// tie), and emits [previous t, next t) with the two values in force, the last
// rectangle running to b.  Here the walk is computed in parallel:
//   * an event is a breakpoint after a side's start point, keyed by (time,
//     rank among the points of the same PCF with that time); equal keys of f
//     and g are one event that advances both, which is how the walk pairs
//     ties, including repeated times (the r-th copy in f meets the r-th in g);
//   * an event's place in the walk is the number of distinct keys below it:
//     its index in its own list, plus the other list's keys below it (binary
//     search), minus the matched pairs below it (a prefix count of matches);
//   * after event k the walk stands at event k's time (the side that did not
//     move is at a time no later), with f and g at the points the event and
//     the search name;
//   * rectangle k spans event k-1 (or a) to event k (or b), clipped to b, and
//     exists while its left end is below b.
// Times are assumed sorted within a PCF (the PCF contract); unsorted input
// gives some rectangles but never an out-of-range access.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

namespace sbg
{
  namespace
  {
    template <typename T> struct Pt { T t, v; };
    template <typename T> struct Event { T t; uint64_t fi, gi; };

    // index of the first point of p whose time equals p[i].t
    template <typename T>
    __device__ uint64_t first_equal(const Pt<T>* p, uint64_t i)
    {
      uint64_t lo = 0, hi = i;
      const T t = p[i].t;
      while (lo < hi)
      {
        const uint64_t mid = (lo + hi) >> 1;
        if (p[mid].t < t) lo = mid + 1; else hi = mid;
      }
      return lo;
    }

    // number of points j in [lo, n) of p whose key (time, rank) is below (t, r)
    template <typename T>
    __device__ uint64_t keys_below(const Pt<T>* p, uint64_t lo, uint64_t n, T t, uint64_t r)
    {
      uint64_t L = lo, H = n;
      while (L < H)
      {
        const uint64_t mid = (L + H) >> 1;
        const T tm = p[mid].t;
        const bool below = tm < t || (tm == t && mid - first_equal(p, mid) < r);
        if (below) L = mid + 1; else H = mid;
      }
      return L - lo;
    }

    template <typename T>
    __device__ bool key_at(const Pt<T>* p, uint64_t j, uint64_t n, T t, uint64_t r)
    {
      return j < n && p[j].t == t && j - first_equal(p, j) == r;
    }

    // Per candidate event: the other side's keys below it and whether the
    // other side holds the same key.  Candidates are f[fs+1..nf) then g[gs+1..ng).
    template <typename T>
    __global__ void rank_kernel(const Pt<T>* f, uint64_t nf, uint64_t fs, const Pt<T>* g, uint64_t ng, uint64_t gs,
                                uint64_t* below, uint32_t* match)
    {
      const uint64_t ef = nf - fs - 1, eg = ng - gs - 1;
      for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < ef + eg;
           k += (uint64_t)gridDim.x * blockDim.x)
      {
        const bool from_f = k < ef;
        const Pt<T>* p = from_f ? f : g;
        const Pt<T>* o = from_f ? g : f;
        const uint64_t i = from_f ? fs + 1 + k : gs + 1 + (k - ef);
        const uint64_t olo = from_f ? gs + 1 : fs + 1, on = from_f ? ng : nf;
        const uint64_t r = i - first_equal(p, i);
        const uint64_t c = keys_below(o, olo, on, p[i].t, r);
        below[k] = c;
        match[k] = key_at(o, olo + c, on, p[i].t, r) ? 1u : 0u;
      }
    }

    // Exclusive prefix sums of the match flags, separately over the f and the
    // g candidates (one CTA, chunk by chunk); the number of matched pairs in
    // *pairs.
    __global__ void match_scan_kernel(const uint32_t* match, uint64_t ef, uint64_t eg, uint32_t* prefix,
                                      uint64_t* pairs)
    {
      __shared__ uint32_t s[1024];
      __shared__ uint32_t carry;
      for (int side = 0; side < 2; ++side)
      {
        const uint64_t off = side == 0 ? 0 : ef, n = side == 0 ? ef : eg;
        if (threadIdx.x == 0) carry = 0;
        __syncthreads();
        for (uint64_t base = 0; base < n; base += blockDim.x)
        {
          const uint64_t i = base + threadIdx.x;
          const uint32_t x = i < n ? match[off + i] : 0u;
          s[threadIdx.x] = x;
          __syncthreads();
          for (unsigned d = 1; d < blockDim.x; d <<= 1)
          {
            const uint32_t y = threadIdx.x >= d ? s[threadIdx.x - d] : 0u;
            __syncthreads();
            s[threadIdx.x] += y;
            __syncthreads();
          }
          if (i < n) prefix[off + i] = carry + s[threadIdx.x] - x;
          __syncthreads();
          if (threadIdx.x == blockDim.x - 1) carry += s[threadIdx.x];
          __syncthreads();
        }
        if (threadIdx.x == 0 && side == 0) *pairs = carry;
        __syncthreads();
      }
    }

    // Events in walk order; a matched g candidate is the same event as its f
    // partner and writes nothing.
    template <typename T>
    __global__ void event_kernel(const Pt<T>* f, uint64_t nf, uint64_t fs, const Pt<T>* g, uint64_t ng, uint64_t gs,
                                 const uint64_t* below, const uint32_t* match, const uint32_t* prefix, Event<T>* ev,
                                 uint64_t n_events)
    {
      const uint64_t ef = nf - fs - 1, eg = ng - gs - 1;
      for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < ef + eg;
           k += (uint64_t)gridDim.x * blockDim.x)
      {
        const bool from_f = k < ef;
        const uint64_t kk = from_f ? k : k - ef;
        if (!from_f && match[k]) continue;
        const uint64_t c = below[k];
        const uint64_t pos = kk + c - prefix[k];
        if (pos >= n_events) continue;  // never expected: the counts are consistent
        Event<T> e;
        if (from_f)
        {
          e.fi = fs + 1 + kk;
          e.gi = match[k] ? gs + 1 + c : gs + c;
          e.t = f[e.fi].t;
        }
        else
        {
          e.gi = gs + 1 + kk;
          e.fi = fs + c;
          e.t = g[e.gi].t;
        }
        ev[pos] = e;
      }
    }

    // Rectangle k: [event k-1 or a, event k or b) clipped to b, with the
    // values in force after event k-1 (at the start points for k = 0).
    template <typename T>
    __global__ void rect_kernel(const Pt<T>* f, uint64_t fs, const Pt<T>* g, uint64_t gs, const Event<T>* ev,
                                uint64_t n_events, uint64_t n_rects, T a, T b, T* out)
    {
      for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n_rects;
           k += (uint64_t)gridDim.x * blockDim.x)
      {
        const T left = k == 0 ? a : ev[k - 1].t;
        const T right = k < n_events ? (ev[k].t < b ? ev[k].t : b) : b;
        const uint64_t fi = k == 0 ? fs : ev[k - 1].fi;
        const uint64_t gi = k == 0 ? gs : ev[k - 1].gi;
        out[4 * k + 0] = left;
        out[4 * k + 1] = right;
        out[4 * k + 2] = f[fi].v;
        out[4 * k + 3] = g[gi].v;
      }
    }

    // first event whose time is at or after b (events are in time order)
    template <typename T>
    __global__ void cut_kernel(const Event<T>* ev, uint64_t n_events, T b, uint64_t* cut)
    {
      if (threadIdx.x != 0 || blockIdx.x != 0) return;
      uint64_t lo = 0, hi = n_events;
      while (lo < hi)
      {
        const uint64_t mid = (lo + hi) >> 1;
        if (ev[mid].t < b) lo = mid + 1; else hi = mid;
      }
      *cut = lo;
    }

    struct DevMem
    {
      DeviceBuffer buf;
      void* p;
      explicit DevMem(size_t bytes) : buf(bytes), p(buf.get()) { }
      template <typename U> U* as() const { return buf.as<U>(); }
    };

    template <typename T>
    T to_time(double x)
    {
      if (std::numeric_limits<T>::is_integer)
      {
        if (std::isnan(x)) throw Error(ST_INVALID_ARGUMENT, "integration bounds must not be NaN");
        if (x >= (double)std::numeric_limits<T>::max()) return std::numeric_limits<T>::max();
        if (x <= (double)std::numeric_limits<T>::lowest()) return std::numeric_limits<T>::lowest();
        return (T)x;
      }
      return (T)x;
    }

    template <typename T>
    uint64_t start_point(const T* pts, uint64_t n, T a)
    {
      // max_time_iterator_prior_to: the last point with t <= a, else the first
      uint64_t lo = 0, hi = n;
      while (lo < hi)
      {
        const uint64_t mid = (lo + hi) / 2;
        if (!(a < pts[2 * mid])) lo = mid + 1; else hi = mid;
      }
      return lo == 0 ? 0 : lo - 1;
    }

    template <typename T>
    uint64_t rectangles(const T* fp, uint64_t nf, const T* gp, uint64_t ng, double a_, double b_, T* out, uint64_t cap)
    {
      if (nf == 0 || ng == 0) throw Error(ST_INVALID_ARGUMENT, "a PCF needs at least one breakpoint");
      const T a = to_time<T>(a_), b = to_time<T>(b_);
      const uint64_t fs = start_point(fp, nf, a), gs = start_point(gp, ng, a);
      const uint64_t ef = nf - fs - 1, eg = ng - gs - 1, ne = ef + eg;
      DevMem df(nf * sizeof(Pt<T>)), dg(ng * sizeof(Pt<T>));
      SBG_CUDA(cudaMemcpy(df.p, fp, nf * sizeof(Pt<T>), cudaMemcpyHostToDevice));
      SBG_CUDA(cudaMemcpy(dg.p, gp, ng * sizeof(Pt<T>), cudaMemcpyHostToDevice));
      DevMem below(std::max<uint64_t>(ne, 1) * sizeof(uint64_t)), match(std::max<uint64_t>(ne, 1) * sizeof(uint32_t)),
          prefix(std::max<uint64_t>(ne, 1) * sizeof(uint32_t)), scal(2 * sizeof(uint64_t)),
          ev(std::max<uint64_t>(ne, 1) * sizeof(Event<T>));
      const int sms = device_info().sms;
      const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((ne + 255) / 256, (uint64_t)sms * 4));
      uint64_t pairs = 0;
      if (ne)
      {
        rank_kernel<T><<<grid, 256>>>(df.as<Pt<T>>(), nf, fs, dg.as<Pt<T>>(), ng, gs, below.as<uint64_t>(),
                                      match.as<uint32_t>());
        SBG_CUDA(launched());
        match_scan_kernel<<<1, 1024>>>(match.as<uint32_t>(), ef, eg, prefix.as<uint32_t>(), scal.as<uint64_t>());
        SBG_CUDA(launched());
        SBG_CUDA(cudaMemcpy(&pairs, scal.p, sizeof(uint64_t), cudaMemcpyDeviceToHost));
      }
      const uint64_t n_events = ne - pairs;
      uint64_t cut = n_events;
      if (n_events)
      {
        event_kernel<T><<<grid, 256>>>(df.as<Pt<T>>(), nf, fs, dg.as<Pt<T>>(), ng, gs, below.as<uint64_t>(),
                                       match.as<uint32_t>(), prefix.as<uint32_t>(), ev.as<Event<T>>(), n_events);
        SBG_CUDA(launched());
        cut_kernel<T><<<1, 32>>>(ev.as<Event<T>>(), n_events, b, scal.as<uint64_t>() + 1);
        SBG_CUDA(launched());
        SBG_CUDA(cudaMemcpy(&cut, scal.as<uint64_t>() + 1, sizeof(uint64_t), cudaMemcpyDeviceToHost));
      }
      // the walk runs while its time is below b
      const uint64_t n_rects = (a < b) ? std::min(cut, n_events) + 1 : 0;
      const uint64_t n_out = std::min(n_rects, cap);
      if (n_out)
      {
        DevMem dr(n_out * 4 * sizeof(T));
        const unsigned rg = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n_out + 255) / 256, (uint64_t)sms * 4));
        rect_kernel<T><<<rg, 256>>>(df.as<Pt<T>>(), fs, dg.as<Pt<T>>(), gs, ev.as<Event<T>>(), n_events, n_out, a, b,
                                    dr.as<T>());
        SBG_CUDA(launched());
        SBG_CUDA(cudaMemcpy(out, dr.p, n_out * 4 * sizeof(T), cudaMemcpyDeviceToHost));
      }
      return n_rects;
    }
  }
}

extern "C" int sbg_iterate_rectangles(int dtype, const void* f_points, uint64_t nf, const void* g_points, uint64_t ng,
                                      double a, double b, void* out, uint64_t cap, uint64_t* count)
{
  using namespace sbg;
  try
  {
    if (!count) throw Error(ST_INVALID_ARGUMENT, "count must not be null");
    if ((nf && !f_points) || (ng && !g_points) || (cap && !out)) throw Error(ST_INVALID_ARGUMENT, "null pointer");
    uint64_t n = 0;
    switch (dtype)
    {
      case SBG_F32: n = rectangles<float>((const float*)f_points, nf, (const float*)g_points, ng, a, b, (float*)out, cap); break;
      case SBG_F64: n = rectangles<double>((const double*)f_points, nf, (const double*)g_points, ng, a, b, (double*)out, cap); break;
      case SBG_I32: n = rectangles<int32_t>((const int32_t*)f_points, nf, (const int32_t*)g_points, ng, a, b, (int32_t*)out, cap); break;
      case SBG_I64: n = rectangles<int64_t>((const int64_t*)f_points, nf, (const int64_t*)g_points, ng, a, b, (int64_t*)out, cap); break;
      default: throw Error(ST_INVALID_ARGUMENT, "dtype must be SBG_F32, SBG_F64, SBG_I32 or SBG_I64");
    }
    *count = n;
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
