// Host engine: planning, device buffers, the band pipeline and the
// stream-ordered device entry.  Replaces the reference's CudaBlockPipeline /
// PcfBlockOp / CudaOffsetDataManager stack
// (include/sbear/cuda/cuda_block_executor.cuh:108-341, pcf_block_op.cuh:32-123,
// cuda_offset_data_manager.cuh:24-44) with a GB300-first design:
//   * the whole CSR is uploaded once (no per-tile re-uploads);
//   * the kernel writes the condensed (or dense) result directly, so a band
//     of rows [rb, re) is one contiguous output range that is copied with a
//     single cudaMemcpyAsync straight into the caller's matrix — there is no
//     dense tile, no memset, no host scatter;
//   * bands alternate between two device buffers so the copy of band b
//     overlaps the kernel of band b + 1.
#include "sbg_internal.hpp"
#include "host_copy.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>

namespace sbg
{
  // ---- errors & settings ----------------------------------------------------

  static thread_local std::string t_last_error;

  void set_last_error(const std::string& msg) { t_last_error = msg; }
  const char* last_error() { return t_last_error.c_str(); }

  void throw_cuda(cudaError_t e, const char* file, int line)
  {
    const char* base = file;
    for (const char* p = file; *p; ++p)
      if (*p == '/') base = p + 1;
    std::string msg = std::string(base) + ":" + std::to_string(line) + ": " + cudaGetErrorString(e);
    int st = (e == cudaErrorMemoryAllocation) ? ST_OUT_OF_MEMORY
           : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? ST_NO_DEVICE : ST_CUDA;
    cudaGetLastError();  // clear a sticky-free error so later calls start clean
    throw Error(st, msg);
  }

  static std::atomic<uint64_t> g_kernel_launches{0};

  cudaError_t launched()
  {
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
  }

  void count_launches(uint64_t n) { g_kernel_launches.fetch_add(n, std::memory_order_relaxed); }
  void uncount_launches(uint64_t n) { g_kernel_launches.fetch_sub(n, std::memory_order_relaxed); }

  uint64_t kernel_launches() { return g_kernel_launches.load(std::memory_order_relaxed); }

  Settings& settings()
  {
    static Settings s;
    return s;
  }

  // ---- device allocations ----------------------------------------------------

  static std::atomic<uint64_t> g_alloc_limit{~0ull};
  static std::atomic<uint64_t> g_alloc_held{0};
  static std::atomic<uint64_t> g_alloc_count{0};

  static void reserve_bytes(size_t bytes)
  {
    const uint64_t held = g_alloc_held.fetch_add(bytes, std::memory_order_relaxed) + bytes;
    const uint64_t limit = g_alloc_limit.load(std::memory_order_relaxed);
    if (held > limit || held < bytes)
    {
      g_alloc_held.fetch_sub(bytes, std::memory_order_relaxed);
      throw Error(ST_OUT_OF_MEMORY, "device allocation of " + std::to_string(bytes) + " bytes refused: " +
                                        std::to_string(held - bytes) + " bytes held, limit " +
                                        std::to_string(limit) + " (sbg_set_alloc_limit)");
    }
  }

  void* device_malloc(size_t bytes)
  {
    reserve_bytes(bytes);
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess)
    {
      g_alloc_held.fetch_sub(bytes, std::memory_order_relaxed);
      throw_cuda(e, __FILE__, __LINE__);
    }
    g_alloc_count.fetch_add(1, std::memory_order_relaxed);
    return p;
  }

  void device_free(void* p, size_t bytes) noexcept
  {
    if (!p) return;
    cudaFree(p);
    g_alloc_held.fetch_sub(bytes, std::memory_order_relaxed);
  }

  void* device_malloc_async(size_t bytes, cudaStream_t st)
  {
    reserve_bytes(bytes);
    void* p = nullptr;
    const cudaError_t e = cudaMallocAsync(&p, bytes, st);
    if (e != cudaSuccess)
    {
      g_alloc_held.fetch_sub(bytes, std::memory_order_relaxed);
      throw_cuda(e, __FILE__, __LINE__);
    }
    g_alloc_count.fetch_add(1, std::memory_order_relaxed);
    return p;
  }

  void device_free_async(void* p, size_t bytes, cudaStream_t st) noexcept
  {
    if (!p) return;
    cudaFreeAsync(p, st);
    g_alloc_held.fetch_sub(bytes, std::memory_order_relaxed);
  }

  void set_alloc_limit(uint64_t bytes) { g_alloc_limit.store(bytes, std::memory_order_relaxed); }
  uint64_t device_allocations() { return g_alloc_count.load(std::memory_order_relaxed); }
  uint64_t device_bytes_held() { return g_alloc_held.load(std::memory_order_relaxed); }

  void DeviceBuffer::reset(size_t bytes)
  {
    release();
    if (bytes)
    {
      m_ptr = device_malloc(bytes);
      m_bytes = bytes;
    }
  }

  void DeviceBuffer::release()
  {
    if (m_ptr)
    {
      device_free(m_ptr, m_bytes);
      m_ptr = nullptr;
      m_bytes = 0;
    }
  }

  DeviceInfo device_info()
  {
    static std::mutex mu;
    static std::map<int, DeviceInfo> cache;
    int dev = 0;
    SBG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    DeviceInfo d;
    d.device = dev;
    SBG_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
    int optin = 0;
    SBG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    d.smem_optin = (size_t)optin;
    int per_sm = 0, threads = 0;
    SBG_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    SBG_CUDA(cudaDeviceGetAttribute(&threads, cudaDevAttrMaxThreadsPerMultiProcessor, dev));
    d.smem_per_sm = (size_t)per_sm;
    d.threads_per_sm = threads;
    cache[dev] = d;
    return d;
  }

  int ctas_per_sm(const DeviceInfo& dev, int warps, size_t smem_bytes)
  {
    const int threads = std::max(1, warps) * 32;
    int n = std::max(1, dev.threads_per_sm / threads);
    n = std::min(n, std::max(1, 65536 / (threads * 64)));  // the register file at 64 per thread
    const size_t per = smem_bytes + 1024;
    if (smem_bytes > 0 && dev.smem_per_sm > 0) n = std::min<int>(n, std::max<size_t>(1, dev.smem_per_sm / per));
    return n;
  }

  // ---- input contract ------------------------------------------------------

  template <typename T>
  void validate_pcfs(const PcfSet<T>& s, const char* what)
  {
    if (s.n == 0) return;
    if (!s.off || !s.pts) throw Error(ST_INVALID_ARGUMENT, std::string(what) + ": null points/offsets");
    if (s.off[0] != 0) throw Error(ST_INVALID_INPUT, std::string(what) + ": offsets must start at 0");
    // PCFs [i0, i1): the first invalid one, or i1; its error in *msg.
    auto check = [&s, what](uint64_t i0, uint64_t i1, std::string* msg) -> uint64_t {
      for (uint64_t i = i0; i < i1; ++i)
      {
        const uint64_t a = s.off[i], b = s.off[i + 1];
        if (b <= a) { *msg = std::string(what) + ": PCF " + std::to_string(i) + " has no breakpoints"; return i; }
        if (b - a > 0xffffffffull) { *msg = std::string(what) + ": PCF " + std::to_string(i) + " is too long"; return i; }
        const T* p = s.pts + 2 * a;
        if (p[0] != T(0))
        {
          *msg = std::string(what) + ": PCF " + std::to_string(i) +
                 ": the first breakpoint must have time t=0 (got t=" + std::to_string((double)p[0]) + ").";
          return i;
        }
        for (uint64_t k = 0; k < b - a; ++k)
        {
          const T t = p[2 * k];
          if (!std::isfinite(t))
          {
            *msg = std::string(what) + ": PCF " + std::to_string(i) + ": breakpoint times must be finite";
            return i;
          }
          if (k > 0 && !(p[2 * (k - 1)] <= t))
          {
            *msg = std::string(what) + ": PCF " + std::to_string(i) + ": Breakpoints must be given in non-decreasing time order.";
            return i;
          }
        }
      }
      return i1;
    };
    // Large inputs are checked in parallel over contiguous ranges of PCFs;
    // the error reported is the first invalid PCF's, as in a serial scan.
    const unsigned parts = s.off[s.n] >= (1ull << 20) && s.n >= 1024 ? host_parts() : 1u;
    if (parts <= 1)
    {
      std::string msg;
      if (check(0, s.n, &msg) < s.n) throw Error(ST_INVALID_INPUT, msg);
      return;
    }
    std::vector<uint64_t> bad(parts, ~0ull);
    std::vector<std::string> msgs(parts);
    host_parallel([&](unsigned k) {
      const uint64_t i0 = s.n * k / parts, i1 = s.n * (k + 1) / parts;
      const uint64_t r = check(i0, i1, &msgs[k]);
      if (r < i1) bad[k] = r;
    });
    for (unsigned k = 0; k < parts; ++k)
      if (bad[k] != ~0ull) throw Error(ST_INVALID_INPUT, msgs[k]);
  }

  template void validate_pcfs<float>(const PcfSet<float>&, const char*);
  template void validate_pcfs<double>(const PcfSet<double>&, const char*);

  // ---- planning ---------------------------------------------------------------

  int op_kind(int op, double p)
  {
    if (op == 0) return OPK_L1;
    if (op == 1)
    {
      if (p == 1.0) return OPK_L1;
      if (p == 2.0) return OPK_L2DIST;
      return OPK_LP;
    }
    if (op == 2) return OPK_INNER;
    throw Error(ST_INVALID_ARGUMENT, "unknown op " + std::to_string(op));
  }

  uint64_t output_count(int mode, uint64_t nr, uint64_t nc)
  {
    if (mode == MODE_PDIST) return nr == 0 ? 0 : nr * (nr - 1) / 2;
    if (mode == MODE_KERNEL) return nr * (nr + 1) / 2;
    return nr * nc;
  }

  uint64_t row_output_start(int mode, uint64_t r, uint64_t nc)
  {
    if (mode == MODE_PDIST) return r == 0 ? 0 : r * (r - 1) / 2;
    if (mode == MODE_KERNEL) return r * (r + 1) / 2;
    return r * nc;
  }

  static uint64_t items_for(int mode, uint64_t rb, uint64_t re, uint64_t nc, uint32_t q)
  {
    ProblemDesc<float> d{};
    d.mode = mode; d.nc = nc; d.row_begin = rb; d.row_end = re; d.q = q;
    return problem_item_count(d);
  }

  // ---- launch-shape cache (sbg_autotune_device) ---------------------------------

  static std::mutex g_tune_mu;
  static std::map<TuneKey, std::pair<int, int>> g_tune_cache;

  static int floor_log2(uint64_t x)
  {
    int r = -1;
    while (x) { x >>= 1; ++r; }
    return r;
  }

  TuneKey tune_key(int elem_bytes, int opk, int mode, uint64_t n, uint32_t lmax)
  {
    return TuneKey{elem_bytes, opk, mode, floor_log2(n), floor_log2(lmax)};
  }

  bool tune_cache_get(const TuneKey& k, int* warps, int* q)
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(k);
    if (it == g_tune_cache.end()) return false;
    *warps = it->second.first;
    *q = it->second.second;
    return true;
  }

  void tune_cache_put(const TuneKey& k, int warps, int q)
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[k] = {warps, q};
  }

  void tune_cache_clear()
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache.clear();
  }

  template <typename T>
  Plan make_plan(int mode, uint64_t nr, uint64_t nc, const LengthStats& rs, const LengthStats& cs, const DeviceInfo& dev,
                 int opk)
  {
    Plan pl;
    const int U = kernel_unroll(sizeof(T) == 8);
    const size_t es = sizeof(Elem<T>);
    const size_t reserve = 2048;  // static shared memory + slack
    const size_t usable = dev.smem_optin > reserve ? dev.smem_optin - reserve : 0;
    const uint32_t lmax_c = std::max<uint32_t>(cs.lmax, 1);
    const uint32_t lmax_r = std::max<uint32_t>(rs.lmax, 1);
    const int variant = settings().variant.load();
    // Row buffer: the row, then sentinel copies for the advances past its
    // end.  The default walk (variant 5) pulls the row address back every
    // block, so U copies do; the others need one per step of the longest
    // column.
#ifndef SBG_ROW_PAD_FULL
    const bool short_pad = variant == 0 || variant == 5;
#else
    const bool short_pad = false;
#endif
    const uint32_t row_cap_full = lmax_r + lmax_c + (uint32_t)U + 1;
    const uint32_t row_cap = short_pad ? lmax_r + (uint32_t)U + 1 : row_cap_full;
    auto smem_for = [&](int w) { return (size_t)32 * lmax_c * es + (size_t)w * row_cap * es; };

    const int want_w = settings().warps.load();
    // Shared-memory variants (rows and columns staged): the most warps that fit.
    auto most_warps = [&](uint32_t cap) {
      const int cands[] = {32, 24, 16, 12, 8, 4};
      for (int w : cands)
      {
        if (want_w > 0 && w > want_w) continue;
        if ((size_t)32 * lmax_c * es + (size_t)w * cap * es <= usable) return w;
      }
      return 0;
    };
    int warps = 0;
    if (variant == 0 || variant == 1 || variant == 3 || variant == 5) warps = most_warps(row_cap);
    if ((variant == 1 || variant == 3 || variant == 5) && warps == 0)
      throw Error(ST_INVALID_ARGUMENT, "shared-memory variant requested but the PCFs do not fit in shared memory");
    // The automatic choice between this kernel and the time-windowed one is
    // made on the layout with full row padding (at least 16 warps): with the
    // short padding, L ~ U{16..512} also fits 16 warps, but there (N = 4096)
    // the plain kernel measured 2.89 / 2.95 ms against 2.86 / 2.88 ms for the
    // windowed one (L2 kernel / L2 distance).
    const bool plain_auto = variant == 0 && most_warps(row_cap_full) >= 16;

    if (plain_auto || variant == 1 || variant == 3 || variant == 5)
    {
      pl.smem = true;
      pl.packed = false;
      pl.kvar = variant == 3 ? 1 : (variant == 1 ? 2 : 5);  // auto: row times and values apart
      pl.warps = warps;
      pl.lmax_c = lmax_c;
      pl.row_cap = row_cap;
      pl.smem_bytes = smem_for(warps);
    }
    else if (variant == 7 || variant == 8)
    {
      // the float32 measurement variants (pair_variants.cu); never automatic
      if (sizeof(T) != 4) throw Error(ST_INVALID_ARGUMENT, "variants 7 and 8 are float32 only");
      pl.smem = true;
      pl.packed = false;
      pl.kvar = variant;
      size_t fixed, per_warp;
      if (variant == 7)
      {
        pl.lmax_c = lmax_c;
        pl.row_cap = lmax_r + (uint32_t)U;                   // the row, then U sentinel elements
        fixed = (size_t)32 * lmax_c * es;                     // 32 columns, 8 bytes per element
        per_warp = (size_t)pl.row_cap * 16 * es;              // 16 copies of every row element
      }
      else
      {
        pl.lmax_c = (uint32_t)padded_words((int)lmax_c - 1) + 1;  // padded column stride (words)
        pl.row_cap = (uint32_t)padded_words((int)lmax_r - 1) + 1;
        fixed = (size_t)2 * 32 * pl.lmax_c * sizeof(T);
        per_warp = (size_t)2 * pl.row_cap * sizeof(T);
      }
      int w = 0;
      for (int cand : {32, 24, 20, 16, 12, 8, 4})
      {
        if (want_w > 0 && cand > want_w) continue;
        if (fixed + (size_t)cand * per_warp <= usable) { w = cand; break; }
      }
      if (w == 0) throw Error(ST_INVALID_ARGUMENT, "variant " + std::to_string(variant) +
                                                       ": the PCFs do not fit in shared memory");
      pl.warps = w;
      pl.smem_bytes = fixed + (size_t)w * per_warp;
    }
    else if (variant == 2)
    {
      pl.smem = false;
      pl.packed = true;
      pl.kvar = 0;
      pl.warps = want_w > 0 ? std::min(want_w, 32) : 16;
      pl.lmax_c = lmax_c;
      pl.row_cap = 0;
      pl.smem_bytes = 0;
    }
    else if (variant == 4 || (variant == 0 && sizeof(T) == 8))
    {
      // hybrid: columns staged when the group fits, rows through L1 (the
      // automatic choice for long double PCFs, where the FP64 pipe bounds
      // both and the time-windowed walk measured slower)
      pl.smem = true;
      pl.packed = true;
      pl.kvar = 3;
      pl.warps = want_w > 0 ? std::min(want_w, 32) : 32;
      const uint32_t cap = (uint32_t)std::min<size_t>(usable / (32 * es), 0xffffffffu);
      pl.lmax_c = std::min(lmax_c, cap);
      pl.row_cap = 0;
      pl.smem_bytes = (size_t)32 * pl.lmax_c * es;
    }
    else
    {
      // time-windowed shared memory (float PCFs too long for the plain
      // layout); the layout is sized below, once the rows per item are known
      pl.smem = true;
      pl.packed = false;
      pl.kvar = 6;
      pl.warps = want_w > 0 ? std::min(want_w, 32) : 24;
    }

    // Rows per item = 32 q: as large as possible (fewer column reloads,
    // less end-of-item idling) while keeping >= 6 items per SM.  At most
    // 1024 rows, one processing-order window, so that bands of whole
    // windows start on item boundaries.
    // The hybrid kernel reads rows through L1 and restages only its 32
    // columns per item, so big items buy it little but a ragged tail on
    // uneven lengths: at most 64 rows (f64 stable-rank N = 20,000, L2 kernel
    // / pdist: 1921 / 2458 ms against 2048 / 2533 ms with 1024 rows).
    const uint32_t q_top = pl.kvar == 3 ? 2u : 32u;
    uint32_t q = (uint32_t)std::max(0, settings().rowChunk.load());
    if (q == 0)
    {
      q = 1;
      for (uint32_t cand = q_top; cand >= 1; cand /= 2)
      {
        if (items_for(mode, 0, nr, nc, cand) >= (uint64_t)dev.sms * 6) { q = cand; break; }
      }
    }
    pl.q = q;
    // Problems too small for 6 items per SM even at 32 rows per item: two
    // CTAs of 16 warps per SM, so one CTA's column staging and row fills
    // overlap the other's merges (N = 1000: 123.5 against 141 us).
    if (settings().warps.load() == 0 && settings().rowChunk.load() == 0 && pl.kvar == 5 && q == 1 &&
        pl.warps > 16 && items_for(mode, 0, nr, nc, 1) < (uint64_t)dev.sms * 6 &&
        ctas_per_sm(dev, 16, smem_for(16)) >= 2)
    {
      pl.warps = 16;
      pl.smem_bytes = smem_for(16);
    }
    if (pl.kvar == 6)
    {
      bool fit = false;
      for (int w = pl.warps; w >= 4 && !fit; w -= 4)
        fit = window_layout(pl, es, w, 32 * q, std::max(lmax_r, lmax_c), usable);
      if (!fit) throw Error(ST_INVALID_ARGUMENT, "time-windowed variant: the window setting does not fit in shared memory");
    }
    // A launch shape sbg_autotune_device measured for problems of this
    // shape bucket, unless the caller fixed warps or rows per item.  Only
    // the warps and rows per item change; the time-windowed kernel keeps the
    // window cap of the default plan, so no result changes by a bit.
    if (opk >= 0 && settings().warps.load() == 0 && settings().rowChunk.load() == 0)
    {
      int tw = 0, tq = 0;
      if (tune_cache_get(tune_key((int)sizeof(T), opk, mode, nr, std::max(lmax_r, lmax_c)), &tw, &tq) && tw > 0 &&
          tq > 0 && tq <= 32)
      {
        Plan trial = pl;
        bool ok = true;
        if (pl.kvar == 6)
          ok = window_layout(trial, es, tw, 32u * (uint32_t)tq, std::max(lmax_r, lmax_c), usable, pl.win_r);
        else if (pl.kvar == 5 || pl.kvar == 1 || pl.kvar == 2)
        {
          ok = smem_for(tw) <= usable;
          trial.warps = tw;
          trial.smem_bytes = smem_for(tw);
        }
        else
          trial.warps = tw;
        if (ok)
        {
          trial.q = (uint32_t)tq;
          pl = trial;
          q = pl.q;
        }
      }
    }
    const uint64_t items = items_for(mode, 0, nr, nc, q);
    const int per_sm = (pl.kvar == 0) ? 2 : ctas_per_sm(dev, pl.warps, pl.smem_bytes);
    pl.grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(items, (uint64_t)dev.sms * per_sm));
    return pl;
  }

  bool window_layout(Plan& pl, size_t es, int warps, uint32_t rows_per_item, uint32_t lmax, size_t usable,
                     uint32_t cap)
  {
    const uint32_t U = (uint32_t)kernel_unroll(es == 16);
    const size_t slots = ((size_t)rows_per_item * 4 + 15) / 16 * 16;
    auto bytes = [&](uint32_t X) { return (size_t)32 * X * es + (size_t)warps * (2 * X + U + 1) * es + slots; };
    const uint32_t top = std::max<uint32_t>(8, (lmax + 7) / 8 * 8);
    uint32_t X = cap ? cap : (uint32_t)std::max(0, settings().windowCap.load());
    if (X == 0)
    {
      // bytes(X) is linear in X: the largest multiple of 8 that fits
      const size_t fixed = bytes(0), per = bytes(1) - bytes(0);
      if (usable < fixed + 8 * per) return false;
      X = (uint32_t)std::min<size_t>((usable - fixed) / per / 8 * 8, top);
    }
    if (bytes(X) > usable) return false;
    pl.warps = warps;
    pl.lmax_c = X;
    pl.win_r = X;
    pl.row_cap = 2 * X + U + 1;
    pl.row_slots = rows_per_item;
    pl.smem_bytes = bytes(X);
    return true;
  }

  template Plan make_plan<float>(int, uint64_t, uint64_t, const LengthStats&, const LengthStats&, const DeviceInfo&,
                                  int);
  template Plan make_plan<double>(int, uint64_t, uint64_t, const LengthStats&, const LengthStats&, const DeviceInfo&,
                                   int);

  static LengthStats host_length_stats(const uint64_t* off, uint64_t n)
  {
    LengthStats s;
    if (n == 0) return s;
    uint64_t mx = 0, mn = ~0ull, sum = 0;
    for (uint64_t i = 0; i < n; ++i)
    {
      uint64_t l = off[i + 1] - off[i];
      mx = std::max(mx, l);
      mn = std::min(mn, l);
      sum += l;
    }
    s.lmax = (uint32_t)mx;
    s.lmin = (uint32_t)mn;
    s.mean = (double)sum / (double)n;
    return s;
  }


  // ---- device entry -------------------------------------------------------------

  namespace
  {
    template <typename T>
    struct AsyncBuf
    {
      void* p = nullptr;
      size_t n = 0;
      cudaStream_t s = nullptr;
      AsyncBuf(size_t bytes, cudaStream_t st) : n(bytes), s(st)
      {
        if (bytes) p = device_malloc_async(bytes, st);
      }
      ~AsyncBuf()
      {
        if (p) device_free_async(p, n, s);
      }
      AsyncBuf(const AsyncBuf&) = delete;
      AsyncBuf& operator=(const AsyncBuf&) = delete;
    };

    // Max length over a CSR held on the device (one small reduction + sync).
    __global__ void max_len_kernel(const uint64_t* off, uint64_t n, unsigned int* out)
    {
      uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
      unsigned int v = 0;
      for (; i < n; i += (uint64_t)gridDim.x * blockDim.x)
      {
        uint64_t l = off[i + 1] - off[i];
        v = max(v, (unsigned int)(l < 0xffffffffull ? l : 0xffffffffull));
      }
      v = __reduce_max_sync(0xffffffffu, v);
      if ((threadIdx.x & 31) == 0) atomicMax(out, v);
    }
  }

  template <typename T>
  static uint32_t device_max_len(const uint64_t* off, uint64_t n, cudaStream_t st, const DeviceInfo& dev)
  {
    AsyncBuf<T> buf(sizeof(unsigned int), st);
    SBG_CUDA(cudaMemsetAsync(buf.p, 0, sizeof(unsigned int), st));
    unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)dev.sms * 4);
    if (blocks == 0) blocks = 1;
    max_len_kernel<<<blocks, 256, 0, st>>>(off, n, (unsigned int*)buf.p);
    SBG_CUDA(launched());
    unsigned int h = 0;
    SBG_CUDA(cudaMemcpyAsync(&h, buf.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    SBG_CUDA(cudaStreamSynchronize(st));
    return h;
  }

  // One launch of the persistent kernel over rows [d.row_begin, d.row_end)
  // of one problem.  The queue counter is stream-ordered scratch.
  template <typename T>
  static void launch_problem(ProblemDesc<T> d, const Plan& pl, int opk, cudaStream_t st,
                             unsigned long long* given_queue = nullptr)
  {
    d.item_begin = 0;
    d.n_items = problem_item_count(d);
    if (d.n_items == 0) return;
    std::unique_ptr<AsyncBuf<T>> own;
    unsigned long long* queue = given_queue;
    if (!queue)
    {
      own.reset(new AsyncBuf<T>(sizeof(unsigned long long), st));
      queue = static_cast<unsigned long long*>(own->p);
    }
    SBG_CUDA(cudaMemsetAsync(queue, 0, sizeof(unsigned long long), st));
    LaunchParams<T> L{};
    L.one = d;
    L.probs = nullptr;
    L.n_probs = 1;
    L.total_items = d.n_items;
    L.queue = queue;
    L.lmax_c = pl.lmax_c;
    L.row_cap = pl.row_cap;
    L.win_r = pl.win_r;
    L.row_slots = pl.row_slots;
    const int grid = (int)std::min<uint64_t>((uint64_t)pl.grid, d.n_items);
    SBG_CUDA(launch_pairs<T>(L, opk, pl.kvar, pl.warps, grid, pl.smem_bytes, st));
  }

  template <typename T>
  void compute_device(int mode, int op, double p, const PcfSet<T>& rows, const PcfSet<T>* cols,
                      const uint32_t* rperm, const uint32_t* cperm, uint32_t lmax, T* out, uint64_t out_base,
                      uint64_t row_begin, uint64_t row_end, cudaStream_t st)
  {
    const DeviceInfo dev = device_info();
    if (mode == MODE_CROSS && !cols) throw Error(ST_INVALID_ARGUMENT, "cdist needs a column set");
    const PcfSet<T>& cs = (mode == MODE_CROSS) ? *cols : rows;
    if (row_end > rows.n) row_end = rows.n;
    if (row_begin >= row_end || cs.n == 0) return;
    const int opk = op_kind(op, p);

    if (lmax == 0)
    {
      lmax = device_max_len<T>(rows.off, rows.n, st, dev);
      if (mode == MODE_CROSS) lmax = std::max(lmax, device_max_len<T>(cs.off, cs.n, st, dev));
    }
    LengthStats ls;
    ls.lmax = lmax;
    ls.lmin = 1;
    ls.mean = lmax;
    const Plan pl = make_plan<T>(mode, rows.n, cs.n, ls, ls, dev, opk);
    if (row_begin % (32ull * pl.q) != 0)
      throw Error(ST_INVALID_ARGUMENT, "row_begin must be a multiple of the row chunk (32*q)");

    // Processing order: by breakpoint count within windows of
    // LENGTH_ORDER_WINDOW PCFs, computed on the stream, unless the caller or
    // the order setting fixed one.  The band must be whole windows: the
    // order permutes PCFs only inside a window, so such a band holds the
    // same rows in either order and its results stay in the band's
    // contiguous output range.  The permutation is the one the host entry
    // uses, so both give the same bits.
    std::unique_ptr<AsyncBuf<T>> order_buf;
    const bool windows = row_begin % LENGTH_ORDER_WINDOW == 0 &&
                         (row_end % LENGTH_ORDER_WINDOW == 0 || row_end == rows.n);
    const bool caller_perm = rperm || cperm;
    if (!caller_perm && windows && settings().order.load() != 1 && rows.n <= 0xffffffffull &&
        cs.n <= 0xffffffffull)
    {
      const uint64_t nr = rows.n, nc = (mode == MODE_CROSS) ? cs.n : 0;
      const size_t perm_bytes = ((nr + nc) * sizeof(uint32_t) + 255) / 256 * 256;
      const size_t key_bytes = std::max(length_order_scratch_bytes(nr), length_order_scratch_bytes(nc));
      order_buf.reset(new AsyncBuf<T>(perm_bytes + key_bytes, st));
      uint32_t* rp = static_cast<uint32_t*>(order_buf->p);
      void* keys = static_cast<char*>(order_buf->p) + perm_bytes;
      length_order_device(rows.off, nr, rp, keys, st);
      rperm = rp;
      if (mode == MODE_CROSS)
      {
        length_order_device(cs.off, nc, rp + nr, keys, st);
        cperm = rp + nr;
      }
    }

    ProblemDesc<T> d{};
    d.rpts = rows.pts; d.roff = rows.off; d.rperm = rperm; d.nr = rows.n;
    d.cpts = cs.pts; d.coff = cs.off; d.cperm = (mode == MODE_CROSS) ? cperm : rperm; d.nc = cs.n;
    d.out = out; d.out_base = out_base; d.ld = cs.n;
    d.row_begin = row_begin; d.row_end = row_end;
    d.q = pl.q; d.mode = mode; d.p = (T)p;
    {
      // rows [row_begin, row_end) in caller order, or in the windowed length
      // order, own one contiguous range; with a caller's order the results
      // may land anywhere in the matrix
      const uint64_t hi = caller_perm ? output_count(mode, rows.n, cs.n) : row_output_start(mode, row_end, cs.n);
      d.out_count = hi > out_base ? hi - out_base : 0;
    }

    // Packed segment layout for the global-memory variant (needs the point
    // totals, read back with one synchronisation).
    std::unique_ptr<AsyncBuf<T>> rpack, cpack;
    if (pl.packed)
    {
      uint64_t rtot = 0, ctot = 0;
      SBG_CUDA(cudaMemcpyAsync(&rtot, rows.off + rows.n, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
      if (mode == MODE_CROSS)
        SBG_CUDA(cudaMemcpyAsync(&ctot, cs.off + cs.n, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
      SBG_CUDA(cudaStreamSynchronize(st));
      rpack.reset(new AsyncBuf<T>(sizeof(Elem<T>) * std::max<uint64_t>(rtot, 1), st));
      SBG_CUDA(launch_pack<T>(rows.pts, rows.off, rows.n, (Elem<T>*)rpack->p, rtot, dev.sms, st));
      d.rpts = reinterpret_cast<const T*>(rpack->p);
      d.cpts = d.rpts;
      d.rcap = rtot;
      d.ccap = rtot;
      if (mode == MODE_CROSS)
      {
        cpack.reset(new AsyncBuf<T>(sizeof(Elem<T>) * std::max<uint64_t>(ctot, 1), st));
        SBG_CUDA(launch_pack<T>(cs.pts, cs.off, cs.n, (Elem<T>*)cpack->p, ctot, dev.sms, st));
        d.cpts = reinterpret_cast<const T*>(cpack->p);
        d.ccap = ctot;
      }
    }
    launch_problem<T>(d, pl, opk, st);
  }

  template void compute_device<float>(int, int, double, const PcfSet<float>&, const PcfSet<float>*, const uint32_t*,
                                      const uint32_t*, uint32_t, float*, uint64_t, uint64_t, uint64_t, cudaStream_t);
  template void compute_device<double>(int, int, double, const PcfSet<double>&, const PcfSet<double>*,
                                       const uint32_t*, const uint32_t*, uint32_t, double*, uint64_t, uint64_t,
                                       uint64_t, cudaStream_t);

  template <typename T>
  size_t scratch_needed(int mode, uint64_t n_rows, uint64_t n_cols, uint32_t lmax, uint64_t row_points,
                        uint64_t col_points)
  {
    const DeviceInfo dev = device_info();
    LengthStats ls;
    ls.lmax = lmax; ls.lmin = 1; ls.mean = lmax;
    const Plan pl = make_plan<T>(mode, n_rows, mode == MODE_CROSS ? n_cols : n_rows, ls, ls, dev, -1);
    size_t need = 256;  // work-queue counter
    if (pl.packed)
    {
      need += ((sizeof(Elem<T>) * row_points + 255) / 256) * 256;
      if (mode == MODE_CROSS) need += ((sizeof(Elem<T>) * col_points + 255) / 256) * 256;
    }
    return need;
  }

  template <typename T>
  void compute_device_scratch(int mode, int op, double p, const PcfSet<T>& rows, const PcfSet<T>* cols,
                              const uint32_t* rperm, const uint32_t* cperm, uint32_t lmax, uint64_t row_points,
                              uint64_t col_points, T* out, uint64_t out_base, uint64_t row_begin, uint64_t row_end,
                              void* scratch, size_t scratch_bytes, cudaStream_t st)
  {
    const DeviceInfo dev = device_info();
    if (mode == MODE_CROSS && !cols) throw Error(ST_INVALID_ARGUMENT, "cdist needs a column set");
    if (lmax == 0) throw Error(ST_INVALID_ARGUMENT, "max_points must be given (measuring it would allocate)");
    const PcfSet<T>& cs = (mode == MODE_CROSS) ? *cols : rows;
    if (row_end == 0 || row_end > rows.n) row_end = rows.n;
    if (row_begin >= row_end || cs.n == 0) return;
    const int opk = op_kind(op, p);
    LengthStats ls;
    ls.lmax = lmax; ls.lmin = 1; ls.mean = lmax;
    const Plan pl = make_plan<T>(mode, rows.n, cs.n, ls, ls, dev, opk);
    if (row_begin % (32ull * pl.q) != 0)
      throw Error(ST_INVALID_ARGUMENT, "row_begin must be a multiple of the row chunk (32*q)");
    const size_t need = scratch_needed<T>(mode, rows.n, cs.n, lmax, row_points, col_points);
    if (need > scratch_bytes)
      throw Error(ST_INVALID_ARGUMENT, "problem needs " + std::to_string(need) + " bytes of scratch; the limit is " +
                  std::to_string(scratch_bytes) + " bytes");

    ProblemDesc<T> d{};
    d.rpts = rows.pts; d.roff = rows.off; d.rperm = rperm; d.nr = rows.n;
    d.cpts = cs.pts; d.coff = cs.off; d.cperm = (mode == MODE_CROSS) ? cperm : rperm; d.nc = cs.n;
    d.out = out; d.out_base = out_base; d.ld = cs.n;
    d.row_begin = row_begin; d.row_end = row_end;
    d.q = pl.q; d.mode = mode; d.p = (T)p;
    {
      const uint64_t hi = (rperm || cperm) ? output_count(mode, rows.n, cs.n) : row_output_start(mode, row_end, cs.n);
      d.out_count = hi > out_base ? hi - out_base : 0;
    }
    char* base = static_cast<char*>(scratch);
    if (pl.packed)
    {
      Elem<T>* rp = reinterpret_cast<Elem<T>*>(base + 256);
      SBG_CUDA(launch_pack<T>(rows.pts, rows.off, rows.n, rp, row_points, dev.sms, st));
      d.rpts = reinterpret_cast<const T*>(rp);
      d.cpts = d.rpts;
      d.rcap = row_points;
      d.ccap = row_points;
      if (mode == MODE_CROSS)
      {
        Elem<T>* cp = reinterpret_cast<Elem<T>*>(base + 256 + ((sizeof(Elem<T>) * row_points + 255) / 256) * 256);
        SBG_CUDA(launch_pack<T>(cs.pts, cs.off, cs.n, cp, col_points, dev.sms, st));
        d.cpts = reinterpret_cast<const T*>(cp);
        d.ccap = col_points;
      }
    }
    launch_problem<T>(d, pl, opk, st, reinterpret_cast<unsigned long long*>(base));
  }

  template size_t scratch_needed<float>(int, uint64_t, uint64_t, uint32_t, uint64_t, uint64_t);
  template size_t scratch_needed<double>(int, uint64_t, uint64_t, uint32_t, uint64_t, uint64_t);
  template void compute_device_scratch<float>(int, int, double, const PcfSet<float>&, const PcfSet<float>*,
                                              const uint32_t*, const uint32_t*, uint32_t, uint64_t, uint64_t, float*,
                                              uint64_t, uint64_t, uint64_t, void*, size_t, cudaStream_t);
  template void compute_device_scratch<double>(int, int, double, const PcfSet<double>&, const PcfSet<double>*,
                                               const uint32_t*, const uint32_t*, uint32_t, uint64_t, uint64_t,
                                               double*, uint64_t, uint64_t, uint64_t, void*, size_t, cudaStream_t);

  // ---- host pipeline ----------------------------------------------------------

  namespace
  {
    // With the device-verbose setting on, the host entry reports on stderr
    // when each of its phases ended (host clock, ms since the call began);
    // declared first in the call, it reports last, after the buffers are
    // freed.
    struct PhaseLog
    {
      bool on = settings().deviceVerbose.load();
      std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
      std::string text;
      void mark(const char* what, long k = -1)
      {
        if (!on) return;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        char buf[64];
        if (k >= 0) std::snprintf(buf, sizeof buf, " %s%ld %.1f", what, k, ms);
        else std::snprintf(buf, sizeof buf, " %s %.1f", what, ms);
        text += buf;
      }
      ~PhaseLog()
      {
        if (!on) return;
        mark("freed");
        std::fprintf(stderr, "sbgpu host entry, ms since start:%s\n", text.c_str());
      }
    };

    struct StreamGuard
    {
      cudaStream_t s = nullptr;
      StreamGuard() { SBG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
      ~StreamGuard() { if (s) cudaStreamDestroy(s); }
    };
    struct EventGuard
    {
      cudaEvent_t e = nullptr;
      EventGuard() { SBG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming)); }
      ~EventGuard() { if (e) cudaEventDestroy(e); }
    };

    template <typename T>
    struct DeviceSet
    {
      DeviceBuffer pts, off;
      PcfSet<T> view;
      void upload(const PcfSet<T>& h, cudaStream_t s)
      {
        const uint64_t npts = h.n ? h.off[h.n] : 0;
        pts.reset(std::max<uint64_t>(1, npts) * 2 * sizeof(T));
        off.reset((h.n + 1) * sizeof(uint64_t));
        if (npts) upload_pageable(pts.get(), h.pts, npts * 2 * sizeof(T), s);
        SBG_CUDA(cudaMemcpyAsync(off.get(), h.off, (h.n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
        view.pts = pts.as<T>();
        view.off = off.as<uint64_t>();
        view.n = h.n;
      }
    };
  }

  template <typename T>
  void compute_host(int mode, int op, double p, const PcfSet<T>& rows, const PcfSet<T>* cols, T* out, bool validate,
                    const RunControl& ctl)
  {
    PhaseLog phases;
    if (mode == MODE_CROSS && !cols) throw Error(ST_INVALID_ARGUMENT, "cdist needs a column set");
    const PcfSet<T>& cs = (mode == MODE_CROSS) ? *cols : rows;
    if (validate)
    {
      validate_pcfs(rows, mode == MODE_CROSS ? "X" : "input");
      if (mode == MODE_CROSS) validate_pcfs(cs, "Y");
    }
    phases.mark("checked");
    (void)op_kind(op, p);
    const uint64_t total = output_count(mode, rows.n, cs.n);
    if (total == 0) return;
    if (!out) throw Error(ST_INVALID_ARGUMENT, "null output");

    const DeviceInfo dev = device_info();
    const LengthStats rstat = host_length_stats(rows.off, rows.n);
    const LengthStats cstat = (mode == MODE_CROSS) ? host_length_stats(cs.off, cs.n) : rstat;
    const uint32_t lmax = std::max(rstat.lmax, cstat.lmax);

    StreamGuard compute, copy;
    DeviceSet<T> drows, dcols;
    drows.upload(rows, compute.s);
    if (mode == MODE_CROSS) dcols.upload(cs, compute.s);
    phases.mark("uploaded");

    // Processing order: by length within windows (unless the order setting
    // asks for the caller's), the permutation the device entry computes on
    // the GPU, so both entries give the same bits.
    size_t freeb = 0, totalb = 0;
    SBG_CUDA(cudaMemGetInfo(&freeb, &totalb));
    const size_t out_bytes = (size_t)total * sizeof(T);
    const size_t budget = (size_t)((double)freeb * 0.8);
    int order = settings().order.load();
    const bool sorted = order != 1 && rows.n <= 0xffffffffull && cs.n <= 0xffffffffull;
    DeviceBuffer drperm, dcperm;
    if (sorted)
    {
      // computed on the stream from the uploaded offsets (one launch)
      drperm.reset(std::max<uint64_t>(1, rows.n) * sizeof(uint32_t));
      length_order_device(drows.view.off, rows.n, drperm.as<uint32_t>(), nullptr, compute.s);
      if (mode == MODE_CROSS)
      {
        dcperm.reset(std::max<uint64_t>(1, cs.n) * sizeof(uint32_t));
        length_order_device(dcols.view.off, cs.n, dcperm.as<uint32_t>(), nullptr, compute.s);
      }
    }

    const Plan pl = make_plan<T>(mode, rows.n, cs.n, rstat, cstat, dev, op_kind(op, p));
    const uint64_t chunk_rows = 32ull * pl.q;
    phases.mark("ordered");

    // Output route.  Direct: on coherent hosts (Grace + NVLink-C2C, where the
    // device walks the host page tables) the kernel stores straight into the
    // caller's matrix, one launch, no device output buffer and no copies.
    // Staged: bands of whole row chunks into two device buffers, each band
    // copied out while the next band computes (HostStager).
    int out_mode = settings().outputMode.load();
    bool direct = false;
    if (out_mode == 2)
    {
      int pageable = 0, hpt = 0;
      host_memory_access(&pageable, &hpt);
      if (!(pageable && hpt))
        throw Error(ST_INVALID_ARGUMENT, "direct host output needs a device that uses the host page tables");
      direct = true;
    }

    // Bands of whole row chunks.  One band when writing directly or when the
    // output is small.  In length order the bands are also whole order
    // windows: the order only permutes PCFs inside a window, so the rows of
    // a band of windows are the same set in either order, and every pair
    // with its later PCF in the band lands in the band's contiguous range
    // of the condensed (or dense) output.
    uint64_t band_bytes = settings().bandBytes.load();
    const bool auto_bands = band_bytes == 0;
    if (band_bytes == 0) band_bytes = out_bytes > (512ull << 20) ? out_bytes / 8 + 1 : out_bytes;
    band_bytes = std::min<uint64_t>(band_bytes, budget / 2 > 0 ? budget / 2 : band_bytes);
    std::vector<std::pair<uint64_t, uint64_t>> bands;
    uint64_t align = chunk_rows;
    if (sorted)
    {
      uint64_t g = align, h = LENGTH_ORDER_WINDOW;
      while (h) { const uint64_t r = g % h; g = h; h = r; }
      align = align / g * LENGTH_ORDER_WINDOW;  // lcm(chunk_rows, window)
    }
    if (direct || band_bytes >= out_bytes)
    {
      if (!direct && out_bytes > budget) throw Error(ST_OUT_OF_MEMORY, "output does not fit in device memory");
      bands.emplace_back(0, rows.n);
    }
    else
    {
      // Bands of whole row units, from the last row down.  Nothing overlaps
      // the copy-out of the band computed last, and in a triangle the first
      // rows hold the least output, so the schedule ends on them.  With
      // automatic sizes the two lowest bands are cut into parts of about
      // 1/2, 1/4, ... of their output, top part first, so the last copy is
      // the first unit's output (about 2 MB for 1024 rows in float32), not
      // a full band's.
      const uint64_t units = (rows.n + align - 1) / align;
      auto ustart = [&](uint64_t u) { return std::min<uint64_t>(rows.n, u * align); };
      uint64_t ue = units;
      while (ue > 0)
      {
        uint64_t ub = ue - 1;
        while (ub > 0)
        {
          const uint64_t bytes =
              (row_output_start(mode, ustart(ue), cs.n) - row_output_start(mode, ustart(ub - 1), cs.n)) * sizeof(T);
          if (bytes > band_bytes) break;
          --ub;
        }
        bands.emplace_back(ustart(ub), ustart(ue));
        ue = ub;
      }
      if (auto_bands && bands.size() > 1)
      {
        // The two lowest bands are cut again into parts of about half the
        // remaining output each: every part's copy-out (about 3x faster than
        // the kernel writes it) then hides behind the compute of the next,
        // which is at least half its size, and the last part is unit 0.
        bands.pop_back();
        const auto above = bands.back();  // the lowest two end here
        bands.pop_back();
        uint64_t top = (above.second + align - 1) / align;
        auto out_of = [&](uint64_t u0, uint64_t u1) {
          return row_output_start(mode, ustart(u1), cs.n) - row_output_start(mode, ustart(u0), cs.n);
        };
        while (top > 1)
        {
          const uint64_t half = out_of(0, top) / 2;
          uint64_t ub = top - 1;
          while (ub > 1 && out_of(ub, top) < half) --ub;
          bands.emplace_back(ustart(ub), ustart(top));
          top = ub;
        }
        bands.emplace_back(0, ustart(top));
      }
    }
    uint64_t max_band = 0;
    for (auto& b : bands)
      max_band = std::max<uint64_t>(max_band, row_output_start(mode, b.second, cs.n) - row_output_start(mode, b.first, cs.n));
    const int nbuf = direct ? 0 : (bands.size() > 1 ? 2 : 1);
    DeviceBuffer obuf[2];
    for (int b = 0; b < nbuf; ++b) obuf[b].reset(std::max<uint64_t>(1, max_band) * sizeof(T));
    EventGuard computed[2], copied[2];
    phases.mark("buffers");

    // Packed segment layout, once, for the global-memory variant.
    DeviceBuffer rpack, cpack;
    const T* kr_pts = drows.view.pts;
    const T* kc_pts = (mode == MODE_CROSS) ? dcols.view.pts : drows.view.pts;
    if (pl.packed)
    {
      rpack.reset(sizeof(Elem<T>) * std::max<uint64_t>(1, rows.off[rows.n]));
      SBG_CUDA(launch_pack<T>(drows.view.pts, drows.view.off, rows.n, rpack.as<Elem<T>>(), rows.off[rows.n], dev.sms,
                              compute.s));
      kr_pts = reinterpret_cast<const T*>(rpack.get());
      kc_pts = kr_pts;
      if (mode == MODE_CROSS)
      {
        cpack.reset(sizeof(Elem<T>) * std::max<uint64_t>(1, cs.off[cs.n]));
        SBG_CUDA(launch_pack<T>(dcols.view.pts, dcols.view.off, cs.n, cpack.as<Elem<T>>(), cs.off[cs.n], dev.sms,
                                compute.s));
        kc_pts = reinterpret_cast<const T*>(cpack.get());
      }
    }
    const int opk = op_kind(op, p);

    // Bands alternate between two compute streams, one per output buffer:
    // a band's CTAs start on the SMs that the previous band's last wave
    // leaves idle, instead of after its last item.  Bands share nothing but
    // the inputs, which the second stream waits for.
    StreamGuard compute2;
    EventGuard inputs_ready;
    SBG_CUDA(cudaEventRecord(inputs_ready.e, compute.s));
    SBG_CUDA(cudaStreamWaitEvent(compute2.s, inputs_ready.e, 0));
    auto band_stream = [&](size_t k) { return (k % 2) ? compute2.s : compute.s; };

    auto launch_band = [&](size_t k) {
      const int b = (int)(k % 2);
      const cudaStream_t bs = band_stream(k);
      if (k >= 2) SBG_CUDA(cudaStreamWaitEvent(bs, copied[b].e, 0));
      ProblemDesc<T> d{};
      d.rpts = kr_pts; d.roff = drows.view.off; d.nr = rows.n;
      d.cpts = kc_pts; d.coff = (mode == MODE_CROSS) ? dcols.view.off : drows.view.off; d.nc = cs.n;
      d.rperm = sorted ? drperm.as<uint32_t>() : nullptr;
      d.cperm = sorted ? (mode == MODE_CROSS ? dcperm.as<uint32_t>() : drperm.as<uint32_t>()) : nullptr;
      d.out = direct ? out : obuf[b].as<T>();
      d.out_base = direct ? 0 : row_output_start(mode, bands[k].first, cs.n);
      d.out_count = direct ? total : row_output_start(mode, bands[k].second, cs.n) - d.out_base;
      d.ld = cs.n;
      d.row_begin = bands[k].first; d.row_end = bands[k].second;
      d.q = pl.q; d.mode = mode; d.p = (T)p;
      d.rcap = rows.off[rows.n];
      d.ccap = cs.off[cs.n];
      // The small bands at the end of the schedule take fewer rows per item,
      // so that each still gives the planner's 6 items per SM instead of
      // ending on a ragged last wave.  Only an even q is halved, so the new
      // row chunk divides the old one and the band starts stay multiples of
      // it.  No pair's arithmetic depends on the item shape.
      if (!direct)
        while (d.q % 2 == 0 && problem_item_count(d) < 6ull * (uint64_t)dev.sms) d.q /= 2;
      launch_problem<T>(d, pl, opk, bs);
      SBG_CUDA(cudaEventRecord(computed[b].e, bs));
    };

    bool cancelled = false;
    if (direct)
    {
      launch_band(0);
      SBG_CUDA(cudaStreamSynchronize(compute.s));
      if (ctl.progress) ctl.progress(total);
      return;
    }
    HostStager stager(std::min<uint64_t>(std::max<uint64_t>(max_band * sizeof(T), 1), 256ull << 20));
    launch_band(0);
    for (size_t k = 0; k < bands.size(); ++k)
    {
      const int b = (int)(k % 2);
      if (k + 1 < bands.size() && !(ctl.stop && ctl.stop->load())) launch_band(k + 1);
      const uint64_t rb = bands[k].first, re = bands[k].second;
      const uint64_t lo = row_output_start(mode, rb, cs.n);
      const uint64_t hi = row_output_start(mode, re, cs.n);
      SBG_CUDA(cudaStreamWaitEvent(copy.s, computed[b].e, 0));
      if (hi > lo) stager.copy(out + lo, obuf[b].as<T>(), (hi - lo) * sizeof(T), copy.s);
      stager.flush();
      phases.mark("band", (long)k);
      SBG_CUDA(cudaEventRecord(copied[b].e, copy.s));
      if (ctl.progress) ctl.progress(hi - lo);
      if (ctl.stop && ctl.stop->load()) { cancelled = true; break; }
    }
    stager.flush();
    SBG_CUDA(cudaStreamSynchronize(compute.s));
    SBG_CUDA(cudaStreamSynchronize(compute2.s));
    SBG_CUDA(cudaStreamSynchronize(copy.s));
    phases.mark("synced");
    if (cancelled) throw Error(ST_CANCELLED, "task was cancelled");
  }

  template void compute_host<float>(int, int, double, const PcfSet<float>&, const PcfSet<float>*, float*, bool,
                                    const RunControl&);
  template void compute_host<double>(int, int, double, const PcfSet<double>&, const PcfSet<double>*, double*, bool,
                                     const RunControl&);
}
