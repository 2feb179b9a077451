// Batched pairwise integration: many independent PCF arrays of uneven size
// in one persistent launch.
//
// A batch is planned once (sbg_batch_create) and launched many times:
//   * per problem, PCFs are visited in order of breakpoint count (a length
//     permutation), so each 32-column group holds similar lengths and the
//     warp-uniform step count wastes little;
//   * the packed segment layout of every problem is built once;
//   * problem descriptors are ordered by estimated merge work, largest
//     first, so the device work queue hands out the long items early and the
//     tail of the launch is short;
//   * a launch is one queue reset plus one kernel; with SBG_BATCH_GRAPH the
//     pair is captured once into a CUDA graph and replayed;
//   * sbg_batch_autotune times a few (warps per CTA, rows per item)
//     settings on the real batch, then a few splits of shared memory between
//     the column block and the row buffers (the hybrid kernel's column
//     block; with SBG_BATCH_TUNE_WINDOW the time-windowed kernel's window
//     cap), and keeps the fastest.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <vector>

namespace sbg
{
  struct BatchBase
  {
    virtual ~BatchBase() = default;
    virtual void launch(cudaStream_t st) = 0;
    virtual double autotune(cudaStream_t st) = 0;
    virtual void info(uint64_t* items, uint64_t* pairs, int* warps, int* rows_per_item) const = 0;
    virtual uint32_t shared_split() const = 0;
  };

  template <typename T>
  struct Batch : BatchBase
  {
    int op = 0, mode = 0, opk = 0;
    double p = 1.0;
    bool use_graph = false;
    bool tune_window = false;   // the autotune may move the window cap (and so window ends)
    DeviceInfo dev;
    std::vector<ProblemDesc<T>> descs;   // host copy, in launch order
    std::vector<uint64_t> q_base;        // per launch-order problem: chosen q at scale 1
    DeviceBuffer d_descs, d_queue, d_perm, d_packed;
    Plan pl;
    uint32_t q_scale = 1;
    uint64_t total_items = 0, total_pairs = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t graph_kernels = 0;  // kernels one replay of the graph runs
    bool windowed = false;       // time-windowed kernel (else the hybrid one)
    uint32_t lmax = 1;           // longest PCF of the batch
    size_t usable = 0;           // shared memory per CTA
    uint32_t win_cap = 0;        // slice cap, fixed for the batch: window ends (and so the
                                 // rounding of every sum) do not change with the autotuned shape

    ~Batch() override { drop_graph(); }

    void drop_graph()
    {
      if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
      if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
    }

    // Rows per item and warps; the time-windowed layout depends on both.
    // False (and nothing changed) when that layout does not fit.
    uint64_t max_q(uint32_t qscale) const
    {
      uint64_t qmax = 1;
      for (size_t k = 0; k < descs.size(); ++k) qmax = std::max<uint64_t>(qmax, q_base[k] * qscale);
      return qmax;
    }

    bool rebuild_items(uint32_t warps, uint32_t qscale)
    {
      if (windowed)
      {
        const uint64_t qmax = max_q(qscale);
        Plan trial = pl;
        if (qmax > 1024 ||
            !window_layout(trial, sizeof(Elem<T>), (int)warps, (uint32_t)(32 * qmax), lmax, usable, win_cap))
          return false;
        pl = trial;
      }
      uint64_t begin = 0;
      for (size_t k = 0; k < descs.size(); ++k)
      {
        descs[k].q = (uint32_t)std::max<uint64_t>(1, q_base[k] * qscale);
        descs[k].item_begin = begin;
        descs[k].n_items = problem_item_count(descs[k]);
        begin += descs[k].n_items;
      }
      total_items = begin;
      pl.warps = (int)warps;
      q_scale = qscale;
      SBG_CUDA(cudaMemcpy(d_descs.get(), descs.data(), sizeof(ProblemDesc<T>) * descs.size(), cudaMemcpyHostToDevice));
      drop_graph();
      return true;
    }

    void enqueue(cudaStream_t st)
    {
      if (total_items == 0) return;
      SBG_CUDA(cudaMemsetAsync(d_queue.get(), 0, sizeof(unsigned long long), st));
      LaunchParams<T> L{};
      L.probs = d_descs.as<ProblemDesc<T>>();
      L.n_probs = (int)descs.size();
      L.total_items = total_items;
      L.queue = d_queue.as<unsigned long long>();
      L.lmax_c = pl.lmax_c;
      L.row_cap = pl.row_cap;
      L.win_r = pl.win_r;
      L.row_slots = pl.row_slots;
      const int grid = (int)std::min<uint64_t>((uint64_t)dev.sms * ctas_per_sm(dev, pl.warps, pl.smem_bytes),
                                                 total_items);
      SBG_CUDA(launch_pairs<T>(L, opk, pl.kvar, pl.warps, grid, pl.smem_bytes, st));
    }

    void launch(cudaStream_t st) override
    {
      if (!use_graph)
      {
        enqueue(st);
        return;
      }
      if (!exec)
      {
        // Capture on a private stream, then replay on the caller's stream.
        cudaStream_t cap;
        SBG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess)
        {
          // kernels recorded during capture have not run: count them per replay
          const uint64_t before = kernel_launches();
          try { enqueue(cap); } catch (...) { cudaGraph_t g0; cudaStreamEndCapture(cap, &g0); if (g0) cudaGraphDestroy(g0); cudaStreamDestroy(cap); throw; }
          graph_kernels = kernel_launches() - before;
          uncount_launches(graph_kernels);
          e = cudaStreamEndCapture(cap, &graph);
        }
        cudaStreamDestroy(cap);
        if (e != cudaSuccess) throw_cuda(e, __FILE__, __LINE__);
        SBG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
      }
      SBG_CUDA(cudaGraphLaunch(exec, st));
      count_launches(graph_kernels);
    }

    double time_once(cudaStream_t st, int reps)
    {
      cudaEvent_t a, b;
      SBG_CUDA(cudaEventCreate(&a));
      SBG_CUDA(cudaEventCreate(&b));
      enqueue(st);  // warm
      SBG_CUDA(cudaEventRecord(a, st));
      for (int r = 0; r < reps; ++r) enqueue(st);
      SBG_CUDA(cudaEventRecord(b, st));
      SBG_CUDA(cudaEventSynchronize(b));
      float ms = 0.f;
      SBG_CUDA(cudaEventElapsedTime(&ms, a, b));
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return ms / reps;
    }

    double autotune(cudaStream_t st) override
    {
      const uint32_t w0 = (uint32_t)pl.warps, s0 = q_scale;
      double best = 1e300;
      uint32_t bw = w0, bs = s0;
      const uint32_t warps_c[] = {8, 16, 24, 32};
      const uint32_t scale_c[] = {1, 2, 4};
      for (uint32_t w : warps_c)
      {
        for (uint32_t s : scale_c)
        {
          if (!rebuild_items(w, s)) continue;
          const double ms = time_once(st, 2);
          if (ms < best) { best = ms; bw = w; bs = s; }
        }
      }
      if (!rebuild_items(bw, bs)) throw Error(ST_INTERNAL, "batch autotune: the chosen layout no longer fits");
      if (windowed)
      {
        if (!tune_window) return best;
        // Window caps from the largest that fits the chosen shape down to
        // half the batch's cap: a smaller cap leaves fewer elements per
        // window in the column block and row buffers (more windows per
        // pair), a larger one only fits fewer warps or rows per item.
        const uint32_t base = win_cap;
        uint32_t most = base;
        Plan probe;
        const uint64_t qmax = max_q(bs);
        if (qmax <= 1024 &&
            window_layout(probe, sizeof(Elem<T>), (int)bw, (uint32_t)(32 * qmax), lmax, usable, 0))
          most = std::max(most, probe.lmax_c);
        uint32_t bc = base;
        for (uint32_t c : {most, base * 3 / 4, base / 2})
        {
          if (c < 8 || c == base) continue;
          win_cap = c;
          if (!rebuild_items(bw, bs)) continue;
          const double ms = time_once(st, 2);
          if (ms < best) { best = ms; bc = c; }
        }
        win_cap = bc;
        if (!rebuild_items(bw, bs)) throw Error(ST_INTERNAL, "batch autotune: the chosen window cap no longer fits");
        return best;
      }
      // Hybrid kernel: column groups longer than the staging block read
      // their columns through L1; a smaller block leaves more of the SM's
      // unified L1/shared memory to the rows, which are always read through L1.
      const uint32_t full = pl.lmax_c;
      uint32_t bc = full;
      for (uint32_t c : {full / 2, full / 4})
      {
        if (c < 32) continue;
        set_column_block(c);
        const double ms = time_once(st, 2);
        if (ms < best) { best = ms; bc = c; }
      }
      set_column_block(bc);
      return best;
    }

    void set_column_block(uint32_t cap)
    {
      pl.lmax_c = cap;
      pl.smem_bytes = (size_t)32 * cap * sizeof(Elem<T>);
      drop_graph();
    }

    void info(uint64_t* items, uint64_t* pairs, int* warps, int* rows_per_item) const override
    {
      if (items) *items = total_items;
      if (pairs) *pairs = total_pairs;
      if (warps) *warps = pl.warps;
      if (rows_per_item) *rows_per_item = (int)(32 * q_scale);
    }

    // elements per PCF in the shared column block: the window cap of the
    // time-windowed kernel, or the hybrid kernel's column block
    uint32_t shared_split() const override { return pl.lmax_c; }
  };

  template <typename T>
  static BatchBase* make_batch(int op, double p, int mode, const sbg_problem* probs, uint64_t n, int flags)
  {
    std::unique_ptr<Batch<T>> b(new Batch<T>);
    b->op = op; b->p = p; b->mode = mode; b->opk = op_kind(op, p);
    b->use_graph = (flags & SBG_BATCH_GRAPH) != 0;
    b->tune_window = (flags & SBG_BATCH_TUNE_WINDOW) != 0;
    b->dev = device_info();
    const bool sort_len = (flags & SBG_BATCH_CALLER_ORDER) == 0;
    // the time-windowed kernel for float (the hybrid one on request), the
    // hybrid one for double (FP64-bound either way; it measured faster)
    const int var = settings().variant.load();
    b->windowed = var == 6 || (var != 4 && sizeof(T) == 4);

    // Host copies of the offsets (given, or read back once).
    std::vector<std::vector<uint64_t>> hoff(n);
    uint64_t tot_pts = 0, tot_n = 0;
    uint32_t lmax = 1;
    for (uint64_t k = 0; k < n; ++k)
    {
      const sbg_problem& P = probs[k];
      if (P.n == 0) continue;
      if (!P.points || !P.offsets || !P.out) throw Error(ST_INVALID_ARGUMENT, "problem " + std::to_string(k) + ": null pointer");
      hoff[k].resize(P.n + 1);
      if (P.host_offsets) std::copy(P.host_offsets, P.host_offsets + P.n + 1, hoff[k].begin());
      else SBG_CUDA(cudaMemcpy(hoff[k].data(), P.offsets, (P.n + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost));
      for (uint64_t i = 0; i < P.n; ++i)
      {
        const uint64_t l = hoff[k][i + 1] - hoff[k][i];
        if (l == 0) throw Error(ST_INVALID_INPUT, "problem " + std::to_string(k) + ": PCF " + std::to_string(i) + " has no breakpoints");
        lmax = (uint32_t)std::max<uint64_t>(lmax, l);
      }
      tot_pts += hoff[k][P.n];
      tot_n += P.n;
    }

    // Length permutations and packed layouts, concatenated.
    b->d_perm.reset(std::max<uint64_t>(1, tot_n) * sizeof(uint32_t));
    if (!b->windowed) b->d_packed.reset(std::max<uint64_t>(1, tot_pts) * sizeof(Elem<T>));
    std::vector<uint32_t> hperm(tot_n);
    uint64_t pbase = 0, ebase = 0;
    struct Pending { ProblemDesc<T> d; double cost; uint64_t qb; };
    std::vector<Pending> pend;
    for (uint64_t k = 0; k < n; ++k)
    {
      const sbg_problem& P = probs[k];
      if (P.n == 0) continue;
      uint32_t* hp = hperm.data() + pbase;
      std::iota(hp, hp + P.n, 0u);
      const uint64_t* o = hoff[k].data();
      if (sort_len)
        std::stable_sort(hp, hp + P.n, [o](uint32_t a, uint32_t c) { return (o[a + 1] - o[a]) < (o[c + 1] - o[c]); });
      ProblemDesc<T> d{};
      if (b->windowed) d.rpts = static_cast<const T*>(P.points);  // the CSR itself
      else
      {
        Elem<T>* packed = b->d_packed.template as<Elem<T>>() + ebase;
        SBG_CUDA(launch_pack<T>(static_cast<const T*>(P.points), P.offsets, P.n, packed, o[P.n], b->dev.sms, 0));
        d.rpts = reinterpret_cast<const T*>(packed);
      }
      d.roff = P.offsets; d.nr = P.n;
      d.cpts = d.rpts; d.coff = P.offsets; d.nc = P.n;
      d.rperm = sort_len ? b->d_perm.template as<uint32_t>() + pbase : nullptr;
      d.cperm = d.rperm;
      d.out = static_cast<T*>(P.out); d.out_base = 0; d.ld = P.n;
      d.out_count = output_count(mode, P.n, P.n);
      d.row_begin = 0; d.row_end = P.n;
      d.mode = mode; d.p = (T)p;
      d.rcap = o[P.n]; d.ccap = o[P.n];
      const double meanL = (double)o[P.n] / (double)P.n;
      const double pairs = (double)output_count(mode, P.n, P.n);
      // rows per item: 32 q with at least a few items per problem
      uint64_t qb = 1;
      while (qb < 16 && 32ull * qb * 4 <= P.n) qb *= 2;
      pend.push_back({d, pairs * 2.0 * meanL, qb});
      b->total_pairs += (uint64_t)pairs;
      pbase += P.n;
      ebase += o[P.n];
    }
    if (tot_n) SBG_CUDA(cudaMemcpy(b->d_perm.get(), hperm.data(), tot_n * sizeof(uint32_t), cudaMemcpyHostToDevice));
    std::stable_sort(pend.begin(), pend.end(), [](const Pending& a, const Pending& c) { return a.cost > c.cost; });
    for (auto& x : pend)
    {
      b->descs.push_back(x.d);
      b->q_base.push_back(x.qb);
    }

    // One plan for the whole batch: the time-windowed kernel on the CSR
    // (windows only where PCFs are long), or on request the hybrid kernel
    // (columns in shared memory when a group fits, rows through L1) on the
    // packed layout.
    Plan pl;
    const size_t es = sizeof(Elem<T>);
    b->usable = b->dev.smem_optin > 2048 ? b->dev.smem_optin - 2048 : 0;
    b->lmax = lmax;
    const int want_w = settings().warps.load();
    pl.smem = true;
    pl.q = 1;
    pl.grid = b->dev.sms;
    if (b->windowed)
    {
      pl.packed = false;
      pl.kvar = 6;
      pl.warps = want_w > 0 ? std::min(want_w, 32) : 24;
      // One cap for every shape the autotune tries (up to 32 warps and 4x
      // the rows per item), else the one that fits the starting shape.
      uint64_t qb = 1;
      for (uint64_t x : b->q_base) qb = std::max(qb, x);
      Plan probe;
      if (window_layout(probe, es, 32, (uint32_t)(32 * qb * 4), lmax, b->usable))
        b->win_cap = probe.lmax_c;
      else if (window_layout(probe, es, pl.warps, (uint32_t)(32 * qb), lmax, b->usable))
        b->win_cap = probe.lmax_c;
    }
    else
    {
      pl.packed = true;
      pl.kvar = 3;
      pl.warps = want_w > 0 ? std::min(want_w, 32) : 32;
      pl.lmax_c = (uint32_t)std::min<size_t>(lmax, b->usable / (32 * es));
      pl.row_cap = 0;
      pl.smem_bytes = (size_t)32 * pl.lmax_c * es;
    }
    b->pl = pl;
    b->d_descs.reset(std::max<size_t>(1, b->descs.size()) * sizeof(ProblemDesc<T>));
    b->d_queue.reset(256);
    SBG_CUDA(cudaDeviceSynchronize());
    bool fit = false;
    for (int w = pl.warps; w >= 4 && !fit; w -= 4) fit = b->rebuild_items((uint32_t)w, 1);
    if (!fit) throw Error(ST_INVALID_ARGUMENT, "batch: the window setting does not fit in shared memory");
    return b.release();
  }
}

struct sbg_batch
{
  std::unique_ptr<sbg::BatchBase> impl;
};

namespace
{
  template <typename F>
  int guarded_batch(F&& f)
  {
    try
    {
      f();
      sbg::set_last_error("");
      return SBG_OK;
    }
    catch (const sbg::Error& e)
    {
      sbg::set_last_error(e.what());
      return e.status;
    }
    catch (const std::exception& e)
    {
      sbg::set_last_error(e.what());
      return SBG_ERR_INTERNAL;
    }
  }
}

extern "C"
{
  int sbg_batch_create(int dtype, int op, double p, int skip_mode, const sbg_problem* problems, uint64_t n_problems,
                       int flags, sbg_batch** batch)
  {
    return guarded_batch([&] {
      using namespace sbg;
      if (!batch) throw Error(ST_INVALID_ARGUMENT, "null batch pointer");
      *batch = nullptr;
      if (dtype != SBG_F32 && dtype != SBG_F64) throw Error(ST_INVALID_ARGUMENT, "dtype must be SBG_F32 or SBG_F64");
      if (op != SBG_OP_L1 && op != SBG_OP_LP && op != SBG_OP_L2_INNER) throw Error(ST_INVALID_ARGUMENT, "unknown op");
      if (op == SBG_OP_LP && !(p >= 1.0)) throw Error(ST_INVALID_ARGUMENT, "p must be >= 1.");
      if (skip_mode != SBG_SKIP_LOWER_NODIAG && skip_mode != SBG_SKIP_LOWER)
        throw Error(ST_INVALID_ARGUMENT, "batches hold pdist (SBG_SKIP_LOWER_NODIAG) or kernel (SBG_SKIP_LOWER) problems");
      if (n_problems > 0 && !problems) throw Error(ST_INVALID_ARGUMENT, "null problem array");
      std::unique_ptr<sbg_batch> b(new sbg_batch);
      if (dtype == SBG_F32) b->impl.reset(make_batch<float>(op, p, skip_mode, problems, n_problems, flags));
      else b->impl.reset(make_batch<double>(op, p, skip_mode, problems, n_problems, flags));
      *batch = b.release();
    });
  }

  int sbg_batch_launch(sbg_batch* batch, void* stream)
  {
    return guarded_batch([&] {
      if (!batch) throw sbg::Error(sbg::ST_INVALID_ARGUMENT, "null batch");
      batch->impl->launch(static_cast<cudaStream_t>(stream));
    });
  }

  int sbg_batch_autotune(sbg_batch* batch, void* stream, double* best_ms)
  {
    return guarded_batch([&] {
      if (!batch) throw sbg::Error(sbg::ST_INVALID_ARGUMENT, "null batch");
      const double ms = batch->impl->autotune(static_cast<cudaStream_t>(stream));
      if (best_ms) *best_ms = ms;
    });
  }

  int sbg_batch_info(const sbg_batch* batch, uint64_t* items, uint64_t* pairs, int* warps, int* rows_per_item)
  {
    return guarded_batch([&] {
      if (!batch) throw sbg::Error(sbg::ST_INVALID_ARGUMENT, "null batch");
      batch->impl->info(items, pairs, warps, rows_per_item);
    });
  }

  int sbg_batch_shared_split(const sbg_batch* batch, uint32_t* column_elements)
  {
    return guarded_batch([&] {
      if (!batch || !column_elements) throw sbg::Error(sbg::ST_INVALID_ARGUMENT, "null pointer");
      *column_elements = batch->impl->shared_split();
    });
  }

  void sbg_batch_destroy(sbg_batch* batch)
  {
    delete batch;
  }
}
