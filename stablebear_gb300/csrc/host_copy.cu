// Device -> host result transfer for the band pipeline.
//
// A D2H cudaMemcpy into pageable memory is staged by the driver through one
// CPU thread (~10 GB/s on the Grace host), which would make the host-facing
// path slower than the kernel.  Instead each band is copied in chunks into
// two pinned staging buffers over NVLink-C2C, and a pool of host threads
// moves each chunk into the caller's matrix while the next chunk (and the
// next band's kernel) is in flight.
#include "host_copy.hpp"

#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <unistd.h>
#include <vector>

namespace sbg
{
  namespace
  {
    // Fixed pool of host threads.  run() splits one job into parts, one per
    // thread plus the caller, and returns when every part is done.  The pool
    // lives until the process ends and is never joined: a child forked after
    // the threads started has none of them, and joining them there (at exit)
    // would wait forever.
    class CopyPool
    {
    public:
      static CopyPool& get()
      {
        static CopyPool* pool = new CopyPool();
        return *pool;
      }

      unsigned parts() const { return (unsigned)m_threads.size() + 1; }

      // job(part) for part in [0, parts()); the caller runs the last part.
      void run(const std::function<void(unsigned)>& job)
      {
        if (m_threads.empty() || getpid() != m_pid)
        {
          // no pool threads, or a child forked after they started (it has
          // none of them): every part on the calling thread
          for (unsigned k = 0; k < parts(); ++k) job(k);
          return;
        }
        std::unique_lock<std::mutex> call(m_call);  // one job at a time
        {
          std::lock_guard<std::mutex> lk(m_mu);
          m_job = &job;
          m_pending = m_threads.size();
          ++m_gen;
        }
        m_cv.notify_all();
        job((unsigned)m_threads.size());
        std::unique_lock<std::mutex> lk(m_mu);
        m_done.wait(lk, [this] { return m_pending == 0; });
        m_job = nullptr;
      }

      void copy(void* dst, const void* src, size_t bytes)
      {
        const size_t nt = parts();
        if (bytes < (8u << 20) || nt == 1)
        {
          std::memcpy(dst, src, bytes);
          return;
        }
        const size_t part = ((bytes / nt) + 4095) & ~size_t(4095);
        run([&](unsigned k) {
          const size_t off = part * k;
          if (off < bytes)
            std::memcpy(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, std::min(part, bytes - off));
        });
      }

    private:
      CopyPool() : m_pid(getpid())
      {
        unsigned hc = std::thread::hardware_concurrency();
        unsigned n = hc > 1 ? std::min(hc, 32u) - 1 : 0;
        for (unsigned i = 0; i < n; ++i) m_threads.emplace_back([this, i] { work(i); });
      }
      void work(unsigned idx)
      {
        uint64_t seen = 0;
        for (;;)
        {
          const std::function<void(unsigned)>* job;
          {
            std::unique_lock<std::mutex> lk(m_mu);
            m_cv.wait(lk, [&] { return m_gen != seen; });
            seen = m_gen;
            job = m_job;
          }
          (*job)(idx);
          {
            std::lock_guard<std::mutex> lk(m_mu);
            if (--m_pending == 0) m_done.notify_all();
          }
        }
      }

      std::vector<std::thread> m_threads;
      std::mutex m_mu, m_call;
      std::condition_variable m_cv, m_done;
      const std::function<void(unsigned)>* m_job = nullptr;
      size_t m_pending = 0;
      uint64_t m_gen = 0;
      pid_t m_pid;
    };

    // Process-wide pinned staging buffers (allocated on first use, reused).
    struct StagingPool
    {
      std::mutex mu;
      bool busy = false;
      void* buf[2] = {nullptr, nullptr};
      size_t bytes = 0;
    };
    StagingPool& staging_pool()
    {
      static StagingPool p;
      return p;
    }
  }

  HostStager::HostStager(size_t chunk_bytes) : m_chunk(chunk_bytes)
  {
    StagingPool& p = staging_pool();
    std::lock_guard<std::mutex> lk(p.mu);
    if (!p.busy)
    {
      if (p.bytes < chunk_bytes)
      {
        for (void*& b : p.buf)
          if (b) { cudaFreeHost(b); b = nullptr; }
        p.bytes = 0;
        for (void*& b : p.buf) SBG_CUDA(cudaHostAlloc(&b, chunk_bytes, cudaHostAllocDefault));
        p.bytes = chunk_bytes;
      }
      p.busy = true;
      m_shared = true;
      m_buf[0] = p.buf[0];
      m_buf[1] = p.buf[1];
    }
    else
    {
      for (void*& b : m_buf) SBG_CUDA(cudaHostAlloc(&b, chunk_bytes, cudaHostAllocDefault));
    }
    for (auto& e : m_ev) SBG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }

  HostStager::~HostStager()
  {
    try { flush(); } catch (...) { }
    for (auto& e : m_ev) if (e) cudaEventDestroy(e);
    if (m_shared)
    {
      StagingPool& p = staging_pool();
      std::lock_guard<std::mutex> lk(p.mu);
      p.busy = false;
    }
    else
    {
      for (void* b : m_buf) if (b) cudaFreeHost(b);
    }
  }

  void HostStager::finish_pending()
  {
    if (!m_has_pending) return;
    SBG_CUDA(cudaEventSynchronize(m_ev[m_pending_slot]));
    CopyPool::get().copy(m_pending_dst, m_buf[m_pending_slot], m_pending_bytes);
    m_has_pending = false;
  }

  void HostStager::copy(void* host_dst, const void* dev_src, size_t bytes, cudaStream_t st)
  {
    char* dst = static_cast<char*>(host_dst);
    const char* src = static_cast<const char*>(dev_src);
    while (bytes > 0)
    {
      const size_t n = std::min(bytes, m_chunk);
      const int slot = m_next;
      // the slot's previous chunk was consumed by finish_pending() below at
      // the latest one iteration ago
      SBG_CUDA(cudaMemcpyAsync(m_buf[slot], src, n, cudaMemcpyDeviceToHost, st));
      SBG_CUDA(cudaEventRecord(m_ev[slot], st));
      finish_pending();
      m_has_pending = true;
      m_pending_slot = slot;
      m_pending_dst = dst;
      m_pending_bytes = n;
      m_next ^= 1;
      dst += n;
      src += n;
      bytes -= n;
    }
  }

  void HostStager::flush() { finish_pending(); }

  unsigned host_parts() { return CopyPool::get().parts(); }

  void host_parallel(const std::function<void(unsigned)>& job) { CopyPool::get().run(job); }

  namespace
  {
    // Two pinned buffers and two events for uploads, allocated on first use
    // and reused; one pool per device, because an event can only be recorded
    // on a stream of the device it was created on.
    struct UploadPool
    {
      static constexpr size_t CHUNK = 32u << 20;
      std::mutex mu;
      void* buf[2] = {nullptr, nullptr};
      cudaEvent_t ev[2] = {nullptr, nullptr};
    };
    constexpr int kUploadDevices = 64;
    UploadPool& upload_pool(int dev)
    {
      static UploadPool pools[kUploadDevices];
      return pools[dev];
    }
  }

  void upload_pageable(void* dev_dst, const void* host_src, size_t bytes, cudaStream_t st)
  {
    int dev = 0;
    SBG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kUploadDevices)
    {
      SBG_CUDA(cudaMemcpyAsync(dev_dst, host_src, bytes, cudaMemcpyHostToDevice, st));
      return;
    }
    UploadPool& p = upload_pool(dev);
    std::unique_lock<std::mutex> lk(p.mu, std::try_to_lock);
    if (bytes < (16u << 20) || !lk.owns_lock())
    {
      // small, or another thread holds the buffers: the driver's own path
      SBG_CUDA(cudaMemcpyAsync(dev_dst, host_src, bytes, cudaMemcpyHostToDevice, st));
      return;
    }
    // each piece on its own, so a failed allocation leaves nothing half made
    for (int k = 0; k < 2; ++k)
    {
      if (!p.ev[k]) SBG_CUDA(cudaEventCreateWithFlags(&p.ev[k], cudaEventDisableTiming));
      if (!p.buf[k]) SBG_CUDA(cudaHostAlloc(&p.buf[k], UploadPool::CHUNK, cudaHostAllocDefault));
    }
    char* dst = static_cast<char*>(dev_dst);
    const char* src = static_cast<const char*>(host_src);
    int slot = 0;
    while (bytes > 0)
    {
      const size_t n = std::min(bytes, UploadPool::CHUNK);
      // the slot's previous DMA has read the buffer
      SBG_CUDA(cudaEventSynchronize(p.ev[slot]));
      CopyPool::get().copy(p.buf[slot], src, n);
      SBG_CUDA(cudaMemcpyAsync(dst, p.buf[slot], n, cudaMemcpyHostToDevice, st));
      SBG_CUDA(cudaEventRecord(p.ev[slot], st));
      slot ^= 1;
      dst += n;
      src += n;
      bytes -= n;
    }
    // the buffers are reused by the next upload: wait for the last DMAs
    SBG_CUDA(cudaEventSynchronize(p.ev[0]));
    SBG_CUDA(cudaEventSynchronize(p.ev[1]));
  }

  void host_memory_access(int* pageable, int* host_page_tables)
  {
    int dev = 0;
    SBG_CUDA(cudaGetDevice(&dev));
    int a = 0, b = 0;
    SBG_CUDA(cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev));
    SBG_CUDA(cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
    if (pageable) *pageable = a;
    if (host_page_tables) *host_page_tables = b;
  }
}
