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
#include <mutex>
#include <thread>
#include <vector>

namespace sbg
{
  namespace
  {
    // Fixed pool of copy threads; parallel_copy splits one memcpy over them.
    class CopyPool
    {
    public:
      static CopyPool& get()
      {
        static CopyPool pool;
        return pool;
      }

      void copy(void* dst, const void* src, size_t bytes)
      {
        const size_t nt = m_threads.size() + 1;
        if (bytes < (8u << 20) || nt == 1)
        {
          std::memcpy(dst, src, bytes);
          return;
        }
        std::unique_lock<std::mutex> call(m_call);  // one parallel copy at a time
        const size_t part = ((bytes / nt) + 4095) & ~size_t(4095);
        {
          std::lock_guard<std::mutex> lk(m_mu);
          m_dst = static_cast<char*>(dst);
          m_src = static_cast<const char*>(src);
          m_bytes = bytes;
          m_part = part;
          m_pending = m_threads.size();
          ++m_gen;
        }
        m_cv.notify_all();
        // the calling thread takes the last part
        const size_t off = part * m_threads.size();
        if (off < bytes) std::memcpy(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, bytes - off);
        std::unique_lock<std::mutex> lk(m_mu);
        m_done.wait(lk, [this] { return m_pending == 0; });
      }

    private:
      CopyPool()
      {
        unsigned hc = std::thread::hardware_concurrency();
        unsigned n = hc > 1 ? std::min(hc, 32u) - 1 : 0;
        for (unsigned i = 0; i < n; ++i) m_threads.emplace_back([this, i] { run(i); });
      }
      ~CopyPool()
      {
        {
          std::lock_guard<std::mutex> lk(m_mu);
          m_quit = true;
          ++m_gen;
        }
        m_cv.notify_all();
        for (auto& t : m_threads) t.join();
      }

      void run(unsigned idx)
      {
        uint64_t seen = 0;
        for (;;)
        {
          char* dst;
          const char* src;
          size_t bytes, part;
          {
            std::unique_lock<std::mutex> lk(m_mu);
            m_cv.wait(lk, [&] { return m_gen != seen; });
            seen = m_gen;
            if (m_quit) return;
            dst = m_dst; src = m_src; bytes = m_bytes; part = m_part;
          }
          const size_t off = part * idx;
          if (off < bytes) std::memcpy(dst + off, src + off, std::min(part, bytes - off));
          {
            std::lock_guard<std::mutex> lk(m_mu);
            if (--m_pending == 0) m_done.notify_all();
          }
        }
      }

      std::vector<std::thread> m_threads;
      std::mutex m_mu, m_call;
      std::condition_variable m_cv, m_done;
      char* m_dst = nullptr;
      const char* m_src = nullptr;
      size_t m_bytes = 0, m_part = 0, m_pending = 0;
      uint64_t m_gen = 0;
      bool m_quit = false;
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
