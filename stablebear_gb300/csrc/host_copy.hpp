// Chunked device -> pinned -> pageable host transfer (host_copy.cu).
#pragma once

#include "sbg_internal.hpp"

#include <functional>

namespace sbg
{
  class HostStager
  {
  public:
    explicit HostStager(size_t chunk_bytes);
    ~HostStager();
    HostStager(const HostStager&) = delete;
    HostStager& operator=(const HostStager&) = delete;

    // Enqueue dev_src -> host_dst (bytes) on stream st.  Returns once every
    // chunk but the last has landed in host_dst; flush() finishes the last.
    void copy(void* host_dst, const void* dev_src, size_t bytes, cudaStream_t st);
    void flush();

  private:
    void finish_pending();

    size_t m_chunk;
    void* m_buf[2] = {nullptr, nullptr};
    cudaEvent_t m_ev[2] = {nullptr, nullptr};
    bool m_shared = false;
    int m_next = 0;
    bool m_has_pending = false;
    int m_pending_slot = 0;
    void* m_pending_dst = nullptr;
    size_t m_pending_bytes = 0;
  };

  // Host -> device copy from pageable host memory (16 MB and up): chunks
  // are copied by the host thread pool into two pinned buffers while the
  // previous chunk's DMA runs.  Returns when the data is on the device.
  void upload_pageable(void* dev_dst, const void* host_src, size_t bytes, cudaStream_t st);

  // The host thread pool: host_parallel(job) runs job(part) for every part
  // in [0, host_parts()) and returns when all are done.
  unsigned host_parts();
  void host_parallel(const std::function<void(unsigned)>& job);

  // cudaDevAttrPageableMemoryAccess / ...UsesHostPageTables of the current
  // device: 1/1 on coherent hosts (Grace + NVLink-C2C) where kernels may
  // store straight into malloc'd host memory.
  void host_memory_access(int* pageable, int* host_page_tables);
}
