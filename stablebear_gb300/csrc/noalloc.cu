// Pairwise integration for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc (or any allocator) at the point where
// they need a distance or kernel matrix: an application that hands all device
// memory to its own pool up front and forbids other allocations, code that
// runs while another component is recording a CUDA graph and must not add
// allocation nodes or implicit synchronisation, or a plugin host that owns
// every device buffer and only lends the plugin its inputs and outputs.
// sbg_pairwise_device allocates a few bytes of stream-ordered scratch (the
// persistent kernel's work-queue counter, and for PCFs too long for shared
// memory a packed copy of the breakpoints).  This entry point takes that
// scratch from a fixed array compiled into the library instead.
#include "../../include/sbgpu.h"
#include "sbg_internal.hpp"

#include <cuda.h>  // CUcontext / CUresult types; the two driver calls are looked up through the runtime

#include <mutex>

namespace sbg
{
  namespace
  {
    // The scratch every call of sbg_pairwise_device_noalloc uses.  It exists
    // once per device for as long as the library stays loaded.  Layout: the
    // 8-byte work-queue counter in the first 256 bytes, then (only for PCFs
    // too long for the shared-memory kernel) the packed breakpoints.
    __device__ __align__(256) unsigned char g_noalloc_scratch[SBG_NOALLOC_SCRATCH_BYTES];

    constexpr int kMaxDevices = 64;
    std::mutex g_setup_mu;
    struct ScratchAddr
    {
      void* ptr = nullptr;
      unsigned long long context = 0;  // id of the CUDA context the address belongs to
    };
    ScratchAddr g_scratch_addr[kMaxDevices];

    using CtxGetCurrentFn = CUresult (*)(CUcontext*);
    using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

    // Unique id of the calling thread's current CUDA context (cuCtxGetId), 0
    // when none is current yet.  A device reset makes a new context with a
    // new id, and the library module (with the array) is loaded anew in it.
    unsigned long long current_context_id()
    {
      static CtxGetCurrentFn get_current = nullptr;
      static CtxGetIdFn get_id = nullptr;
      static std::once_flag once;
      std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
          get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
        fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
          get_id = reinterpret_cast<CtxGetIdFn>(fn);
        cudaGetLastError();
      });
      if (!get_current || !get_id) throw Error(ST_CUDA, "cuCtxGetCurrent / cuCtxGetId not available from the driver");
      CUcontext ctx = nullptr;
      if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
      unsigned long long id = 0;
      if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
      return id;
    }

    // Device address of g_noalloc_scratch in the current device's context.
    // Host code only has a stand-in for the array, so the address is looked
    // up with cudaGetSymbolAddress, with the device current, the first time a
    // context is seen (once per device, again after a device reset), and
    // cached under the context's id.
    void* scratch_for_current_device()
    {
      int dev = 0;
      SBG_CUDA(cudaGetDevice(&dev));
      if (dev < 0 || dev >= kMaxDevices) throw Error(ST_INVALID_ARGUMENT, "device index out of range");
      std::lock_guard<std::mutex> lock(g_setup_mu);
      ScratchAddr& s = g_scratch_addr[dev];
      const unsigned long long ctx = current_context_id();
      if (!s.ptr || ctx == 0 || ctx != s.context)
      {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // also makes the primary context current
        if (e != cudaSuccess || !p)
        {
          cudaGetLastError();
          throw Error(ST_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch) failed: ") + cudaGetErrorString(e));
        }
        s.ptr = p;
        s.context = current_context_id();
      }
      return s.ptr;
    }
  }
}

extern "C" int sbg_pairwise_device_noalloc(int dtype, int op, double p, int skip_mode, const void* row_points,
                                           const uint64_t* row_offsets, uint64_t n_rows, uint64_t n_row_points,
                                           const void* col_points, const uint64_t* col_offsets, uint64_t n_cols,
                                           uint64_t n_col_points, const uint32_t* row_perm, const uint32_t* col_perm,
                                           uint32_t max_points, void* out, uint64_t out_base, uint64_t row_begin,
                                           uint64_t row_end, void* stream)
{
  using namespace sbg;
  try
  {
    if (dtype != SBG_F32 && dtype != SBG_F64) throw Error(ST_INVALID_ARGUMENT, "dtype must be SBG_F32 or SBG_F64");
    if (op != SBG_OP_L1 && op != SBG_OP_LP && op != SBG_OP_L2_INNER) throw Error(ST_INVALID_ARGUMENT, "unknown op");
    if (op == SBG_OP_LP && !(p >= 1.0)) throw Error(ST_INVALID_ARGUMENT, "p must be >= 1.");
    if (skip_mode != SBG_SKIP_NONE && skip_mode != SBG_SKIP_LOWER_NODIAG && skip_mode != SBG_SKIP_LOWER)
      throw Error(ST_INVALID_ARGUMENT, "unknown skip mode");
    if (n_rows > 0 && (!row_points || !row_offsets)) throw Error(ST_INVALID_ARGUMENT, "null row points/offsets");
    if (skip_mode == SBG_SKIP_NONE && n_cols > 0 && (!col_points || !col_offsets))
      throw Error(ST_INVALID_ARGUMENT, "null column points/offsets");
    if (output_count(skip_mode, n_rows, n_cols) > 0 && !out) throw Error(ST_INVALID_ARGUMENT, "null output");
    if (max_points == 0)
      throw Error(ST_INVALID_ARGUMENT, "max_points must be given to the no-allocation entry point");
    void* scratch = scratch_for_current_device();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == SBG_F32)
    {
      PcfSet<float> r{static_cast<const float*>(row_points), row_offsets, n_rows};
      PcfSet<float> c{static_cast<const float*>(col_points), col_offsets, n_cols};
      compute_device_scratch<float>(skip_mode, op, p, r, skip_mode == SBG_SKIP_NONE ? &c : nullptr, row_perm,
                                    col_perm, max_points, n_row_points, n_col_points, static_cast<float*>(out),
                                    out_base, row_begin, row_end, scratch, SBG_NOALLOC_SCRATCH_BYTES, st);
    }
    else
    {
      PcfSet<double> r{static_cast<const double*>(row_points), row_offsets, n_rows};
      PcfSet<double> c{static_cast<const double*>(col_points), col_offsets, n_cols};
      compute_device_scratch<double>(skip_mode, op, p, r, skip_mode == SBG_SKIP_NONE ? &c : nullptr, row_perm,
                                     col_perm, max_points, n_row_points, n_col_points, static_cast<double*>(out),
                                     out_base, row_begin, row_end, scratch, SBG_NOALLOC_SCRATCH_BYTES, st);
    }
    set_last_error("");
    return SBG_OK;
  }
  catch (const Error& e)
  {
    set_last_error(std::string("sbg_pairwise_device_noalloc: ") + e.what());
    return e.status;
  }
  catch (const std::exception& e)
  {
    set_last_error(std::string("sbg_pairwise_device_noalloc: ") + e.what());
    return SBG_ERR_INTERNAL;
  }
}
