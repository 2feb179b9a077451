/*
 * sbgpu.h — C ABI of the GB300 pairwise-integration engine for arrays of
 * piecewise constant functions (PCFs): Lp distance matrices (pdist / cdist,
 * p >= 1) and L2 kernel (Gram) matrices.
 *
 * Plain C: pointers, sizes and status codes; no exceptions cross it.  Every
 * entry point returns SBG_OK (0) or a negative sbg_status; sbg_last_error()
 * then holds a message for the calling thread.
 *
 * Input layout (all entry points): the reference's CSR of SimplePoint
 * (include/sbear/cuda/offset_data_manager.hpp:42-68,
 *  include/sbear/cuda/cuda_matrix_integrate_structs.cuh:9-14):
 *   points  — interleaved (t, v) pairs of the element type, PCF i at
 *             points[2*offsets[i] .. 2*offsets[i+1])
 *   offsets — n + 1 uint64 values, offsets[0] == 0.
 * Each PCF starts at t = 0 with non-decreasing, finite times
 * (src/python/pypcf_support.hpp:76-89); host entry points check this.
 *
 * Output layouts are the reference's:
 *   DistanceMatrix (pdist):  n(n-1)/2 values, (i, j), i > j at i(i-1)/2 + j
 *                            (include/sbear/distance_matrix.hpp:141-146)
 *   SymmetricMatrix (kernel): n(n+1)/2 values, (i, j), i >= j at i(i+1)/2 + j
 *                            (include/sbear/symmetric_matrix.hpp:248-260)
 *   dense (cdist):           n_rows x n_cols row-major
 *                            (include/sbear/cuda/cuda_result_writer.hpp:17-34)
 */
#ifndef SBGPU_H
#define SBGPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define SBG_API_VERSION 1

typedef enum sbg_status {
  SBG_OK = 0,
  SBG_ERR_INVALID_ARGUMENT = -1,
  SBG_ERR_INVALID_INPUT = -2,   /* input violates the PCF contract */
  SBG_ERR_CUDA = -3,            /* "file:line: <cuda message>" (cuda_util.cuh:8-10) */
  SBG_ERR_OUT_OF_MEMORY = -4,
  SBG_ERR_CANCELLED = -5,       /* request_stop() ended the task */
  SBG_ERR_NO_DEVICE = -6,
  SBG_ERR_TIMEOUT = -7,
  SBG_ERR_INTERNAL = -8,
  SBG_ERR_LOGIC = -9            /* logic_error (cuda_result_writer.hpp:63-90) */
} sbg_status;

typedef enum sbg_dtype { SBG_F32 = 0, SBG_F64 = 1, SBG_I32 = 2, SBG_I64 = 3 } sbg_dtype;
/* (SBG_I32 / SBG_I64: integer-valued PCFs, taken by sbg_iterate_rectangles only) */

/* Pair operations (include/sbear/functional/operations.cuh:19-65). */
typedef enum sbg_op { SBG_OP_L1 = 0, SBG_OP_LP = 1, SBG_OP_L2_INNER = 2 } sbg_op;

/* Which pairs / which layout; values equal the reference's TriangleSkipMode
 * (include/sbear/cuda/triangle_skip_mode.hpp:7-12). */
typedef enum sbg_skip_mode {
  SBG_SKIP_NONE = 0,           /* cdist: all pairs, dense row-major */
  SBG_SKIP_LOWER_NODIAG = 1,   /* pdist: i > j, DistanceMatrix order */
  SBG_SKIP_LOWER = 2           /* l2 kernel: i >= j, SymmetricMatrix order */
} sbg_skip_mode;

/* ---- library --------------------------------------------------------------- */

int sbg_api_version(void);
/* Message of the last failing call on this thread ("" if none). */
const char* sbg_last_error(void);
/* "CUDA" — the library has no CPU path (pymodule.cpp: _build_type). */
const char* sbg_build_type(void);
/* Number of visible CUDA devices (pymodule.cpp: get_ngpus). */
int sbg_get_ngpus(int* n);

/* ---- settings: sb::Settings (include/sbear/settings.hpp:8-23) and the
 *      setters bound in src/python/pymodule.cpp:136-151 ------------------------ */

int sbg_set_force_cpu(int on);            /* accepted; the library always runs on the GPU */
int sbg_get_force_cpu(void);
int sbg_set_cuda_threshold(uint64_t n);   /* accepted; no CPU path to fall back to */
uint64_t sbg_get_cuda_threshold(void);
int sbg_set_block_dim(unsigned x, unsigned y);
int sbg_set_min_block_side(uint64_t n);
int sbg_limit_gpus(int n);
int sbg_limit_cpus(int n);
int sbg_set_device_verbose(int on);
int sbg_get_device_verbose(void);
/* Engine knobs (0 = automatic): warps per CTA, rows per work item / 32,
 * variant (1 shared-memory with 8-byte row elements, 2 global-memory, 3
 * shared-memory with a two-load walk, 4 hybrid: columns in shared memory,
 * rows read through L1, 5 shared-memory with the row as separate time and
 * value arrays, the automatic choice when the PCFs fit, 6 time-windowed
 * shared memory: each work item walks time windows holding at most a cap of
 * elements of every PCF, the automatic choice for longer PCFs; 7 and 8,
 * float32 only and never automatic, kept to measure two other designs: 7
 * one unified shared-memory load per step from a row replicated 16 times, 8
 * merge path with one pair per warp), order
 * (1 caller's, 2 sorted
 * by breakpoint count), output bytes per pipeline band (automatic: 1/8 of
 * the output, the last eighth cut into halving parts so that little of the
 * copy-out runs after the last kernel). */
int sbg_set_tuning(int warps, int row_chunk, int variant, int order, uint64_t band_bytes);

/* Time-windowed variant: the most elements of one PCF inside a window
 * (0 = the most that fit in shared memory).  SBG_ERR_INVALID_ARGUMENT
 * outside [0, 1048576]; a cap too large for shared memory fails the call
 * that plans with it. */
int sbg_set_window_cap(int cap);
int sbg_get_window_cap(void);

/* How host-buffer entry points return results: 0 automatic (= 1), 1 device
 * bands copied out through pinned staging buffers while the next band
 * computes, 2 the kernel stores straight into the caller's host buffer
 * (only on devices that use the host page tables, e.g. Grace + NVLink-C2C;
 * SBG_ERR_INVALID_ARGUMENT elsewhere). */
int sbg_set_output_mode(int mode);
/* cudaDevAttrPageableMemoryAccess and ...UsesHostPageTables of the current
 * device (both 1 where output mode 2 is available). */
int sbg_host_memory_access(int* pageable, int* uses_host_page_tables);

/* ---- tasks: the 12 factories of include/sbear/cuda/cuda_matrix_integrate_api.hpp:19-113
 *      and StoppableTask (include/sbear/task.hpp:15-172) ------------------------ */

typedef struct sbg_task sbg_task;

/* pdist (skip_mode SBG_SKIP_LOWER_NODIAG, out = DistanceMatrix storage) or
 * l2 kernel (SBG_SKIP_LOWER, out = SymmetricMatrix storage) of one PCF set.
 * Replaces create_cuda_block_integrate_{l1,lp,l2_kernel}_task
 * (cuda_matrix_integrate_api.hpp:19-63).  The PCFs are copied into the task
 * (as pcf_block_op.cuh:143 copies them); `out` is caller-owned host memory
 * that must outlive the task.  op SBG_OP_LP takes p >= 1. */
int sbg_create_integrate_task(int dtype, int op, double p, int skip_mode,
                              const void* points, const uint64_t* offsets, uint64_t n,
                              void* out, sbg_task** task);

/* cdist between two PCF sets into a dense n_rows x n_cols host matrix.
 * Replaces create_cuda_block_cdist_{l1,lp,l2_kernel}_task
 * (cuda_matrix_integrate_api.hpp:67-113). */
int sbg_create_cdist_task(int dtype, int op, double p,
                          const void* row_points, const uint64_t* row_offsets, uint64_t n_rows,
                          const void* col_points, const uint64_t* col_offsets, uint64_t n_cols,
                          void* out, sbg_task** task);

/* StoppableTask::start_async (task.hpp:43-49): runs on a worker thread. */
int sbg_task_start(sbg_task* task);
/* StoppableTask::wait_for (task.hpp:84-96): *finished = 0 while running,
 * 1 once done; the worker's error status is returned once, on the call that
 * observes completion. */
int sbg_task_wait_for(sbg_task* task, int64_t timeout_ms, int* finished);
/* StoppableTask::wait (task.hpp:98-107). */
int sbg_task_wait(sbg_task* task);
/* StoppableTask::request_stop / stop_requested (task.hpp:21-31). */
int sbg_task_request_stop(sbg_task* task);
int sbg_task_stop_requested(const sbg_task* task);
/* work_total / work_completed / work_step (task.hpp:51-64). */
int sbg_task_progress(const sbg_task* task, uint64_t* work_total, uint64_t* work_completed, uint64_t* work_step);
/* work_step_desc / work_step_unit (task.hpp:66-76), NUL-terminated into buf. */
int sbg_task_step_text(const sbg_task* task, char* desc, size_t desc_cap, char* unit, size_t unit_cap);
/* Waits for a running task, then frees it. */
void sbg_task_destroy(sbg_task* task);

/* ---- synchronous host-buffer entry (blocking; what the task runs) --------- */

/* skip_mode as above; col_* ignored unless skip_mode == SBG_SKIP_NONE.
 * validate != 0 checks the input contract first. */
int sbg_pairwise_host(int dtype, int op, double p, int skip_mode,
                      const void* row_points, const uint64_t* row_offsets, uint64_t n_rows,
                      const void* col_points, const uint64_t* col_offsets, uint64_t n_cols,
                      void* out, int validate);

/* ---- stream-ordered device entry --------------------------------------------
 * All pointers are device pointers on the current device; work is enqueued on
 * `stream` (a cudaStream_t, NULL = legacy default stream).  out_base is
 * subtracted from every output index (a caller writing rows
 * [row_begin, row_end) of a condensed matrix into a band buffer passes the
 * band's first index); row_end = 0 means all rows.  max_points is the largest
 * breakpoint count over rows and columns (0: measured on the device, which
 * synchronises the stream).  row_perm / col_perm (optional, uint32) give the
 * processing order; results always land at the callers' (i, j).  Inputs are
 * not validated; malformed times cannot make the kernel read out of bounds. */
int sbg_pairwise_device(int dtype, int op, double p, int skip_mode,
                        const void* row_points, const uint64_t* row_offsets, uint64_t n_rows,
                        const void* col_points, const uint64_t* col_offsets, uint64_t n_cols,
                        const uint32_t* row_perm, const uint32_t* col_perm, uint32_t max_points,
                        void* out, uint64_t out_base, uint64_t row_begin, uint64_t row_end,
                        void* stream);

/* The persistent kernel's work items for rows [row_begin, row_end) of a
 * problem with 32*q rows per item: writes (chunk, column group) pairs for
 * item ids 0.. into out (2*cap uint64) and returns the item count.  Host-only
 * (no device needed); used by tests and tooling to check that the items tile
 * the requested triangle or rectangle exactly once. */
uint64_t sbg_enumerate_items(int skip_mode, uint64_t n_rows, uint64_t n_cols, uint64_t row_begin,
                             uint64_t row_end, uint32_t q, uint64_t* out, uint64_t cap);

/* Measured issue rate of the current device for the roofline: kind 0 =
 * FP32 FFMA, 1 = FP64 DFMA, in lane-operations per second (one FMA
 * instruction per lane = one lane-op), from a register-only FMA loop. */
int sbg_measure_peak(int kind, double* lane_ops_per_s);

/* ---- gradients --------------------------------------------------------------------
 * No counterpart in the reference (it has no gradients).  Given grad_out =
 * dL/dM for the condensed output M of a pdist (L2: op SBG_OP_LP with p = 2, or
 * L1) or L2 kernel problem, writes dL/d(points) into grad_points, laid out
 * like the points: (n_points, 2) pairs [dL/dt, dL/dv].  forward_out is the
 * forward result M (needed for the L2 distance, optional otherwise).  The
 * merge is recomputed.  Times that coincide with a breakpoint of the other
 * PCF of a pair (ties) and each PCF's first time t = 0 get no gradient from
 * that pair.  Accumulation uses atomic adds (order not deterministic).
 * Device pointers, stream-ordered; grad_points is overwritten. */
int sbg_pairwise_backward_device(int dtype, int op, double p, int skip_mode,
                                 const void* points, const uint64_t* offsets, uint64_t n, uint64_t n_points,
                                 uint32_t max_points, const void* grad_out, const void* forward_out,
                                 void* grad_points, void* stream);

/* ---- the rectangles of one pair --------------------------------------------------
 * Replaces sb::iterate_rectangles (include/sbear/algorithms/functional/iterate_rectangles.hpp:37-104)
 * as bound for Python (src/python/functional/py_pcf.cpp:92-96, the Backend_*::iterate_rectangles of
 * stablebear.iterate_rectangles, stablebear/functional/pcf.py:347-374): the intervals [left, right)
 * on which both PCFs are constant, in time order, from the last breakpoint at or before a (the first
 * if none) up to b, each with f's and g's value there.  f_points / g_points: host arrays of nf / ng
 * interleaved (t, v) points of the dtype (SBG_F32, SBG_F64, SBG_I32, SBG_I64), times sorted.  a and
 * b are converted to the dtype (for integer types, infinities to its limits).  Writes up to cap
 * rectangles as (left, right, f_value, g_value) of the dtype into out and the number of rectangles
 * (all of them, also past cap; at most nf + ng - 1) into *count.  Runs on the current device and
 * returns when the result is on the host. */
int sbg_iterate_rectangles(int dtype, const void* f_points, uint64_t nf, const void* g_points, uint64_t ng,
                           double a, double b, void* out, uint64_t cap, uint64_t* count);

/* ---- batches: many independent problems in one persistent launch ----------------
 * No single counterpart in the reference (it runs one problem per task); each
 * problem is what create_cuda_block_integrate_{l1,lp,l2_kernel}_task computes.
 * Plan once, launch many times.  Problems are device-resident pdist or kernel
 * problems of one dtype and operation; their outputs are device buffers in
 * DistanceMatrix / SymmetricMatrix order. */
typedef struct sbg_problem {
  const void* points;           /* device: interleaved (t, v) */
  const uint64_t* offsets;      /* device: n + 1 offsets */
  const uint64_t* host_offsets; /* optional host copy of offsets (NULL: read back once at create) */
  uint64_t n;
  void* out;                    /* device output, n(n-1)/2 or n(n+1)/2 elements */
} sbg_problem;

typedef struct sbg_batch sbg_batch;
#define SBG_BATCH_GRAPH 1         /* launch through a captured CUDA graph */
#define SBG_BATCH_CALLER_ORDER 2  /* keep the caller's PCF order (default: sorted by breakpoint count) */
#define SBG_BATCH_TUNE_WINDOW 4   /* let sbg_batch_autotune move the time-windowed kernel's window cap */

/* Builds the batch: length orders, packed layouts, descriptors ordered by
 * estimated merge work (largest first).  Synchronises the device once. */
int sbg_batch_create(int dtype, int op, double p, int skip_mode, const sbg_problem* problems, uint64_t n_problems,
                     int flags, sbg_batch** batch);
/* Computes every problem of the batch on `stream` (queue reset + one kernel;
 * graph replay when created with SBG_BATCH_GRAPH). */
int sbg_batch_launch(sbg_batch* batch, void* stream);
/* Times (warps per CTA, rows per work item) settings on this batch, then
 * splits of shared memory between the column block and the row buffers,
 * and keeps the fastest; *best_ms receives its time per launch.  The split
 * is the hybrid kernel's column block (f64, or variant 4) and, only for a
 * batch created with SBG_BATCH_TUNE_WINDOW, the time-windowed kernel's
 * window cap.  Without that flag no tuned setting changes a bit of a
 * result; with it, window ends move with the cap, so sums may change in
 * their last bits (within the kernel's stated accuracy). */
int sbg_batch_autotune(sbg_batch* batch, void* stream, double* best_ms);
int sbg_batch_info(const sbg_batch* batch, uint64_t* items, uint64_t* pairs, int* warps, int* rows_per_item);
/* Elements per PCF held in the shared column block: the window cap of the
 * time-windowed kernel, or the hybrid kernel's column block. */
int sbg_batch_shared_split(const sbg_batch* batch, uint32_t* column_elements);
void sbg_batch_destroy(sbg_batch* batch);

/* ---- device entry that allocates nothing --------------------------------------
 * No counterpart in the reference; an addition of this library.
 *
 * For callers that cannot allocate device memory when they need a matrix: an
 * application whose allocator owns all device memory, a component running
 * while a CUDA graph is being recorded around it, a plugin host that only lends
 * inputs and outputs.  Same computation and arguments as sbg_pairwise_device,
 * plus the total breakpoint counts of the row and column sets; it calls no
 * cudaMalloc, cudaFree or other allocating routine.  Its scratch (the
 * persistent kernel's work-queue counter and, for PCFs too long for the
 * shared-memory kernel, a packed copy of the breakpoints) lives in one
 * fixed array of SBG_NOALLOC_SCRATCH_BYTES inside the library, which every
 * GPU that loads the library holds until the process exits.
 *   - max_points must be given (measuring it would need scratch of its own).
 *   - n_row_points / n_col_points must equal row_offsets[n_rows] /
 *     col_offsets[n_cols] (the host cannot read device offsets without a
 *     copy).  They size the packed copy; an undercount leaves the entries of
 *     PCFs past it unwritten while the call still returns SBG_OK.
 *   - A problem whose scratch would exceed SBG_NOALLOC_SCRATCH_BYTES is
 *     rejected with SBG_ERR_INVALID_ARGUMENT and a message giving both sizes;
 *     PCFs that fit the shared-memory kernel need only 256 bytes, whatever n.
 *   - The first call on each device looks up the array's device address on
 *     that device (cudaGetSymbolAddress); make that first call before any
 *     stream capture.
 *   - All calls share the one array: calls whose work overlaps on the GPU (on
 *     different streams, or from different threads) race on it.  Serialise
 *     them, e.g. on one stream. */
#define SBG_NOALLOC_SCRATCH_BYTES (4u << 20)
int sbg_pairwise_device_noalloc(int dtype, int op, double p, int skip_mode,
                                const void* row_points, const uint64_t* row_offsets, uint64_t n_rows,
                                uint64_t n_row_points,
                                const void* col_points, const uint64_t* col_offsets, uint64_t n_cols,
                                uint64_t n_col_points,
                                const uint32_t* row_perm, const uint32_t* col_perm, uint32_t max_points,
                                void* out, uint64_t out_base, uint64_t row_begin, uint64_t row_end,
                                void* stream);

/* ---- launch-shape autotuning for single problems ---------------------------------
 * No counterpart in the reference, whose block dimension and minimum block
 * side are user settings (include/sbear/settings.hpp:8-23).
 *
 * sbg_autotune_device runs the problem (same arguments as
 * sbg_pairwise_device over the whole problem, results into out) for a few
 * (warps per CTA, rows per work item) shapes, times each with CUDA events on
 * the stream (it synchronises), and caches the fastest under the problem's
 * key: element type, operation, skip mode and its shape bucket (floor(log2)
 * of n_rows and of max_points).  Later sbg_pairwise_device /
 * sbg_pairwise_host / task calls whose key matches use the cached shape
 * unless sbg_set_tuning fixed warps or rows per item.  These two knobs never
 * change a result bit (the time-windowed kernel keeps its window cap), so a
 * cached shape only changes the time.  The search sets the process-wide
 * tuning while it runs: do not run other calls concurrently with it.
 * *warps / *rows_per_item receive the shape kept, *best_ms its time per call. */
int sbg_autotune_device(int dtype, int op, double p, int skip_mode,
                        const void* row_points, const uint64_t* row_offsets, uint64_t n_rows,
                        const void* col_points, const uint64_t* col_offsets, uint64_t n_cols,
                        uint32_t max_points, void* out, void* stream,
                        int* warps, int* rows_per_item, double* best_ms);
/* Whether the cache holds a shape for this key (*hit 1 or 0), and which. */
int sbg_tuning_cache_lookup(int dtype, int op, double p, int skip_mode, uint64_t n_rows, uint32_t max_points,
                            int* warps, int* rows_per_item, int* hit);
/* Pins a shape for a key by hand (e.g. a table saved from an earlier
 * process): warps in [1, 32], rows_per_item a multiple of 32 in [32, 1024].
 * A shape that does not fit the problem's shared memory is ignored when
 * planning. */
int sbg_tuning_cache_store(int dtype, int op, double p, int skip_mode, uint64_t n_rows, uint32_t max_points,
                           int warps, int rows_per_item);
int sbg_tuning_cache_clear(void);

/* The processing order sbg_pairwise_device uses when it picks one itself:
 * perm[i] is the index of the PCF visited i-th, by breakpoint count within
 * each window of 1024 consecutive PCFs (ties by index).  Device pointers,
 * caller's stream.  Pass it as row_perm / col_perm to keep that order on a
 * band of rows.  No counterpart in the reference. */
int sbg_length_order_device(const uint64_t* offsets, uint64_t n, uint32_t* perm, void* stream);

/* Kernels this library has launched in this process so far (all threads and
 * devices; a CUDA graph replay counts the kernels it holds).  Read it before
 * and after a region to count the region's launches.  No counterpart in the
 * reference. */
uint64_t sbg_kernel_launches(void);

/* Host-side fault injection for the out-of-memory path.  Every device
 * allocation of the library (scratch, packed layouts, output bands) goes
 * through one allocator; with a limit set, an allocation that would take the
 * bytes the library holds above it fails before any CUDA call, and the entry
 * point returns SBG_ERR_OUT_OF_MEMORY with a message naming the sizes, as a
 * real cudaMalloc failure does.  No device memory is touched, so the next
 * call (with the limit lifted) runs normally.  SBG_ALLOC_UNLIMITED (the
 * default) removes the limit; 0 refuses every allocation.  Process-wide.
 * Replaces the reference's CHK_CUDA failure path
 * (include/sbear/cuda/cuda_util.cuh:8-10), which has no injection hook. */
#define SBG_ALLOC_UNLIMITED (~(uint64_t)0)
int sbg_set_alloc_limit(uint64_t bytes);
/* Device allocations the library has made in this process so far, and the
 * bytes it holds now.  No counterpart in the reference. */
uint64_t sbg_device_allocations(void);
uint64_t sbg_device_bytes_held(void);

/* Number of output elements of a problem (n(n-1)/2, n(n+1)/2 or n_rows*n_cols). */
uint64_t sbg_output_count(int skip_mode, uint64_t n_rows, uint64_t n_cols);

/* One scheduler block of the output: the dense row_height x col_width tile of
 * rows [row_start, row_start + row_height) against columns [col_start,
 * col_start + col_width), row-major with stride col_width, into a device
 * matrix the caller has cleared.  Entries the skip mode excludes (global
 * column > row, or >= row without the diagonal) are left zero.  Row and
 * column CSRs may be the same (pdist, kernel) or different (cdist); their
 * offsets are absolute into their points.  Device pointers, caller's stream.
 * Replaces PcfBlockOp::exec_block (include/sbear/cuda/pcf_block_op.cuh:82-122). */
int sbg_block_device(int dtype, int op, double p, int skip_mode, const void* row_points,
                     const uint64_t* row_offsets, const void* col_points, const uint64_t* col_offsets,
                     uint64_t row_start, uint64_t row_height, uint64_t col_start, uint64_t col_width,
                     uint32_t max_points, void* tile, void* stream);

/* ---- device-resident result containers ------------------------------------ */

/* Dense rows [row_begin, row_end) of the n x n matrix held in condensed form
 * on the device: skip_mode SBG_SKIP_LOWER_NODIAG for DistanceMatrix storage
 * (zero diagonal), SBG_SKIP_LOWER for SymmetricMatrix storage.  Row i lands
 * at dense + (i - row_begin) * ld (elements, ld >= n), on the caller's stream.
 * Replaces DistanceMatrix / SymmetricMatrix `to_dense`
 * (src/python/py_distance_matrix.hpp:37-49, py_symmetric_matrix.hpp), a
 * serial host loop in the reference. */
int sbg_condensed_to_dense_device(int dtype, int skip_mode, uint64_t n, const void* condensed, void* dense,
                                  uint64_t ld, uint64_t row_begin, uint64_t row_end, void* stream);

/* Condensed storage of a dense n x n device matrix (row stride ld), with the
 * reference's `from_dense` checks (py_distance_matrix.hpp:50-73,
 * py_symmetric_matrix.hpp:62-81) OR-ed into *flags (a device word the caller
 * zeroes): SBG_FLAG_ASYMMETRIC, and for DistanceMatrix storage
 * SBG_FLAG_DIAGONAL (a non-zero diagonal entry) and SBG_FLAG_NEGATIVE.  The
 * storage is written whatever the flags say; the caller rejects it. */
#define SBG_FLAG_ASYMMETRIC 1u
#define SBG_FLAG_DIAGONAL 2u
#define SBG_FLAG_NEGATIVE 4u
int sbg_dense_to_condensed_device(int dtype, int skip_mode, uint64_t n, const void* dense, uint64_t ld,
                                  void* condensed, unsigned int* flags, void* stream);

/* The adjoint of the symmetric expansion (sbg_condensed_to_dense_device):
 * each stored entry receives dense[i][j] + dense[j][i], i > j, and for
 * SymmetricMatrix storage the diagonal entry dense[i][i]; nothing is
 * checked.  This maps dL/d(dense) to dL/d(condensed) for gradients through
 * the expansion.  No counterpart in the reference (it has no gradients). */
int sbg_dense_fold_to_condensed_device(int dtype, int skip_mode, uint64_t n, const void* dense, uint64_t ld,
                                       void* condensed, void* stream);

/* ---- single-PCF integrals --------------------------------------------------- */

/* out[i] = ||f_i||_p over [0, inf) for the n PCFs of the CSR (p >= 1): the
 * reference's l1_norm (p == 1) and lp_norm (any other p, through pow)
 * (include/sbear/algorithms/functional/apply_functional.hpp:63-100, bound as
 * Norms_f32_f32 / Norms_f64_f64 .lpnorm_l1 / .lpnorm_lp in
 * src/python/functional/py_norms.cpp:24-56).  Device pointers, caller's
 * stream; the CSR is not validated. */
int sbg_lp_norm_device(int dtype, double p, const void* points, const uint64_t* offsets, uint64_t n, void* out,
                       void* stream);
/* The same from host memory, blocking, with the input checks of the
 * pairwise entries. */
int sbg_lp_norm_host(int dtype, double p, const void* points, const uint64_t* offsets, uint64_t n, void* out);

/* ---- barcodes to PCFs ---------------------------------------------------------- */

/* kind: the summary a barcode is turned into. */
#define SBG_STABLE_RANK 0 /* include/sbear/persistence/stable_rank.hpp:17-66 */
#define SBG_BETTI_CURVE 1 /* include/sbear/persistence/betti_curve.hpp:21-84 */

/* Upper bound on the points of the PCFs of n_barcodes barcodes holding
 * n_bars bars in all: n_bars + n_barcodes (stable rank), 2 n_bars +
 * n_barcodes (Betti curve). */
uint64_t sbg_barcode_pcf_capacity(int kind, uint64_t n_barcodes, uint64_t n_bars);

/* PCF of every barcode of a CSR of bars (interleaved (birth, death) pairs,
 * bar_offsets[n_barcodes + 1]), as a PCF CSR: out_points (interleaved
 * (t, v), room for out_capacity >= sbg_barcode_pcf_capacity points) and
 * out_offsets[n_barcodes + 1].  Device pointers, caller's stream.  Replaces
 * the reference's barcode_to_stable_rank / barcode_to_betti_curve tasks
 * (PersistenceBarcodeSummary32/64 in src/python/persistence/
 * py_barcode_summary.cpp), which convert one barcode at a time on the CPU. */
int sbg_barcodes_to_pcfs_device(int kind, int dtype, const void* bars, const uint64_t* bar_offsets,
                                uint64_t n_barcodes, uint64_t n_bars, void* out_points, uint64_t out_capacity,
                                uint64_t* out_offsets, void* stream);
/* The same from and to host memory, blocking. */
int sbg_barcodes_to_pcfs_host(int kind, int dtype, const void* bars, const uint64_t* bar_offsets,
                              uint64_t n_barcodes, void* out_points, uint64_t out_capacity, uint64_t* out_offsets);

#ifdef __cplusplus
}
#endif

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#endif /* SBGPU_H */
