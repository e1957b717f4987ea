/*
 * trove_gb300 — C ABI of the GB300 AoS load/store library.
 *
 * The reference (bryancatanzaro/trove) is a header-only device library with
 * no host API: users write kernels that call load_warp_contiguous /
 * store_warp_contiguous, the block interface or coalesced_ptr, and launch
 * them themselves (the reference's tests/benchmark.cu:52-128 and
 * tests/block.cu:13-54 are exactly such kernels).  This header is the host
 * boundary that replaces those hand-written kernels: each entry point
 * launches a kernel built on this library's own implementation of that
 * device API (the include/trove headers, same names and signatures as the
 * reference), on one GPU, stream-ordered and asynchronous.
 *
 * Conventions
 *  - Every function returns a trv_status (0 == TRV_OK); nothing throws.
 *  - Pointers are device pointers owned by the caller unless a name says
 *    _host.  `stream` is a cudaStream_t passed as void* (NULL = legacy
 *    default stream).  Sizes are 64-bit: n counts structs, width is
 *    sizeof(T) in bytes.
 *  - Work is enqueued on `stream`; the call returns before it finishes.
 *    Argument errors are reported synchronously; a launch failure returns
 *    TRV_ERR_CUDA with the CUDA error available from trv_last_cuda_error().
 *  - Results are bit-exact copies of the source bytes.
 *  - Indices are int32.  Gather/scatter skip an index outside [0, bound):
 *    that output struct (gather) or that source struct (scatter) is left
 *    untouched, so a bad index never faults the GPU.
 *  - Threads: the stateless calls (copy, gather, scatter, layout, fills) and
 *    the autotuner cache may be used from any number of host threads at
 *    once.  A trv_batch handle is used by one thread at a time; a trv_server
 *    handle may be used from several (it locks internally).
 *    trv_batch_run_static shares one device array between all callers, so
 *    its calls must not overlap.
 *  - Devices: the current device of the calling thread.  Batches, servers,
 *    trv_batch_run_static and the staged form of trv_copy_host serve
 *    devices 0-63 of the process (others get an error status); the other
 *    calls serve any device.
 */
#ifndef TROVE_GB300_H
#define TROVE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum trv_status {
    TRV_OK = 0,
    TRV_ERR_INVALID_ARGUMENT = 1, /* null pointer with n > 0, width 0, size overflow */
    TRV_ERR_UNSUPPORTED = 2,      /* path/width combination not offered */
    TRV_ERR_MISALIGNED = 3,       /* explicit path needs an alignment the pointers lack */
    TRV_ERR_CUDA = 4,             /* a CUDA call failed; see trv_last_cuda_error() */
    TRV_ERR_OUT_OF_MEMORY = 5,
    TRV_ERR_BUDGET = 6,           /* request larger than the configured HBM budget */
    TRV_ERR_TIMEOUT = 7,
    TRV_ERR_NOT_FOUND = 8,
    TRV_ERR_BUSY = 9,
    TRV_ERR_CANCELLED = 10,
    TRV_ERR_DEVICE_FLAG = 11      /* a kernel reported an error flag */
} trv_status;

/* Data-movement strategy.  AUTO picks per (op, width, length, alignment). */
typedef enum trv_path {
    TRV_PATH_AUTO = 0,
    TRV_PATH_WARP = 1,    /* copy: load/store_warp_contiguous (coalesced rounds + register transpose);
                             gather/scatter: warp-cooperative row-form rounds, no transpose */
    TRV_PATH_BLOCK = 2,   /* block interface: *_array_warp_contiguous, load/store_array fallback */
    TRV_PATH_VECTOR = 3,  /* flat copy with the widest vector both pointers allow */
    TRV_PATH_BULK = 4,    /* TMA bulk copy (cp.async.bulk) staged through shared memory */
    TRV_PATH_DIRECT = 5,  /* compiler-generated per-thread struct access (baseline) */
    TRV_PATH_COALESCED = 6 /* coalesced_ptr: contiguity check, warp path or per-thread words */
} trv_path;

/* Optional launch shape; zero fields mean "choose". */
typedef struct trv_launch {
    int32_t path;          /* trv_path */
    int32_t unroll;        /* structs per thread per pass: 1, 2, 4 or 8 */
    int32_t block_threads; /* 256 (the only block size offered; 0 = 256) */
    int32_t grid_blocks;   /* 0: one pass per warp (full grid); -1: persistent grid of
                              resident blocks; > 0: that many blocks, grid-stride */
    int32_t chunk_bytes;   /* TRV_PATH_BULK: bytes per shared-memory stage, multiple of 16 */
    int32_t cache_policy;  /* gather / scatter, TRV_PATH_WARP: 0 default; 1 streaming index and
                              contiguous side (evict-first); 2 as 1, random side L2-only;
                              3 as 1, random side kept in L2 (evict-last); 4 as 1, random-side
                              loads with a 64-byte L2 prefetch-size hint; 5 as 1, random-side
                              loads with a 128-byte L2 prefetch-size hint (gathers); 6 (scatters)
                              as 1, in passes over 64 MiB parts of the destination, so that
                              partial-sector writes of narrow structs merge in L2 (the default
                              for structs of at most 16 bytes onto destinations above 64 MiB) */
} trv_launch;

const char* trv_status_string(int32_t status);
int32_t trv_version(void);
/* Last CUDA error code seen by this thread's calls (0 if none). */
int32_t trv_last_cuda_error(void);

/* Sets the current context's L2 fetch granularity hint (bytes: 32, 64 or 128;
 * cudaLimitMaxL2FetchGranularity) and returns the previous value in
 * *previous (may be NULL).  Measured on GB300 random gathers: 128 helps
 * 8-byte structs by ~20 % and costs wide ones 4-10 %, 32 hurts narrow ones;
 * the default (64) is the best single setting.  It is a per-process context
 * setting (released with the context), applies to every kernel the context
 * runs afterwards, and may synchronize the device: set it once at start-up. */
int32_t trv_set_l2_fetch_granularity(int32_t bytes, int32_t* previous);

/* Synchronizes `stream`, then reads and clears the current device's error
 * flag, which a kernel sets when one of its bounded waits gives up (the TMA
 * bulk path).  TRV_ERR_DEVICE_FLAG if it was set. */
int32_t trv_check_device(void* stream);

/* Testing hook for the bounded waits of the TMA bulk path: the copy loop's
 * mbarrier waits give up after `polls` polls (0xFFFFFFFF restores the default
 * of about a second).  A wait that gives up sets the device flag that
 * trv_check_device reports; the kernel still waits (with the default budget)
 * for every transfer it has in flight before it exits, so the context stays
 * usable.  With 0 polls every launch reports the flag. */
int32_t trv_debug_set_bulk_wait_polls(uint32_t polls);

/* dst[i] = src[i] for i < n structs of `width` bytes.
 * Replaces the user kernel `T v = load_warp_contiguous(src + i);
 * store_warp_contiguous(v, dst + i);` (reference trove/aos.h:66-105,
 * pattern of tests/benchmark.cu:52-88). */
int32_t trv_copy(void* dst, const void* src, uint64_t n, uint32_t width, void* stream);
int32_t trv_copy_ex(void* dst, const void* src, uint64_t n, uint32_t width,
                    const trv_launch* cfg, void* stream);

/* Copy with a data-dependent early exit: struct i is copied unless its first
 * 32-bit word w satisfies w % modulus == modulus - 1 (modulus 0: never).
 * Lanes that exit leave their warp non-converged, so the remaining lanes take
 * the per-thread fallback.  path is TRV_PATH_WARP (warp_converged() ?
 * load/store_warp_contiguous : per-thread) or TRV_PATH_BLOCK (the block
 * interface with its load_array/store_array fallback, reference
 * trove/block.h:35-65 and tests/block.cu:34-54).  width % 4 == 0, <= 64. */
int32_t trv_copy_exit(void* dst, const void* src, uint64_t n, uint32_t width, uint32_t modulus,
                      int32_t path, void* stream);
/* Same, with the launch shape given (cfg->path is TRV_PATH_WARP or TRV_PATH_BLOCK). */
int32_t trv_copy_exit_ex(void* dst, const void* src, uint64_t n, uint32_t width, uint32_t modulus,
                         const trv_launch* cfg, void* stream);

/* dst[i] = src[idx[i]] for i < n; idx[i] outside [0, src_n) is skipped.
 * Widths 4..64 in steps of 4 have per-width kernels; wider multiples of 4
 * use the row-form kernel with a run-time word count; other widths a
 * byte-wise kernel.
 * Replaces the coalesced_ptr gather kernel (reference trove/ptr.h:76-90,
 * tests/benchmark.cu:90-99). */
int32_t trv_gather(void* dst, const void* src, uint64_t src_n, const int32_t* idx, uint64_t n,
                   uint32_t width, void* stream);
int32_t trv_gather_ex(void* dst, const void* src, uint64_t src_n, const int32_t* idx, uint64_t n,
                      uint32_t width, const trv_launch* cfg, void* stream);

/* dst[idx[i]] = src[i] for i < n; idx[i] outside [0, dst_n) is skipped.
 * With repeated indices the surviving write is unspecified (as in the
 * reference).  Replaces tests/benchmark.cu:101-110. */
int32_t trv_scatter(void* dst, uint64_t dst_n, const void* src, const int32_t* idx, uint64_t n,
                    uint32_t width, void* stream);
int32_t trv_scatter_ex(void* dst, uint64_t dst_n, const void* src, const int32_t* idx, uint64_t n,
                       uint32_t width, const trv_launch* cfg, void* stream);

/* Layout conversion for structs of width/4 32-bit fields (width a multiple
 * of 4, at most 64): field j of struct i is aos[i].field[j] and
 * soa[j * n + i].  The AoS side moves through the device API
 * (load/store_warp_contiguous), the SoA side as one coalesced stream per
 * field.  The reference's block interface exists for such per-thread array
 * producers and consumers (README "Block Interface"); these entry points are
 * the conversion kernels users of it write by hand. */
int32_t trv_aos_to_soa(void* dst_soa, const void* src_aos, uint64_t n, uint32_t width, void* stream);
int32_t trv_soa_to_aos(void* dst_aos, const void* src_soa, uint64_t n, uint32_t width, void* stream);
/* The same with an explicit unroll / grid (cfg->path is ignored; unroll 0:
 * the autotuner's choice for TRV_OP_AOS_TO_SOA / TRV_OP_SOA_TO_AOS, else a
 * width rule). */
int32_t trv_aos_to_soa_ex(void* dst_soa, const void* src_aos, uint64_t n, uint32_t width, const trv_launch* cfg,
                          void* stream);
int32_t trv_soa_to_aos_ex(void* dst_aos, const void* src_soa, uint64_t n, uint32_t width, const trv_launch* cfg,
                          void* stream);

/* Synthetic inputs: dst[k] = word k of the seeded splitmix64 stream (the same
 * stream the CPU oracle generates).  No reference counterpart. */
int32_t trv_fill_random_u32(uint32_t* dst, uint64_t nwords, uint64_t seed, void* stream);

/* Synthetic indices: idx[i] = uniform in [0, bound) from the seeded stream
 * (the oracle's orc_uniform_indices gives the same values).  bound < 2^31. */
int32_t trv_fill_uniform_indices(int32_t* idx, uint64_t n, uint32_t bound, uint64_t seed, void* stream);
/* Run pattern (32 <= n < 2^31): each aligned chunk of 32 outputs is, with
 * probability 1/2, a run start + 0..31 (start uniform in [0, n - 32]), else
 * 32 independent indices uniform in [0, n).  Device kernel, stream-ordered. */
int32_t trv_fill_run_indices(int32_t* idx, uint64_t n, uint64_t seed, void* stream);
/* Seeded Fisher-Yates permutation of 0..n-1 (n < 2^31), computed on the host
 * and copied to idx on `stream`; returns after the copy. */
int32_t trv_fill_permutation(int32_t* idx, uint64_t n, uint64_t seed, void* stream);

/* Host-buffer copy; returns when dst_host holds the result.  When the GPU can
 * address both buffers (pinned memory, or any memory where the GPU uses the
 * host page tables) the copy kernel reads and writes them in place; otherwise
 * src_host -> device staging -> copy kernel -> dst_host, chunked and
 * overlapped on internal streams.  No reference counterpart (the reference
 * has no host API). */
int32_t trv_copy_host(void* dst_host, const void* src_host, uint64_t n, uint32_t width);

/* ---- batched execution ---------------------------------------------------
 * Thousands of independent AoS arrays in one persistent launch driven by a
 * device work queue.  No reference counterpart: the reference moves one array
 * per user kernel. */

typedef enum trv_op {
    TRV_OP_COPY = 0,
    TRV_OP_GATHER = 1,
    TRV_OP_SCATTER = 2,
    /* autotuner keys only: the early-exit copy through each device-API path,
       and the two layout conversions */
    TRV_OP_COPY_EXIT_WARP = 3,
    TRV_OP_COPY_EXIT_BLOCK = 4,
    TRV_OP_AOS_TO_SOA = 5,
    TRV_OP_SOA_TO_AOS = 6
} trv_op;

typedef struct trv_task {
    int32_t op;          /* trv_op */
    uint32_t width;      /* bytes per struct: a multiple of 4, at most 64 */
    uint64_t n;          /* structs copied, or number of indices */
    const void* src;     /* device */
    void* dst;           /* device */
    const int32_t* idx;  /* device, n entries (gather / scatter only) */
    uint64_t bound;      /* gather: source length; scatter: destination length */
} trv_task;

typedef struct trv_batch_options {
    int32_t tile_bytes;  /* payload bytes per tile; 0: autotuner cache, else the size rule */
    int32_t copy_path;   /* copy tasks: TRV_PATH_AUTO (the autotuned choice, else TMA bulk tiles
                            where source and destination are 16-byte aligned) or
                            TRV_PATH_VECTOR (flat vector tiles) */
    int32_t grid_blocks; /* 0: resident blocks of the persistent kernel; a positive value is
                            launched as given, capped at the batch's tile count (above the
                            device's grid limit: TRV_ERR_CUDA at launch) */
    int32_t blocks_per_sm; /* resident blocks per SM: 4 (64 registers per thread; every gather and
                              scatter row staged through shared memory) or 2 (128, which also
                              offers the register-held rows of policies 1 and 4);
                              0: the autotuned or default choice (4) */
    int32_t gather_policy; /* gather tasks' random loads: 0 the autotuned or default choice (7);
                              1 rows held in registers, plain loads; 4 the same with the 64-byte
                              L2 prefetch-size hint (at 4 blocks per SM, 1 and 4 are staged like
                              5 and 6); 5 rows staged through shared memory with asynchronous
                              copies (cp.async); 6 / 7 staged, with the 64 / 128-byte L2
                              prefetch-size hint */
    int32_t scatter_policy; /* scatter tasks: 0 the autotuned or default choice (5); 1 rows held
                               in registers (at 4 blocks per SM: staged like 5); 5 the contiguous
                               source staged through shared memory with cp.async, stored to the
                               random rows from there */
} trv_batch_options;

typedef struct trv_batch trv_batch;

/* Validates the tasks, splits them into tiles and uploads the plan (device
 * memory owned by the batch).  Pointers are captured, not the data: the batch
 * may be launched any number of times while the arrays stay allocated. */
int32_t trv_batch_create(const trv_task* tasks, uint64_t count, const trv_batch_options* opt,
                         trv_batch** out);
/* Enqueues one run of the whole batch: counter reset + one persistent kernel,
 * or a replay of the captured graph.  The device current at trv_batch_create
 * must be current (TRV_ERR_INVALID_ARGUMENT otherwise), here and in capture. */
int32_t trv_batch_launch(trv_batch* batch, void* stream);
/* Records counter reset + kernel into a CUDA graph (on `stream`, which must
 * not be the legacy default stream); later trv_batch_launch calls replay it. */
int32_t trv_batch_capture(trv_batch* batch, void* stream);
/* Tiles and algorithmic bytes (read + written + index bytes) of one run. */
int32_t trv_batch_info(const trv_batch* batch, uint64_t* tiles, uint64_t* bytes);
int32_t trv_batch_destroy(trv_batch* batch);

/* Largest batch trv_batch_run_static accepts. */
#define TRV_STATIC_BATCH_MAX_TASKS 4096

/* The batch without any device allocation, for callers that cannot call
 * cudaMalloc: it synchronizes the whole device (stalling latency-critical
 * loops that share the GPU), and processes whose device memory is reserved
 * up front by another allocator may have none to spare.  No counterpart in
 * the reference.  Same tasks, options and results as trv_batch_create +
 * trv_batch_launch, planned and launched in one call on `stream`; the task
 * table, tile prefix and work counter live in one library-owned __device__
 * array (about 300 KB per device, held until the process exits) instead of
 * cudaMalloc'd memory.  At most TRV_STATIC_BATCH_MAX_TASKS tasks
 * (TRV_ERR_UNSUPPORTED beyond).  Every call on a device shares that array and
 * clears its counter on `stream`: calls whose work overlaps on the GPU race
 * and must be ordered by the caller.  The first call on a device looks up the
 * array's address (once per device); make it before any stream capture.  The
 * address stays cached for the process: after cudaDeviceReset of a device, do
 * not call this entry point on that device again.  The plan is copied from
 * pageable host memory that the call frees on return, so the call may wait
 * for `stream`'s earlier work before returning, and a stream that is being
 * captured is refused with TRV_ERR_UNSUPPORTED (trv_batch_capture is the
 * route for graphs).  A positive opt->grid_blocks is launched as given (above
 * the device's grid limit: TRV_ERR_CUDA); a current device index of 64 or
 * more: TRV_ERR_UNSUPPORTED. */
int32_t trv_batch_run_static(const trv_task* tasks, uint64_t count, const trv_batch_options* opt,
                             void* stream);

/* Baseline for the batch: one plain launch per task (trv_copy / trv_gather /
 * trv_scatter, AUTO path), in order, on `stream`. */
int32_t trv_run_per_call(const trv_task* tasks, uint64_t count, void* stream);

/* ---- diagnostics -----------------------------------------------------------------
 * The memory system's ceiling for a random gather, measured on the GPU at hand.
 * For each i < n, reads every block_bytes-aligned block (32, 64 or 128) of src
 * that row idx[i] (bytes idx[i]*width .. +width) overlaps, as whole 16-byte
 * vectors shared by adjacent lanes, with an L2 prefetch-size hint l2_hint
 * (0 none, 64 or 128 bytes); reads idx sequentially and writes n*width bytes
 * to dst sequentially (a fold of the blocks, not the rows).  The time of this
 * call is what a gather of the same rows costs with the best access shape:
 * the denominator that gathers are compared against.  n % 32 == 0, width a
 * multiple of 4 up to 128, src aligned to block_bytes and readable up to
 * src_n*width rounded up to block_bytes, dst 16-byte aligned; indices outside
 * [0, src_n) read nothing.  No reference counterpart. */
int32_t trv_probe_block_gather(void* dst, const void* src, uint64_t src_n, const int32_t* idx, uint64_t n,
                               uint32_t width, uint32_t block_bytes, int32_t l2_hint, void* stream);

/* ---- serving -------------------------------------------------------------------
 * A request loop for copy and gather requests against device-resident sources.
 * Requests are admitted in arrival order while their output fits in the HBM
 * budget (outputs live in one device arena of that size), folded into the
 * batched persistent kernel as soon as a batch slot is free, and up to
 * `max_inflight` batches run concurrently on separate streams, so requests that
 * arrive while others are on the GPU join the next batch (continuous batching).
 * A dispatcher thread owned by the server does admission, launch and
 * completion; while batches are in flight it polls their completion with
 * yields, keeping one host core busy, and when idle it blocks.  No reference
 * counterpart. */

typedef struct trv_server_config {
    uint64_t hbm_budget_bytes;   /* output arena size */
    int32_t max_inflight;        /* concurrent batches (streams), at most 64; 0: 4 */
    int32_t max_batch_requests;  /* requests per batch, at most 65536; 0: 1024 */
    int32_t tile_bytes;          /* 0: autotuner cache, else the size rule */
    int32_t release_when_done;   /* 1: outputs are freed as soon as a request completes */
} trv_server_config;

typedef struct trv_request {
    int32_t op;            /* TRV_OP_COPY or TRV_OP_GATHER */
    uint32_t width;        /* bytes per struct: a multiple of 4, at most 64 */
    uint64_t n;            /* structs produced */
    const void* src;       /* device source (copy: n structs; gather: src_n structs) */
    uint64_t src_n;        /* gather: source length */
    const int32_t* idx;    /* gather: n device indices; the output struct of an index
                              outside [0, src_n) is not written, so it holds whatever
                              the server's arena held there before */
} trv_request;

typedef struct trv_result {
    int32_t status;        /* TRV_OK when done; TRV_ERR_BUSY while queued or running */
    int32_t batch;         /* sequence number of the batch that ran it */
    void* dst;             /* device output (server-owned until released) */
    double submit_ms;      /* host times, ms since the server started */
    double launch_ms;
    double done_ms;
} trv_result;

typedef struct trv_server_stats {
    uint64_t submitted, admitted, completed, rejected;
    uint64_t batches;            /* persistent-kernel launches (a batch holding both small and large
                                    requests is two: the small ones first, completing on their own) */
    uint64_t max_queued;         /* most requests waiting for admission at once */
    uint64_t bytes;              /* algorithmic bytes of completed requests */
    uint64_t budget_in_use;      /* arena bytes held now */
    double p50_ms, p99_ms, mean_ms, max_ms;  /* submit -> done latency of completed requests */
    double first_submit_ms, last_done_ms;
} trv_server_stats;

typedef struct trv_server trv_server;

int32_t trv_server_create(const trv_server_config* cfg, trv_server** out);
/* Queues a request; returns at once.  TRV_ERR_BUDGET if its output alone
 * exceeds the budget.  The server's streams are not ordered after any caller
 * stream: the request's source and index arrays must already be complete on
 * the device (synchronize the stream that wrote them before submitting). */
int32_t trv_server_submit(trv_server* s, const trv_request* req, uint64_t* id);
/* TRV_OK with the result once done, TRV_ERR_BUSY before, TRV_ERR_NOT_FOUND
 * for an unknown or released id. */
int32_t trv_server_poll(trv_server* s, uint64_t id, trv_result* out);
int32_t trv_server_wait(trv_server* s, uint64_t id, double timeout_ms, trv_result* out);
/* Frees a completed request's output (its budget returns to the arena). */
int32_t trv_server_release(trv_server* s, uint64_t id);
int32_t trv_server_stats_get(trv_server* s, trv_server_stats* out);
/* Open-loop load: submits reqs[k] when arrival_ms[k] (ms from the call) is
 * reached, from a native thread, and returns when every request is done.
 * ids (optional, count entries) receives the request ids. */
int32_t trv_server_replay(trv_server* s, const trv_request* reqs, const double* arrival_ms, uint64_t count,
                          uint64_t* ids, trv_server_stats* out);
/* Drains outstanding work, then frees everything. */
int32_t trv_server_destroy(trv_server* s);

/* ---- autotuner -------------------------------------------------------------
 * Launch choices cached per (scope, op, width, length bucket of a factor 4).
 * Scope 0 (per call) steers the AUTO path of trv_copy / trv_gather /
 * trv_scatter (path, unroll and cache policy); scope 1 (batch) gives the
 * batched kernel its tile size, register budget, gather / scatter policy and
 * copy variant per group.  No reference counterpart. */

/* Times every candidate launch shape for (op, width, n) on scratch arrays of
 * n structs, each run after an L2 flush, median of three (uniform random
 * indices for gather / scatter; op may also be
 * TRV_OP_COPY_EXIT_WARP / _BLOCK, tuned with the exit modulus 625, or
 * TRV_OP_AOS_TO_SOA / TRV_OP_SOA_TO_AOS) and caches the fastest in scope 0. */
int32_t trv_autotune_call(int32_t op, uint32_t width, uint64_t n, void* stream);
/* Times tile size, register budget, gather / scatter policy and copy variant
 * for each (op, width, bucket) group of the given tasks, running each group
 * alone as a batch, and caches the fastest in scope 1.  The tasks' arrays
 * are read and written. */
int32_t trv_autotune_batch(const trv_task* tasks, uint64_t count, void* stream);
/* Cached choice for (scope, op, width, n); TRV_ERR_NOT_FOUND if none. */
int32_t trv_autotune_lookup(int32_t scope, int32_t op, uint32_t width, uint64_t n, trv_launch* out,
                            int32_t* tile_bytes);
int32_t trv_autotune_clear(void);
/* JSON file: an array of {scope, op, width, bucket, path, unroll, grid, chunk,
 * tile_bytes, cache_policy, gbs} objects (scope 1 keeps the register budget in
 * grid and the gather / scatter policy in cache_policy). */
int32_t trv_autotune_save(const char* path);
int32_t trv_autotune_load(const char* path);

#ifdef __cplusplus
}
#endif

#endif /* TROVE_GB300_H */
