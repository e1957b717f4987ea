// trv_batch_run_static: the batched kernel without any device allocation.
//
// trv_batch_create allocates the batch's task table, tile prefix and work
// counter with cudaMalloc.  Some callers cannot do that: cudaMalloc
// synchronizes the whole device, which stalls latency-critical loops that
// share the GPU with other streams, and processes whose device memory is
// reserved up front by another allocator (a framework's pool, a fixed arena)
// may have nothing left for a stray cudaMalloc, or must not fragment it.
// This entry point keeps those three tables in one file-scope __device__
// array instead, so a call allocates nothing on the device; the caller still
// provides every input and output array.
//
// Limits and sharing:
//  - at most kStaticMaxTasks tasks per call (larger batches are rejected with
//    TRV_ERR_UNSUPPORTED before anything is enqueued);
//  - the array is one per device, held by every process that loads the
//    library until it exits (about 300 KB), and shared by all calls on that
//    device: a call rewrites it and clears the work counter on its stream, so
//    two calls whose work overlaps on the GPU (different streams, or threads
//    without ordering) race on it and must be serialized by the caller;
//  - the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (once per device, that device current); make that
//    first call before any stream capture begins.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "autotune.h"
#include "batch.h"
#include "runtime.h"
#include "trove_gb300.h"

namespace trv {
namespace {

constexpr int kStaticMaxTasks = TRV_STATIC_BATCH_MAX_TASKS;
constexpr size_t kTaskBytes = sizeof(BatchTask) * kStaticMaxTasks;
constexpr size_t kPrefixOffset = (kTaskBytes + 255) / 256 * 256;
constexpr size_t kPrefixBytes = sizeof(long long) * (kStaticMaxTasks + 1);
constexpr size_t kCounterOffset = (kPrefixOffset + kPrefixBytes + 255) / 256 * 256;
constexpr size_t kScratchBytes = kCounterOffset + 256;

// Task table | tile prefix | work counter, each 256-byte aligned.
static __device__ __align__(256) unsigned char g_batch_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[64] = {};

bool aligned4(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) == 0; }

// Task checks and tile plan, the same rules as trv_batch_create: widths that
// are multiples of 4 up to 64 bytes, 4-byte aligned arrays, tiles of a
// multiple of 32 structs sized by the options, the autotuner cache or the
// size rule (128 KiB copy, 64 KiB index tiles), and one register budget
// chosen for the kernel by the caller or by the tuned majority of bytes.
int plan_static(const trv_task* tasks, uint64_t count, const trv_batch_options* opt, BatchTask* out,
                long long* prefix, int* blocks_per_sm) {
    uint64_t vote2 = 0, vote4 = 0;
    prefix[0] = 0;
    for (uint64_t k = 0; k < count; ++k) {
        const trv_task& t = tasks[k];
        if (t.op < TRV_OP_COPY || t.op > TRV_OP_SCATTER) return TRV_ERR_INVALID_ARGUMENT;
        if (t.width == 0 || t.n > (uint64_t(1) << 62) / t.width || t.bound > (uint64_t(1) << 62) / t.width)
            return TRV_ERR_INVALID_ARGUMENT;
        if (t.width % 4 != 0 || t.width > 64) return TRV_ERR_UNSUPPORTED;
        if (t.n > 0) {
            if (!t.src || !t.dst) return TRV_ERR_INVALID_ARGUMENT;
            if (!aligned4(t.src) || !aligned4(t.dst)) return TRV_ERR_MISALIGNED;
            if (t.op != TRV_OP_COPY) {
                if (!t.idx) return TRV_ERR_INVALID_ARGUMENT;
                if (!aligned4(t.idx)) return TRV_ERR_MISALIGNED;
            }
        }
        TuneChoice c;
        const bool tuned = tune_lookup(TuneKey{SCOPE_BATCH, t.op, int(t.width), len_bucket(t.n)}, &c);
        const int tile_bytes = (opt && opt->tile_bytes > 0)       ? opt->tile_bytes
                               : (tuned && c.tile_bytes > 0)      ? c.tile_bytes
                               : (t.op == TRV_OP_COPY)            ? (128 << 10)
                                                                  : (64 << 10);
        long long tile = (long long)tile_bytes / t.width;
        tile = tile < 32 ? 32 : (tile / 32) * 32;
        if (tile > (1 << 30)) tile = 1 << 30;
        const uintptr_t al = reinterpret_cast<uintptr_t>(t.src) | reinterpret_cast<uintptr_t>(t.dst);
        BatchTask& d = out[k];
        d.src = static_cast<const unsigned char*>(t.src);
        d.dst = static_cast<unsigned char*>(t.dst);
        d.idx = t.idx;
        d.n = (long long)t.n;
        d.bound = (long long)t.bound;
        d.op = t.op;
        d.words = int(t.width / 4);
        d.tile_structs = int(tile);
        d.word_log2 = (t.width % 16 == 0 && (al & 15u) == 0) ? 4 : (t.width % 8 == 0 && (al & 7u) == 0) ? 3 : 2;
        const int gp = (opt && opt->gather_policy) ? opt->gather_policy : 5;
        d.l2_hint = t.op != TRV_OP_GATHER ? 0 : gp == 4 ? 1 : gp == 5 ? 2 : 0;
        d.copy_bulk = opt && opt->copy_path == TRV_PATH_VECTOR ? 0 : 1;
        prefix[k + 1] = prefix[k] + (d.n + tile - 1) / tile;
        const uint64_t tb = 2 * t.n * t.width + (t.op == TRV_OP_COPY ? 0 : 4 * t.n);
        if (tuned && t.op != TRV_OP_COPY && c.grid == 2) vote2 += tb;
        if (tuned && t.op != TRV_OP_COPY && c.grid == 4) vote4 += tb;
    }
    *blocks_per_sm = (opt && opt->blocks_per_sm) ? opt->blocks_per_sm : (vote4 > vote2 ? 4 : 2);
    return TRV_OK;
}

// Device address of g_batch_scratch on the current device (resolved once).
int scratch_for_current_device(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e);
    if (dev < 0 || dev >= 64) return TRV_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_batch_scratch);
        if (e != cudaSuccess) return cuda_fail(e);
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return TRV_OK;
}

}  // namespace
}  // namespace trv

using namespace trv;

extern "C" int32_t trv_batch_run_static(const trv_task* tasks, uint64_t count, const trv_batch_options* opt,
                                        void* stream) {
    if (count > 0 && !tasks) return TRV_ERR_INVALID_ARGUMENT;
    if (count > uint64_t(kStaticMaxTasks)) return TRV_ERR_UNSUPPORTED;
    if (opt && (opt->tile_bytes < 0 || (opt->copy_path != TRV_PATH_AUTO && opt->copy_path != TRV_PATH_VECTOR)))
        return TRV_ERR_INVALID_ARGUMENT;
    if (opt && opt->blocks_per_sm != 0 && opt->blocks_per_sm != 2 && opt->blocks_per_sm != 4)
        return TRV_ERR_UNSUPPORTED;
    std::vector<BatchTask> host(count);
    std::vector<long long> prefix(count + 1);
    int blocks_per_sm = 4;
    const int rc = plan_static(tasks, count, opt, host.data(), prefix.data(), &blocks_per_sm);
    if (rc != TRV_OK) return rc;
    if (count == 0 || prefix[count] == 0) return TRV_OK;
    unsigned char* scratch = nullptr;
    const int src = scratch_for_current_device(&scratch);
    if (src != TRV_OK) return src;
    BatchTask* d_tasks = reinterpret_cast<BatchTask*>(scratch);
    long long* d_prefix = reinterpret_cast<long long*>(scratch + kPrefixOffset);
    unsigned long long* d_counter = reinterpret_cast<unsigned long long*>(scratch + kCounterOffset);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(d_tasks, host.data(), sizeof(BatchTask) * count, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_prefix, prefix.data(), sizeof(long long) * (count + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_fail(e);
    const int resident = resident_blocks(batch_kernel_func(blocks_per_sm), batch_block_threads());
    int grid = (opt && opt->grid_blocks > 0) ? opt->grid_blocks : resident;
    if (prefix[count] < grid) grid = int(prefix[count]);
    e = launch_batch_kernel(d_tasks, int(count), d_prefix, d_counter, grid, blocks_per_sm, st);
    return e == cudaSuccess ? TRV_OK : cuda_fail(e);
}
