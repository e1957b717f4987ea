// Host side of batched execution: validation, the tile plan, the device task
// table, graph capture, and the one-launch-per-task baseline.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <new>
#include <vector>

#include "autotune.h"
#include "batch.h"
#include "runtime.h"
#include "trove_gb300.h"

struct trv_batch {
    int device = 0;
    int ntasks = 0;
    trv::BatchTask* d_tasks = nullptr;
    long long* d_prefix = nullptr;
    unsigned long long* d_counter = nullptr;
    long long total_tiles = 0;
    uint64_t bytes = 0;
    int grid = 0;
    int blocks_per_sm = 4;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// A batch's plan lives on the device that was current when it was created.
bool on_batch_device(const trv_batch* b) {
    int dev = -1;
    return cudaGetDevice(&dev) == cudaSuccess && dev == b->device;
}

void release(trv_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_tasks) cudaFree(b->d_tasks);
    if (b->d_prefix) cudaFree(b->d_prefix);
    if (b->d_counter) cudaFree(b->d_counter);
    b->exec = nullptr;
    b->graph = nullptr;
    b->d_tasks = nullptr;
    b->d_prefix = nullptr;
    b->d_counter = nullptr;
}

}  // namespace

namespace trv {
namespace {

bool aligned4(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) == 0; }

int validate(const trv_task& t) {
    if (t.op < TRV_OP_COPY || t.op > TRV_OP_SCATTER) return TRV_ERR_INVALID_ARGUMENT;
    if (t.width == 0 || t.n > (uint64_t(1) << 62) / t.width || t.bound > (uint64_t(1) << 62) / t.width)
        return TRV_ERR_INVALID_ARGUMENT;
    if (t.width % 4 != 0 || t.width > 64) return TRV_ERR_UNSUPPORTED;
    if (t.n == 0) return TRV_OK;
    if (!t.src || !t.dst) return TRV_ERR_INVALID_ARGUMENT;
    if (!aligned4(t.src) || !aligned4(t.dst)) return TRV_ERR_MISALIGNED;
    if (t.op != TRV_OP_COPY) {
        if (!t.idx) return TRV_ERR_INVALID_ARGUMENT;
        if (!aligned4(t.idx)) return TRV_ERR_MISALIGNED;
    }
    return TRV_OK;
}

// Size rule when no tuned tile exists: big enough to amortise the queue
// step, small enough to balance the tail across 152 SMs.
int default_tile_bytes(int op) { return op == TRV_OP_COPY ? (128 << 10) : (64 << 10); }

}  // namespace

long long plan_task(int op, uint32_t width, uint64_t n, uint64_t bound, const void* src, void* dst,
                    const int32_t* idx, const TaskPlan& p, BatchTask* d) {
    long long tile = (long long)p.tile_bytes / width;
    tile = tile < 32 ? 32 : (tile / 32) * 32;
    if (tile > (1 << 30)) tile = 1 << 30;
    d->src = static_cast<const unsigned char*>(src);
    d->dst = static_cast<unsigned char*>(dst);
    d->idx = idx;
    d->n = (long long)n;
    d->bound = (long long)bound;
    d->op = op;
    d->words = int(width / 4);
    d->tile_structs = int(tile);
    // Word moved per lane by the row-form index movers: the widest of 16 / 8
    // / 4 bytes that divides the width and that both arrays are aligned to.
    const uintptr_t al = reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst);
    d->word_log2 = (width % 16 == 0 && (al & 15u) == 0) ? 4 : (width % 8 == 0 && (al & 7u) == 0) ? 3 : 2;
    d->index_mode = op == TRV_OP_GATHER    ? (p.gather_policy == 4   ? 1
                                              : p.gather_policy >= 5 ? p.gather_policy - 3
                                                                     : 0)
                    : op == TRV_OP_SCATTER ? (p.scatter_policy == 5 ? 2 : 0)
                                           : 0;
    d->copy_bulk = p.copy_bulk;
    return ((long long)n + tile - 1) / tile;
}

int check_batch_options(const trv_batch_options* opt) {
    if (!opt) return TRV_OK;
    if (opt->copy_path != TRV_PATH_AUTO && opt->copy_path != TRV_PATH_VECTOR) return TRV_ERR_UNSUPPORTED;
    if (opt->tile_bytes < 0) return TRV_ERR_INVALID_ARGUMENT;
    if (opt->blocks_per_sm != 0 && opt->blocks_per_sm != 2 && opt->blocks_per_sm != 4) return TRV_ERR_UNSUPPORTED;
    if (opt->gather_policy != 0 && opt->gather_policy != 1 && (opt->gather_policy < 4 || opt->gather_policy > 7))
        return TRV_ERR_INVALID_ARGUMENT;
    if (opt->scatter_policy != 0 && opt->scatter_policy != 1 && opt->scatter_policy != 5)
        return TRV_ERR_INVALID_ARGUMENT;
    return TRV_OK;
}

int plan_batch(const trv_task* tasks, uint64_t count, const trv_batch_options* opt, BatchTask* out,
               long long* prefix, uint64_t* bytes, int* blocks_per_sm) {
    // bytes of gather / scatter tasks whose tuned entry prefers 2 / 4 blocks per
    // SM (their movers set the register budget; copy tiles barely use one)
    uint64_t vote2 = 0, vote4 = 0, total = 0;
    prefix[0] = 0;
    for (uint64_t k = 0; k < count; ++k) {
        const trv_task& t = tasks[k];
        const int rc = validate(t);
        if (rc != TRV_OK) return rc;
        TuneChoice c;
        const bool tuned = tune_lookup(TuneKey{SCOPE_BATCH, t.op, int(t.width), len_bucket(t.n)}, &c);
        TaskPlan p;
        p.tile_bytes = (opt && opt->tile_bytes > 0) ? opt->tile_bytes
                       : (tuned && c.tile_bytes > 0) ? c.tile_bytes
                                                     : default_tile_bytes(t.op);
        // Gather and scatter rows are staged through shared memory with
        // cp.async unless chosen otherwise: on the 4096-array workload (4
        // blocks per SM) its gathers took 12.1 ms that way against 20.5 ms
        // with register-held rows, its scatters 3.5 against 6.3 ms.  Gathers
        // ask L2 for whole 128-byte lines (policy 7): GB300s whose default
        // fetch is 64 bytes then run them as fast as those that fetch 128
        // (12.1 vs 12.9 ms; every width gains, 64-byte structs included).
        p.gather_policy = (opt && opt->gather_policy) ? opt->gather_policy
                          : (tuned && c.cache_policy) ? c.cache_policy
                                                      : 7;
        p.scatter_policy = (opt && opt->scatter_policy) ? opt->scatter_policy
                           : (tuned && c.cache_policy)  ? c.cache_policy
                                                        : 5;
        const int cp = (opt && opt->copy_path) ? opt->copy_path : (tuned && c.path) ? c.path : TRV_PATH_AUTO;
        p.copy_bulk = cp == TRV_PATH_VECTOR ? 0 : 1;
        prefix[k + 1] = prefix[k] + plan_task(t.op, t.width, t.n, t.bound, t.src, t.dst, t.idx, p, &out[k]);
        const uint64_t tb = 2 * t.n * t.width + (t.op == TRV_OP_COPY ? 0 : 4 * t.n);
        total += tb;
        if (tuned && t.op != TRV_OP_COPY && c.grid == 2) vote2 += tb;
        if (tuned && t.op != TRV_OP_COPY && c.grid == 4) vote4 += tb;
    }
    if (bytes) *bytes = total;
    // One register budget for the whole kernel: the caller's, else the one the
    // autotuner preferred for most of the batch's bytes, else 4 blocks per SM:
    // the staged gather / scatter movers and the TMA copy tiles need few
    // registers, and twice the resident blocks overlap their block barriers
    // (4096-array workload, default tiles: 22.9 ms against 27.5 ms at 2).
    *blocks_per_sm = (opt && opt->blocks_per_sm) ? opt->blocks_per_sm : (vote2 > vote4 ? 2 : 4);
    return TRV_OK;
}

}  // namespace trv

using namespace trv;

extern "C" {

static int32_t batch_create_impl(const trv_task* tasks, uint64_t count, const trv_batch_options* opt, trv_batch** out) {
    if (!out) return TRV_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (count > 0 && !tasks) return TRV_ERR_INVALID_ARGUMENT;
    if (count >= uint64_t(INT_MAX)) return TRV_ERR_INVALID_ARGUMENT;
    const int orc = check_batch_options(opt);
    if (orc != TRV_OK) return orc;
    std::vector<BatchTask> host(count);
    std::vector<long long> prefix(count + 1, 0);
    uint64_t bytes = 0;
    int blocks_per_sm = 4;
    const int prc = plan_batch(tasks, count, opt, host.data(), prefix.data(), &bytes, &blocks_per_sm);
    if (prc != TRV_OK) return prc;
    // the error flag and the kernel set-up are resolved now, outside any later graph capture
    if (!device_flag()) return TRV_ERR_CUDA;
    const int resident = batch_grid(blocks_per_sm);
    if (resident < 1) return TRV_ERR_CUDA;
    trv_batch* b = new (std::nothrow) trv_batch;
    if (!b) return TRV_ERR_OUT_OF_MEMORY;
    cudaGetDevice(&b->device);
    b->ntasks = int(count);
    b->total_tiles = prefix[count];
    b->bytes = bytes;
    cudaError_t e = cudaMalloc(&b->d_tasks, sizeof(BatchTask) * (count ? count : 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_prefix, sizeof(long long) * (count + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_counter, sizeof(unsigned long long));
    if (e == cudaSuccess && count)
        e = cudaMemcpy(b->d_tasks, host.data(), sizeof(BatchTask) * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_prefix, prefix.data(), sizeof(long long) * (count + 1), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        release(b);
        delete b;
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? TRV_ERR_OUT_OF_MEMORY : cuda_fail(e);
    }
    b->blocks_per_sm = blocks_per_sm;
    b->grid = (opt && opt->grid_blocks > 0) ? opt->grid_blocks : resident;
    if (b->total_tiles < b->grid) b->grid = b->total_tiles > 0 ? int(b->total_tiles) : 1;
    *out = b;
    return TRV_OK;
}

int32_t trv_batch_create(const trv_task* tasks, uint64_t count, const trv_batch_options* opt, trv_batch** out) {
    return no_throw([&] { return batch_create_impl(tasks, count, opt, out); });
}

int32_t trv_batch_launch(trv_batch* b, void* stream) {
    if (!b || !on_batch_device(b)) return TRV_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (b->exec) {
        const cudaError_t e = cudaGraphLaunch(b->exec, st);
        return e == cudaSuccess ? TRV_OK : cuda_fail(e);
    }
    if (b->total_tiles == 0) return TRV_OK;
    cudaError_t e = cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_fail(e);
    e = launch_batch_kernel(b->d_tasks, b->ntasks, b->d_prefix, b->d_counter, b->grid, b->blocks_per_sm, st);
    return e == cudaSuccess ? TRV_OK : cuda_fail(e);
}

int32_t trv_batch_capture(trv_batch* b, void* stream) {
    if (!b || !stream || !on_batch_device(b)) return TRV_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
    }
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e);
    int rc = TRV_OK;
    if (b->total_tiles > 0) {
        e = cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned long long), st);
        if (e == cudaSuccess) e = launch_batch_kernel(b->d_tasks, b->ntasks, b->d_prefix, b->d_counter, b->grid, b->blocks_per_sm, st);
        if (e != cudaSuccess) rc = cuda_fail(e);
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(st, &g);
    if (rc != TRV_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e);
    cudaGraphExec_t x = nullptr;
    e = cudaGraphInstantiate(&x, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(e);
    }
    b->graph = g;
    b->exec = x;
    return TRV_OK;
}

int32_t trv_batch_info(const trv_batch* b, uint64_t* tiles, uint64_t* bytes) {
    if (!b) return TRV_ERR_INVALID_ARGUMENT;
    if (tiles) *tiles = uint64_t(b->total_tiles);
    if (bytes) *bytes = b->bytes;
    return TRV_OK;
}

int32_t trv_batch_destroy(trv_batch* b) {
    if (!b) return TRV_ERR_INVALID_ARGUMENT;
    release(b);
    delete b;
    return TRV_OK;
}

int32_t trv_run_per_call(const trv_task* tasks, uint64_t count, void* stream) {
    if (count > 0 && !tasks) return TRV_ERR_INVALID_ARGUMENT;
    for (uint64_t k = 0; k < count; ++k) {
        const trv_task& t = tasks[k];
        int rc;
        switch (t.op) {
            case TRV_OP_COPY: rc = trv_copy(t.dst, t.src, t.n, t.width, stream); break;
            case TRV_OP_GATHER: rc = trv_gather(t.dst, t.src, t.bound, t.idx, t.n, t.width, stream); break;
            case TRV_OP_SCATTER: rc = trv_scatter(t.dst, t.bound, t.src, t.idx, t.n, t.width, stream); break;
            default: rc = TRV_ERR_INVALID_ARGUMENT;
        }
        if (rc != TRV_OK) return rc;
    }
    return TRV_OK;
}

}  // extern "C"
