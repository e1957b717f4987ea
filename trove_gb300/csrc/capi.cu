// C ABI entry points (include/trove_gb300.h): argument checks, path choice
// and launch shape, then one kernel launch on the caller's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <map>
#include <mutex>
#include <new>
#include <utility>
#include <vector>

#include "autotune.h"
#include "bulk.h"
#include "flat.h"
#include "ops.h"
#include "runtime.h"
#include "trove_gb300.h"

namespace trv {

thread_local int g_last_cuda_error = 0;

int cuda_fail(cudaError_t e) {
    g_last_cuda_error = int(e);
    return TRV_ERR_CUDA;
}

int check_launch() {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TRV_OK : cuda_fail(e);
}

DeviceInfo& device_info() {
    static std::mutex mu;
    static DeviceInfo infos[64];
    static std::map<int, DeviceInfo> more;  // devices past the array (map nodes never move)
    int dev = 0;
    cudaGetDevice(&dev);
    DeviceInfo* dp;
    if (dev >= 0 && dev < 64) {
        dp = &infos[dev];
    } else {
        std::lock_guard<std::mutex> g(mu);
        dp = &more[dev];
    }
    DeviceInfo& d = *dp;
    if (!d.ready.load(std::memory_order_acquire)) {
        std::lock_guard<std::mutex> g(mu);
        if (!d.ready.load(std::memory_order_relaxed)) {
            cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev);
            if (d.sm_count <= 0) d.sm_count = 1;
            d.device = dev;
            d.ready.store(true, std::memory_order_release);
        }
    }
    return d;
}

// The error flag is a module-scope device variable (one per device, zero at
// load), so finding it allocates nothing: callers that must not allocate
// (trv_batch_run_static) and stream capture can use it.  Resolve it outside
// a capture the first time (trv_batch_create and trv_server_create do).
__device__ int g_device_flag;

int* device_flag() {
    static std::mutex mu;
    DeviceInfo& d = device_info();
    std::lock_guard<std::mutex> g(mu);
    if (!d.flag) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_flag) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        d.flag = static_cast<int*>(p);
    }
    return d.flag;
}

int resident_blocks(const void* func, int block) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, int> cache;  // (device, kernel) at 256 threads
    DeviceInfo& d = device_info();
    const std::pair<int, const void*> key(d.device, func);
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find(key);
        if (it != cache.end() && block == 256) return it->second;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, block, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int r = per_sm * d.sm_count;
    if (block == 256) {
        std::lock_guard<std::mutex> g(mu);
        cache[key] = r;
    }
    return r;
}

int grid_for(const void* func, long long work_items, int items_per_block, int block, int requested) {
    if (requested > 0) return requested;
    long long need = (work_items + items_per_block - 1) / items_per_block;
    if (need < 1) need = 1;
    if (requested < 0) {  // persistent: no more blocks than can be resident at once
        const int cap = resident_blocks(func, block);
        return need < cap ? int(need) : cap;
    }
    return need < 0x7FFFFFFFll ? int(need) : 0x7FFFFFFF;  // one pass per warp
}

// True (and the grid) when the default launch applies: no grid requested and
// one 32*unroll-struct chunk per warp fits in a grid of 256-thread blocks.
bool one_chunk_per_warp(long long n, int unroll, int requested, int* grid) {
    if (requested != 0) return false;
    const long long per_block = 256ll * unroll;
    const long long need = (n + per_block - 1) / per_block;
    if (need < 1 || need > 0x7FFFFFFFll) return false;
    *grid = int(need);
    return true;
}

int unroll_slot(int unroll) {
    switch (unroll) {
        case 1: return 0;
        case 2: return 1;
        case 4: return 2;
        case 8: return 3;
    }
    return -1;
}

// Heuristic unroll when the caller gives none: about 16 words in flight per
// lane (tuned by the autotuner when a cache entry exists).
int default_unroll(unsigned width) {
    const unsigned words = width / 4;
    if (words <= 2) return 8;
    if (words <= 4) return 4;
    if (words <= 8) return 2;
    return 1;
}

}  // namespace trv

using namespace trv;

namespace {

bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

bool size_ok(uint64_t n, uint32_t width) { return width != 0 && n <= (uint64_t(1) << 62) / width; }

bool struct_width(uint32_t width) { return width % 4 == 0 && width >= 4 && width <= 64; }

int copy_flat(void* dst, const void* src, uint64_t nbytes, int unroll, int grid_req, cudaStream_t st) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(src), b = reinterpret_cast<uintptr_t>(dst);
    int vec = 16;
    while (vec > 1 && ((a ^ b) & uintptr_t(vec - 1)) != 0) vec >>= 1;
    long long head = (long long)((vec - (a & uintptr_t(vec - 1))) & uintptr_t(vec - 1));
    if ((uint64_t)head > nbytes) head = (long long)nbytes;
    if (unroll <= 0) unroll = 4;
    if (unroll_slot(unroll) < 0) return TRV_ERR_INVALID_ARGUMENT;
    const void* func = flat_copy_func(vec, unroll);
    const long long body = ((long long)nbytes - head) / vec;
    const int grid = grid_for(func, body, 256 * unroll, 256, grid_req);
    launch_flat_copy(src, dst, (long long)nbytes, vec, int(head), unroll, grid, st);
    return check_launch();
}

int copy_bulk(void* dst, const void* src, uint64_t nbytes, int chunk, int grid_req, cudaStream_t st) {
    if (!bulk_copy_supported(src, dst)) return TRV_ERR_MISALIGNED;
    if (chunk <= 0) chunk = 32 << 10;
    // chunk is bounded before the ring size is computed, which would overflow
    if (chunk % 16 != 0 || chunk > (227 << 10) || bulk_copy_smem_bytes(chunk) > (227 << 10))
        return TRV_ERR_INVALID_ARGUMENT;
    int* flag = device_flag();
    if (!flag) return TRV_ERR_OUT_OF_MEMORY;
    const long long nchunks = (long long)((nbytes + chunk - 1) / chunk);
    int grid = grid_req > 0 ? grid_req : device_info().sm_count;
    if (grid > nchunks) grid = nchunks > 0 ? int(nchunks) : 1;
    const cudaError_t e = launch_bulk_copy(src, dst, (long long)nbytes, chunk, grid, flag, st);
    return e == cudaSuccess ? TRV_OK : cuda_fail(e);
}

// Copy path without a tuned entry: the flat vector copy, one pass per warp.
// It needs no alignment beyond the bytes themselves and measured 7.0-7.1 TB/s
// on 2 GiB arrays at every width on GB300 (TMA bulk 6.8 TB/s; the device-API
// kernels 6.85-7.18 TB/s once tuned).
constexpr int kDefaultCopyPath = TRV_PATH_VECTOR;

}  // namespace

extern "C" {

const char* trv_status_string(int32_t status) {
    switch (status) {
        case TRV_OK: return "ok";
        case TRV_ERR_INVALID_ARGUMENT: return "invalid argument";
        case TRV_ERR_UNSUPPORTED: return "unsupported path/width combination";
        case TRV_ERR_MISALIGNED: return "pointer alignment not supported by the requested path";
        case TRV_ERR_CUDA: return "CUDA error";
        case TRV_ERR_OUT_OF_MEMORY: return "out of device memory";
        case TRV_ERR_BUDGET: return "request exceeds the HBM budget";
        case TRV_ERR_TIMEOUT: return "timed out";
        case TRV_ERR_NOT_FOUND: return "not found";
        case TRV_ERR_BUSY: return "busy";
        case TRV_ERR_CANCELLED: return "cancelled";
        case TRV_ERR_DEVICE_FLAG: return "a kernel reported an error";
    }
    return "unknown status";
}

int32_t trv_version(void) { return 100; }

int32_t trv_last_cuda_error(void) { return g_last_cuda_error; }

int32_t trv_set_l2_fetch_granularity(int32_t bytes, int32_t* previous) {
    if (bytes != 32 && bytes != 64 && bytes != 128) return TRV_ERR_INVALID_ARGUMENT;
    size_t old = 0;
    cudaError_t e = cudaDeviceGetLimit(&old, cudaLimitMaxL2FetchGranularity);
    if (e != cudaSuccess) return cuda_fail(e);
    e = cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, size_t(bytes));
    if (e != cudaSuccess) return cuda_fail(e);
    if (previous) *previous = int32_t(old);
    return TRV_OK;
}

int32_t trv_debug_set_bulk_wait_polls(uint32_t polls) {
    set_bulk_wait_polls(polls);
    return TRV_OK;
}

int32_t trv_check_device(void* stream) {
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e);
    int* flag = device_flag();
    if (!flag) return TRV_ERR_OUT_OF_MEMORY;
    int h = 0;
    e = cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e);
    if (h != 0) {
        e = cudaMemset(flag, 0, sizeof(int));
        if (e != cudaSuccess) return cuda_fail(e);
        return TRV_ERR_DEVICE_FLAG;
    }
    return TRV_OK;
}

int32_t trv_copy_ex(void* dst, const void* src, uint64_t n, uint32_t width, const trv_launch* cfg, void* stream) {
    if (!size_ok(n, width)) return TRV_ERR_INVALID_ARGUMENT;
    if (n == 0) return TRV_OK;
    if (!dst || !src) return TRV_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    trv_launch c = cfg ? *cfg : trv_launch{TRV_PATH_AUTO, 0, 0, 0, 0};
    if (c.block_threads != 0 && c.block_threads != 256) return TRV_ERR_UNSUPPORTED;
    if (c.path == TRV_PATH_AUTO) {
        TuneChoice t;
        if (tune_lookup(TuneKey{SCOPE_CALL, TRV_OP_COPY, int(width), len_bucket(n)}, &t) &&
            (t.path != TRV_PATH_BULK || bulk_copy_supported(src, dst)) &&
            (t.path != TRV_PATH_WARP || (struct_width(width) && aligned(dst, 4) && aligned(src, 4))))
            c = trv_launch{t.path, t.unroll, 0, t.grid, t.chunk, 0};
        else
            c.path = kDefaultCopyPath;
    }
    int path = c.path;
    const int unroll = c.unroll;
    const int grid_req = c.grid_blocks;
    if (path == TRV_PATH_VECTOR) return copy_flat(dst, src, n * width, unroll, grid_req, st);
    if (path == TRV_PATH_BULK) return copy_bulk(dst, src, n * width, c.chunk_bytes, grid_req, st);
    if (path != TRV_PATH_WARP && path != TRV_PATH_BLOCK && path != TRV_PATH_DIRECT) return TRV_ERR_UNSUPPORTED;
    if (!struct_width(width)) return TRV_ERR_UNSUPPORTED;
    if (!aligned(dst, 4) || !aligned(src, 4)) return TRV_ERR_MISALIGNED;
    const int u = unroll > 0 ? unroll : default_unroll(width);
    const int slot = unroll_slot(u);
    if (slot < 0) return TRV_ERR_INVALID_ARGUMENT;
    const int api = path == TRV_PATH_WARP ? 0 : path == TRV_PATH_BLOCK ? 1 : 2;
    const WidthOps* ops = ops_for_words(int(width / 4));
    const int ub = ops->built_unroll[slot];
    int grid = 0;
    const bool once = one_chunk_per_warp((long long)n, ub, grid_req, &grid);
    const CopyKernel& k = once ? ops->copy[api][slot] : ops->copy_grid[api][slot];
    if (!once) grid = grid_for(k.func, (long long)n, 256 * ub, 256, grid_req);
    k.launch(CopyArgs{src, dst, (long long)n, 0u}, grid, 256, st);
    return check_launch();
}

int32_t trv_copy(void* dst, const void* src, uint64_t n, uint32_t width, void* stream) {
    return trv_copy_ex(dst, src, n, width, nullptr, stream);
}

int32_t trv_copy_exit_ex(void* dst, const void* src, uint64_t n, uint32_t width, uint32_t modulus,
                         const trv_launch* cfg, void* stream) {
    if (!size_ok(n, width) || !cfg) return TRV_ERR_INVALID_ARGUMENT;
    if (n == 0) return TRV_OK;
    if (!dst || !src) return TRV_ERR_INVALID_ARGUMENT;
    if (!struct_width(width)) return TRV_ERR_UNSUPPORTED;
    if (cfg->path != TRV_PATH_WARP && cfg->path != TRV_PATH_BLOCK) return TRV_ERR_UNSUPPORTED;
    if (cfg->block_threads != 0 && cfg->block_threads != 256) return TRV_ERR_UNSUPPORTED;
    if (!aligned(dst, 4) || !aligned(src, 4)) return TRV_ERR_MISALIGNED;
    int u = cfg->unroll, grid_req = cfg->grid_blocks;
    if (u == 0) {
        TuneChoice t;
        const int op = cfg->path == TRV_PATH_WARP ? TRV_OP_COPY_EXIT_WARP : TRV_OP_COPY_EXIT_BLOCK;
        if (tune_lookup(TuneKey{SCOPE_CALL, op, int(width), len_bucket(n)}, &t)) {
            u = t.unroll;
            if (grid_req == 0) grid_req = t.grid;
        } else {
            u = default_unroll(width);
        }
    }
    const int slot = unroll_slot(u);
    if (slot < 0) return TRV_ERR_INVALID_ARGUMENT;
    const int api = cfg->path == TRV_PATH_WARP ? 0 : 1;
    const WidthOps* ops = ops_for_words(int(width / 4));
    const int ub = ops->built_unroll[slot];
    int grid = 0;
    const bool once = one_chunk_per_warp((long long)n, ub, grid_req, &grid);
    const CopyKernel& k = once ? ops->copy_exit[api][slot] : ops->copy_exit_grid[api][slot];
    if (!once) grid = grid_for(k.func, (long long)n, 256 * ub, 256, grid_req);
    k.launch(CopyArgs{src, dst, (long long)n, modulus}, grid, 256, static_cast<cudaStream_t>(stream));
    return check_launch();
}

int32_t trv_copy_exit(void* dst, const void* src, uint64_t n, uint32_t width, uint32_t modulus, int32_t path,
                      void* stream) {
    trv_launch cfg = {path, 0, 0, 0, 0, 0};
    return trv_copy_exit_ex(dst, src, n, width, modulus, &cfg, stream);
}

// Destination bytes one pass of a blocked scatter (cache policy 6) covers.
// A random store of a struct narrower than a 32-byte sector is a partial-sector
// write; when the destination is much larger than L2, the sector leaves L2
// before its other structs arrive and DRAM must read, merge and write it.
// Taking only the indices that land in one L2-sized part of the destination
// per pass lets the partial writes merge in L2 (each pass re-reads the index
// and source arrays).  Measured on 2^24-struct permutation scatters of the
// row-form kernel: +53 / +33 / +23 % at 8 / 12 / 16 bytes (2-4 passes);
// at 20 and 24 bytes the 5-6 passes cost more than they save (-25 / -16 %).
constexpr long long kScatterPassBytes = 64ll << 20;

// The blocked scatter pays for narrow structs whose destination exceeds a
// pass and that most of the destination's rows receive.
static bool blocked_scatter_pays(uint32_t width, uint64_t n, uint64_t dst_n) {
    return width <= 16 && (long long)(dst_n * width) > kScatterPassBytes && 2 * n >= dst_n;
}

// Without a tuned entry, struct gathers and scatters take the row-form path
// with 2 structs per lane, streaming index and contiguous side, and (gather)
// random loads with the 64-byte L2 prefetch hint (policy 4): measured on
// GB300 with L2 flushed, the best or within 1 % of the best at every width
// from 8 to 64 bytes on permutations, runs of 32 and the identity.  Narrow
// scatters onto large destinations run in destination passes (policy 6).
static int32_t index_op(bool gather, void* dst, const void* src, uint64_t bound, const int32_t* idx, uint64_t n,
                        uint32_t width, const trv_launch* cfg, void* stream) {
    if (!size_ok(n, width) || !size_ok(bound, width)) return TRV_ERR_INVALID_ARGUMENT;
    if (n == 0) return TRV_OK;
    if (!dst || !src || !idx) return TRV_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    trv_launch c = cfg ? *cfg : trv_launch{TRV_PATH_AUTO, 0, 0, 0, 0};
    if (c.block_threads != 0 && c.block_threads != 256) return TRV_ERR_UNSUPPORTED;
    if (!aligned(idx, 4)) return TRV_ERR_MISALIGNED;
    const bool structs = struct_width(width) && aligned(dst, 4) && aligned(src, 4);
    const bool wide_words = width % 4 == 0 && width > 64 && aligned(dst, 4) && aligned(src, 4);
    if (c.path == TRV_PATH_AUTO) {
        TuneChoice t;
        if (structs && tune_lookup(TuneKey{SCOPE_CALL, gather ? TRV_OP_GATHER : TRV_OP_SCATTER, int(width),
                                           len_bucket(n)},
                                   &t))
            c = trv_launch{t.path, t.unroll, 0, t.grid, 0, t.cache_policy};
        else if (structs)
            c = trv_launch{TRV_PATH_WARP, 2, 0, 0, 0, gather ? 4 : blocked_scatter_pays(width, n, bound) ? 6 : 1};
        else
            c.path = wide_words ? TRV_PATH_WARP : TRV_PATH_VECTOR;
    }
    if (c.cache_policy < 0 || c.cache_policy > 6 || (gather && c.cache_policy == 6)) return TRV_ERR_INVALID_ARGUMENT;
    const int path = c.path;
    const int grid_req = c.grid_blocks;
    if (path == TRV_PATH_VECTOR) {  // generic byte-wise form
        const long long blocks = (long long)((n + 255) / 256);
        const int cap = device_info().sm_count * 8;
        const int g = grid_req > 0 ? grid_req : (blocks < cap ? int(blocks) : cap);
        if (gather)
            launch_gather_bytes(src, (long long)bound, idx, dst, (long long)n, width, g, st);
        else
            launch_scatter_bytes(src, idx, dst, (long long)bound, (long long)n, width, g, st);
        return check_launch();
    }
    if (path != TRV_PATH_COALESCED && path != TRV_PATH_DIRECT && path != TRV_PATH_WARP) return TRV_ERR_UNSUPPORTED;
    if (path == TRV_PATH_WARP && width % 4 == 0 && width > 64) {  // run-time word count
        if (!aligned(dst, 4) || !aligned(src, 4)) return TRV_ERR_MISALIGNED;
        int wb = 16;
        while (wb > 4 && (width % uint32_t(wb) != 0 || !aligned(dst, uintptr_t(wb)) || !aligned(src, uintptr_t(wb))))
            wb >>= 1;
        const long long warps = (long long)((n + 31) / 32);
        const int grid = grid_for(index_rows_rt_func(gather, wb), warps, 8, 256, grid_req);
        launch_index_rows_rt(gather, wb, IndexArgs{src, dst, idx, (long long)n, (long long)bound, c.cache_policy},
                             int(width / uint32_t(wb)), grid, st);
        return check_launch();
    }
    if (!struct_width(width)) return TRV_ERR_UNSUPPORTED;
    if (!aligned(dst, 4) || !aligned(src, 4)) return TRV_ERR_MISALIGNED;
    const int u = c.unroll > 0 ? c.unroll : default_unroll(width);
    const int slot = unroll_slot(u);
    if (slot < 0) return TRV_ERR_INVALID_ARGUMENT;
    const WidthOps* ops = ops_for_words(int(width / 4));
    const IndexKernel* kp;
    if (path == TRV_PATH_WARP) {
        const uintptr_t wb = uintptr_t(ops->rows_word_bytes);
        const int var = (aligned(dst, wb) && aligned(src, wb)) ? 0 : 1;
        kp = gather ? &ops->gather_rows[var][slot] : &ops->scatter_rows[var][slot];
    } else {
        const int mode = path == TRV_PATH_COALESCED ? 0 : 1;
        kp = gather ? &ops->gather[mode][slot] : &ops->scatter[mode][slot];
    }
    const IndexKernel& k = *kp;
    const int grid = grid_for(k.func, (long long)n, 256 * ops->built_unroll[slot], 256, grid_req);
    if (!gather && path == TRV_PATH_WARP && c.cache_policy == 6) {  // destination passes
        const long long dst_bytes = (long long)bound * (long long)width;
        long long passes = (dst_bytes + kScatterPassBytes - 1) / kScatterPassBytes;
        passes = passes < 1 ? 1 : passes > 16 ? 16 : passes;
        for (long long p = 0; p < passes; ++p) {
            IndexArgs a{src, dst, idx, (long long)n, (long long)bound * (p + 1) / passes, 1};
            a.lo = (long long)bound * p / passes;
            k.launch(a, grid, 256, st);
        }
        return check_launch();
    }
    k.launch(IndexArgs{src, dst, idx, (long long)n, (long long)bound, c.cache_policy}, grid, 256, st);
    return check_launch();
}

int32_t trv_gather_ex(void* dst, const void* src, uint64_t src_n, const int32_t* idx, uint64_t n, uint32_t width,
                      const trv_launch* cfg, void* stream) {
    return index_op(true, dst, src, src_n, idx, n, width, cfg, stream);
}

int32_t trv_gather(void* dst, const void* src, uint64_t src_n, const int32_t* idx, uint64_t n, uint32_t width,
                   void* stream) {
    return index_op(true, dst, src, src_n, idx, n, width, nullptr, stream);
}

int32_t trv_scatter_ex(void* dst, uint64_t dst_n, const void* src, const int32_t* idx, uint64_t n, uint32_t width,
                       const trv_launch* cfg, void* stream) {
    return index_op(false, dst, src, dst_n, idx, n, width, cfg, stream);
}

int32_t trv_scatter(void* dst, uint64_t dst_n, const void* src, const int32_t* idx, uint64_t n, uint32_t width,
                    void* stream) {
    return index_op(false, dst, src, dst_n, idx, n, width, nullptr, stream);
}

static int32_t layout_op(bool to_soa, void* dst, const void* src, uint64_t n, uint32_t width, const trv_launch* cfg,
                         void* stream) {
    if (!size_ok(n, width)) return TRV_ERR_INVALID_ARGUMENT;
    if (n == 0) return TRV_OK;
    if (!dst || !src) return TRV_ERR_INVALID_ARGUMENT;
    if (!struct_width(width)) return TRV_ERR_UNSUPPORTED;
    if (!aligned(dst, 4) || !aligned(src, 4)) return TRV_ERR_MISALIGNED;
    if (cfg && cfg->block_threads != 0 && cfg->block_threads != 256) return TRV_ERR_UNSUPPORTED;
    int u = cfg ? cfg->unroll : 0;
    int grid_req = cfg ? cfg->grid_blocks : 0;
    if (u == 0) {
        TuneChoice t;
        if (tune_lookup(TuneKey{SCOPE_CALL, to_soa ? TRV_OP_AOS_TO_SOA : TRV_OP_SOA_TO_AOS, int(width), len_bucket(n)},
                        &t)) {
            u = t.unroll;
            if (grid_req == 0) grid_req = t.grid;
        } else {
            u = default_unroll(width);
        }
    }
    const int slot = unroll_slot(u);
    if (slot < 0) return TRV_ERR_INVALID_ARGUMENT;
    const WidthOps* ops = ops_for_words(int(width / 4));
    const int ub = ops->built_unroll[slot];
    int grid = 0;
    const bool once = one_chunk_per_warp((long long)n, ub, grid_req, &grid);
    const CopyKernel& k = once ? (to_soa ? ops->aos_to_soa[slot] : ops->soa_to_aos[slot])
                               : (to_soa ? ops->aos_to_soa_grid[slot] : ops->soa_to_aos_grid[slot]);
    if (!once) grid = grid_for(k.func, (long long)n, 256 * ub, 256, grid_req);
    k.launch(CopyArgs{src, dst, (long long)n, 0u}, grid, 256, static_cast<cudaStream_t>(stream));
    return check_launch();
}

int32_t trv_aos_to_soa(void* dst_soa, const void* src_aos, uint64_t n, uint32_t width, void* stream) {
    return layout_op(true, dst_soa, src_aos, n, width, nullptr, stream);
}

int32_t trv_soa_to_aos(void* dst_aos, const void* src_soa, uint64_t n, uint32_t width, void* stream) {
    return layout_op(false, dst_aos, src_soa, n, width, nullptr, stream);
}

int32_t trv_aos_to_soa_ex(void* dst_soa, const void* src_aos, uint64_t n, uint32_t width, const trv_launch* cfg,
                          void* stream) {
    return layout_op(true, dst_soa, src_aos, n, width, cfg, stream);
}

int32_t trv_soa_to_aos_ex(void* dst_aos, const void* src_soa, uint64_t n, uint32_t width, const trv_launch* cfg,
                          void* stream) {
    return layout_op(false, dst_aos, src_soa, n, width, cfg, stream);
}

int32_t trv_fill_uniform_indices(int32_t* idx, uint64_t n, uint32_t bound, uint64_t seed, void* stream) {
    if (n == 0) return TRV_OK;
    if (!idx || bound == 0 || bound > 0x7FFFFFFFu || n > (uint64_t(1) << 61)) return TRV_ERR_INVALID_ARGUMENT;
    if (!aligned(idx, 4)) return TRV_ERR_MISALIGNED;
    launch_uniform_indices(idx, (long long)n, bound, seed, device_info().sm_count * 8,
                           static_cast<cudaStream_t>(stream));
    return check_launch();
}

int32_t trv_fill_run_indices(int32_t* idx, uint64_t n, uint64_t seed, void* stream) {
    if (n == 0) return TRV_OK;
    if (!idx || n < 32 || n > 0x7FFFFFFFull) return TRV_ERR_INVALID_ARGUMENT;
    if (!aligned(idx, 4)) return TRV_ERR_MISALIGNED;
    launch_run_indices(idx, (long long)n, seed, device_info().sm_count * 8, static_cast<cudaStream_t>(stream));
    return check_launch();
}

int32_t trv_fill_permutation(int32_t* idx, uint64_t n, uint64_t seed, void* stream) {
    if (n == 0) return TRV_OK;
    if (!idx || n > 0x7FFFFFFFull) return TRV_ERR_INVALID_ARGUMENT;
    if (!aligned(idx, 4)) return TRV_ERR_MISALIGNED;
    // Fisher-Yates from the top: step i (i = n .. 2) swaps slot i - 1 with a
    // slot drawn from word i over [0, i).  Inherently sequential, so it runs
    // on the host and the result is copied once.
    std::vector<int32_t> h;
    try {
        h.resize(n);
    } catch (const std::bad_alloc&) {
        return TRV_ERR_OUT_OF_MEMORY;
    }
    for (uint64_t i = 0; i < n; ++i) h[i] = int32_t(i);
    for (uint64_t i = n; i > 1; --i) std::swap(h[i - 1], h[stream_bounded(seed, i, unsigned(i))]);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(idx, h.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // h is freed on return
    return e == cudaSuccess ? TRV_OK : cuda_fail(e);
}

int32_t trv_fill_random_u32(uint32_t* dst, uint64_t nwords, uint64_t seed, void* stream) {
    if (nwords == 0) return TRV_OK;
    if (!dst || nwords > (uint64_t(1) << 61)) return TRV_ERR_INVALID_ARGUMENT;
    const int grid = device_info().sm_count * 8;
    launch_fill_u32(dst, (long long)nwords, seed, grid, static_cast<cudaStream_t>(stream));
    return check_launch();
}

}  // extern "C"
