// Batched execution: many independent AoS arrays (copy / gather / scatter,
// any width 4..64 bytes in steps of 4) in ONE persistent kernel launch.
//
// The host splits every task into tiles of `tile_structs` structs (per task,
// chosen by the autotuner or a size rule) and uploads a task table plus the
// running tile count (tile_prefix).  The kernel is a device work queue: each
// CTA takes the next tile number from one atomic counter, finds its task by
// binary search over tile_prefix, and moves that tile with all of its warps,
// until the counter passes the last tile.  No per-array launch, no host
// round trip between arrays; one launch (or one CUDA graph replay: counter
// reset + kernel) runs the whole batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <new>
#include <vector>

#include "autotune.h"
#include "batch.h"
#include "kernels.cuh"
#include "runtime.h"
#include "trove_gb300.h"

namespace trv {
namespace {

constexpr int kBatchBlock = 256;
constexpr int kWarps = kBatchBlock / 32;

// ---- per-tile movers (all warps of the CTA cooperate on one tile) --------

// Flat copy of a byte range with the widest vector both pointers allow.
__device__ __forceinline__ void tile_copy_flat(const unsigned char* s, unsigned char* d, long long nbytes) {
    const int tid = threadIdx.x;
    const unsigned a = unsigned(reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d));
    long long done = 0;
    if ((a & 15u) == 0) {
        const long long nv = nbytes >> 4;
        const uint4* sv = reinterpret_cast<const uint4*>(s);
        uint4* dv = reinterpret_cast<uint4*>(d);
        for (long long k = tid; k < nv; k += 4 * kBatchBlock) {
            uint4 r[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (k + u * kBatchBlock < nv) r[u] = __ldg(sv + k + u * kBatchBlock);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (k + u * kBatchBlock < nv) __stcs(dv + k + u * kBatchBlock, r[u]);
        }
        done = nv << 4;
    } else if ((a & 3u) == 0) {
        const long long nv = nbytes >> 2;
        const unsigned* sv = reinterpret_cast<const unsigned*>(s);
        unsigned* dv = reinterpret_cast<unsigned*>(d);
        for (long long k = tid; k < nv; k += kBatchBlock) dv[k] = __ldg(sv + k);
        done = nv << 2;
    }
    for (long long b = done + tid; b < nbytes; b += kBatchBlock) d[b] = s[b];
}

// Device-API copy of structs [first, first + cnt): full 32-struct chunks with
// load/store_warp_contiguous, the ragged end per lane.
template <int S>
__device__ __forceinline__ void tile_copy_warp(const aos<S>* src, aos<S>* dst, long long first, long long cnt) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long end = first + cnt;
    for (long long base = first + warp * 32; base < end; base += kWarps * 32) {
        const long long i = base + lane;
        if (base + 32 <= end) {
            const aos<S> v = trove::load_warp_contiguous(src + i);
            trove::store_warp_contiguous(v, dst + i);
        } else if (i < end) {
            trove::detail::divergent_store(trove::detail::divergent_load(src + i), dst + i);
        }
    }
}

// Row-form gather / scatter over outputs (gather) or inputs (scatter)
// [first, first + cnt), words of V, U chunks of 32 per warp pass.
template <int S, typename V, int U, bool GATHER>
__device__ __forceinline__ void tile_index_rows(const V* src, V* dst, const int* idx, long long bound, long long first,
                                                long long cnt) {
    constexpr int m = S * 4 / int(sizeof(V));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long end = first + cnt;
    for (long long base = first + warp * 32 * U; base < end; base += kWarps * 32 * U) {
        int id[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + lane;
            const int v = i < end ? __ldg(idx + i) : -1;
            id[u] = (v >= 0 && (long long)v < bound) ? v : -1;
        }
        V val[U][m];
        int other[U][m];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int k = 0; k < m; ++k) {
                const int q = lane + 32 * k;
                const int j = q / m;
                other[u][k] = __shfl_sync(0xFFFFFFFFu, id[u], j);
                if (other[u][k] >= 0)
                    val[u][k] = GATHER ? __ldg(src + (long long)other[u][k] * m + (q - j * m))
                                       : __ldg(src + (base + u * 32) * m + q);
            }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int k = 0; k < m; ++k) {
                const int q = lane + 32 * k;
                if (other[u][k] >= 0) {
                    if (GATHER)
                        dst[(base + u * 32) * m + q] = val[u][k];
                    else
                        dst[(long long)other[u][k] * m + (q - (q / m) * m)] = val[u][k];
                }
            }
    }
}

// Unroll for the index movers: about 8 words of payload in flight per lane.
template <int S, typename V>
struct batch_unroll {
    static constexpr int m = S * 4 / int(sizeof(V));
    static constexpr int value = m >= 8 ? 1 : (m >= 4 ? 2 : (m >= 2 ? 4 : 8));
};

template <int S, bool GATHER>
__device__ __forceinline__ void tile_index(const BatchTask& t, long long first, long long cnt) {
    constexpr int wide = (S % 4 == 0) ? 16 : (S % 2 == 0) ? 8 : 4;
    const unsigned a = unsigned(reinterpret_cast<uintptr_t>(t.src) | reinterpret_cast<uintptr_t>(t.dst));
    if constexpr (wide == 16) {
        if ((a & 15u) == 0) {
            tile_index_rows<S, uint4, batch_unroll<S, uint4>::value, GATHER>(
                reinterpret_cast<const uint4*>(t.src), reinterpret_cast<uint4*>(t.dst), t.idx, t.bound, first, cnt);
            return;
        }
    }
    if constexpr (wide >= 8) {
        if ((a & 7u) == 0) {
            tile_index_rows<S, uint2, batch_unroll<S, uint2>::value, GATHER>(
                reinterpret_cast<const uint2*>(t.src), reinterpret_cast<uint2*>(t.dst), t.idx, t.bound, first, cnt);
            return;
        }
    }
    tile_index_rows<S, unsigned, batch_unroll<S, unsigned>::value, GATHER>(
        reinterpret_cast<const unsigned*>(t.src), reinterpret_cast<unsigned*>(t.dst), t.idx, t.bound, first, cnt);
}

template <int S>
__device__ __forceinline__ void run_tile(const BatchTask& t, long long first, long long cnt) {
    if (t.op == TRV_OP_COPY) {
        if (t.variant == TRV_PATH_WARP)
            tile_copy_warp<S>(reinterpret_cast<const aos<S>*>(t.src), reinterpret_cast<aos<S>*>(t.dst), first, cnt);
        else
            tile_copy_flat(t.src + first * 4 * S, t.dst + first * 4 * S, cnt * 4 * S);
    } else if (t.op == TRV_OP_GATHER) {
        tile_index<S, true>(t, first, cnt);
    } else {
        tile_index<S, false>(t, first, cnt);
    }
}

__global__ void __launch_bounds__(kBatchBlock)
batch_kernel(const BatchTask* __restrict__ tasks, int ntasks, const long long* __restrict__ tile_prefix,
             unsigned long long* counter) {
    __shared__ long long s_tile;
    const long long total = tile_prefix[ntasks];
    for (;;) {
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const long long tile = s_tile;
        __syncthreads();
        if (tile >= total) break;
        int lo = 0, hi = ntasks;  // tile_prefix[lo] <= tile < tile_prefix[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(tile_prefix + mid) <= tile)
                lo = mid;
            else
                hi = mid;
        }
        const BatchTask& t = tasks[lo];
        const long long first = (tile - __ldg(tile_prefix + lo)) * t.tile_structs;
        const long long cnt = t.n - first < t.tile_structs ? t.n - first : t.tile_structs;
        switch (t.words) {
            case 1: run_tile<1>(t, first, cnt); break;
            case 2: run_tile<2>(t, first, cnt); break;
            case 3: run_tile<3>(t, first, cnt); break;
            case 4: run_tile<4>(t, first, cnt); break;
            case 5: run_tile<5>(t, first, cnt); break;
            case 6: run_tile<6>(t, first, cnt); break;
            case 7: run_tile<7>(t, first, cnt); break;
            case 8: run_tile<8>(t, first, cnt); break;
            case 9: run_tile<9>(t, first, cnt); break;
            case 10: run_tile<10>(t, first, cnt); break;
            case 11: run_tile<11>(t, first, cnt); break;
            case 12: run_tile<12>(t, first, cnt); break;
            case 13: run_tile<13>(t, first, cnt); break;
            case 14: run_tile<14>(t, first, cnt); break;
            case 15: run_tile<15>(t, first, cnt); break;
            case 16: run_tile<16>(t, first, cnt); break;
        }
    }
}

}  // namespace

const void* batch_kernel_func() { return (const void*)&batch_kernel; }

cudaError_t launch_batch_kernel(const BatchTask* tasks, int ntasks, const long long* tile_prefix,
                                unsigned long long* counter, int grid, cudaStream_t st) {
    batch_kernel<<<grid, kBatchBlock, 0, st>>>(tasks, ntasks, tile_prefix, counter);
    return cudaGetLastError();
}

int batch_block_threads() { return kBatchBlock; }

}  // namespace trv
