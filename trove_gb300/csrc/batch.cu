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

// Thread position read through volatile asm: the movers' lane-derived
// constants are then recomputed per tile instead of being hoisted out of the
// persistent loop for every (op, width) case at once, which would keep
// hundreds of them live and spill.
__device__ __forceinline__ int opaque_tid() {
    int t;
    asm volatile("mov.u32 %0, %%tid.x;" : "=r"(t));
    return t;
}

// Flat copy of a byte range with the widest vector both pointers allow.
__device__ __forceinline__ void tile_copy_flat(const unsigned char* s, unsigned char* d, long long nbytes) {
    const int tid = opaque_tid();
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

// Row-form gather / scatter over outputs (gather) or inputs (scatter)
// [first, first + cnt) in words of V, m words per struct given at run time
// (so one mover serves every width).  Each warp pass moves U chunks of 32
// structs; a chunk's m rounds run in groups of G (loads of the group, then its
// stores).  Round k, lane l: word q = l + 32k of the chunk, i.e. word q % m of
// struct q / m, whose index comes from that struct's lane by one shuffle.  m is
// uniform across the warp, so the guarded shuffles are too.
template <typename V, int U, int G, bool GATHER>
__device__ __forceinline__ void tile_index_rows(const V* src, V* dst, const int* idx, long long bound, long long first,
                                                long long cnt, int m, bool hint) {
    const int tid = opaque_tid();
    const int lane = tid & 31, warp = tid >> 5;
    const long long end = first + cnt;
    for (long long base = first + warp * 32 * U; base < end; base += kWarps * 32 * U) {
        int id[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + lane;
            const int v = i < end ? __ldcs(idx + i) : -1;
            id[u] = (v >= 0 && (long long)v < bound) ? v : -1;
        }
        for (int k0 = 0; k0 < m; k0 += G) {
            V val[U][G];
            int other[U][G];
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const int k = k0 + g;
                    other[u][g] = -1;
                    if (k < m) {
                        const int q = lane + 32 * k;
                        const int j = q / m;
                        other[u][g] = __shfl_sync(0xFFFFFFFFu, id[u], j);
                        if (other[u][g] >= 0)
                            val[u][g] = !GATHER ? __ldcs(src + (base + u * 32) * m + q)
                                        : hint  ? ld_pf64(src + (long long)other[u][g] * m + (q - j * m))
                                                : __ldg(src + (long long)other[u][g] * m + (q - j * m));
                    }
                }
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (other[u][g] < 0) continue;
                    const int q = lane + 32 * (k0 + g);
                    if (GATHER)
                        __stcs(dst + (base + u * 32) * m + q, val[u][g]);
                    else
                        dst[(long long)other[u][g] * m + (q % m)] = val[u][g];
                }
        }
    }
}

template <bool GATHER>
__device__ __forceinline__ void tile_index(const BatchTask& t, long long first, long long cnt) {
    const int m = t.words * 4 >> t.word_log2;
    if (t.word_log2 == 4)
        tile_index_rows<uint4, 2, 2, GATHER>(reinterpret_cast<const uint4*>(t.src), reinterpret_cast<uint4*>(t.dst),
                                             t.idx, t.bound, first, cnt, m, t.l2_hint != 0);
    else if (t.word_log2 == 3)
        tile_index_rows<uint2, 2, 4, GATHER>(reinterpret_cast<const uint2*>(t.src), reinterpret_cast<uint2*>(t.dst),
                                             t.idx, t.bound, first, cnt, m, t.l2_hint != 0);
    else
        tile_index_rows<unsigned, 2, 4, GATHER>(reinterpret_cast<const unsigned*>(t.src),
                                                reinterpret_cast<unsigned*>(t.dst), t.idx, t.bound, first, cnt, m,
                                                t.l2_hint != 0);
}

// MINB resident blocks per SM: 2 gives each thread 128 registers (no
// spills), 4 gives 64 (a few spilled words, twice the warps for latency
// hiding); the batch options or the autotuner pick one.
template <int MINB>
__global__ void __launch_bounds__(kBatchBlock, MINB)
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
        const long long w = 4ll * t.words;
        if (t.op == TRV_OP_COPY)
            tile_copy_flat(t.src + first * w, t.dst + first * w, cnt * w);
        else if (t.op == TRV_OP_GATHER)
            tile_index<true>(t, first, cnt);
        else
            tile_index<false>(t, first, cnt);
    }
}

}  // namespace

const void* batch_kernel_func(int blocks_per_sm) {
    return blocks_per_sm == 2 ? (const void*)&batch_kernel<2> : (const void*)&batch_kernel<4>;
}

cudaError_t launch_batch_kernel(const BatchTask* tasks, int ntasks, const long long* tile_prefix,
                                unsigned long long* counter, int grid, int blocks_per_sm, cudaStream_t st) {
    if (blocks_per_sm == 2)
        batch_kernel<2><<<grid, kBatchBlock, 0, st>>>(tasks, ntasks, tile_prefix, counter);
    else
        batch_kernel<4><<<grid, kBatchBlock, 0, st>>>(tasks, ntasks, tile_prefix, counter);
    return cudaGetLastError();
}

int batch_block_threads() { return kBatchBlock; }

}  // namespace trv
