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
#include <mutex>
#include <new>
#include <vector>

#include "autotune.h"
#include "batch.h"
#include "kernels.cuh"
#include "runtime.h"
#include "tma.cuh"
#include "trove_gb300.h"

namespace trv {
namespace {

// Copy tiles whose source and destination are 16-byte aligned move through
// the TMA bulk engine: one thread streams the tile as kBulkChunk pieces
// through a ring of shared-memory stages (load, then store of each piece; a
// stage is refilled once the store that read it has finished).  The bytes in
// flight then come from shared memory, not from registers.
constexpr int kBulkChunk = 8 << 10;

// Launch shapes of the persistent kernel: block size, resident blocks per SM
// it is built for (hence the register budget), the staged gather / scatter
// piece with its index slots, and the copy ring's stages.  Staged movers
// cycle through two pieces per block; four per block measured slower (18.5
// vs 14.9 ms for the 4096-array batch's gathers at 2 blocks per SM): more
// resident blocks is what pays (12.1 ms at 4), as block barriers then
// overlap.  128-thread blocks, 8 per SM, with 8 KiB pieces measured no
// better (23.8 vs 22.9 ms for the whole batch).  The copy ring reuses the
// piece buffers.  Either shape holds 160 KiB of shared memory per SM.
template <int BLOCK, int MINB, int PIECE, int RING>
struct Shape {
    static constexpr int block = BLOCK;
    static constexpr int warps = BLOCK / 32;
    static constexpr int minb = MINB;
    static constexpr int piece = PIECE;           // bytes of one staged piece
    static constexpr int idx_slots = PIECE / 16;  // indices of one staged piece
    static constexpr int ring = RING;             // copy stages of kBulkChunk bytes
    static constexpr int dyn_smem = 2 * (PIECE + idx_slots * int(sizeof(int)));
    static_assert(RING * kBulkChunk <= 2 * PIECE, "the copy ring fits the piece buffers");
};
using Shape2 = Shape<256, 2, 16 << 10, 4>;  // 128 registers per thread
using Shape4 = Shape<256, 4, 16 << 10, 4>;  // 64 registers

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
template <class S>
__device__ __forceinline__ void tile_copy_flat(const unsigned char* s, unsigned char* d, long long nbytes) {
    const int tid = opaque_tid();
    const unsigned a = unsigned(reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d));
    long long done = 0;
    if ((a & 15u) == 0) {
        const long long nv = nbytes >> 4;
        const uint4* sv = reinterpret_cast<const uint4*>(s);
        uint4* dv = reinterpret_cast<uint4*>(d);
        for (long long k = tid; k < nv; k += 4 * S::block) {
            uint4 r[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (k + u * S::block < nv) r[u] = __ldg(sv + k + u * S::block);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (k + u * S::block < nv) __stcs(dv + k + u * S::block, r[u]);
        }
        done = nv << 4;
    } else if ((a & 3u) == 0) {
        const long long nv = nbytes >> 2;
        const unsigned* sv = reinterpret_cast<const unsigned*>(s);
        unsigned* dv = reinterpret_cast<unsigned*>(d);
        for (long long k = tid; k < nv; k += S::block) dv[k] = __ldg(sv + k);
        done = nv << 2;
    }
    for (long long b = done + tid; b < nbytes; b += S::block) d[b] = s[b];
}

// TMA bulk copy of one tile by the calling thread (thread 0 of the CTA).
// `seq` numbers the loads this CTA has issued over the whole launch: load k
// uses stage k % S and completes phase (k / S) & 1 of that stage's
// mbarrier.  Every wait is bounded; on a timeout the device flag is set, the
// loads still in flight are drained (bounded) and false is returned.
template <class S>
__device__ bool tile_copy_bulk(const unsigned char* s, unsigned char* d, long long nbytes, unsigned char* stage,
                               unsigned long long* bar, unsigned long long& seq, int* flag) {
    const long long body = nbytes & ~15ll;
    const long long nchunks = (body + kBulkChunk - 1) / kBulkChunk;
    auto chunk_bytes = [&](long long c) -> unsigned {
        const long long off = c * kBulkChunk;
        return static_cast<unsigned>(body - off < kBulkChunk ? body - off : kBulkChunk);
    };
    auto issue = [&](long long c) {
        const int st = int((seq + (unsigned long long)c) % S::ring);
        mbar_expect_tx(&bar[st], chunk_bytes(c));
        bulk_load(stage + (size_t)st * kBulkChunk, s + c * kBulkChunk, chunk_bytes(c), &bar[st]);
    };
    const long long prologue = nchunks < S::ring ? nchunks : S::ring;
    fence_proxy_async_shared();  // earlier generic-proxy use of the stages (gather tiles) before TMA writes
    for (long long c = 0; c < prologue; ++c) issue(c);
    long long issued = prologue;
    bool ok = true;
    long long c = 0;
    for (; c < nchunks; ++c) {
        const unsigned long long k = seq + (unsigned long long)c;
        const int st = int(k % S::ring);
        if (!mbar_wait(&bar[st], unsigned((k / S::ring) & 1))) {
            ok = false;
            break;
        }
        fence_proxy_async_shared();
        bulk_store(d + c * kBulkChunk, stage + (size_t)st * kBulkChunk, chunk_bytes(c));
        if (c >= 1 && issued < nchunks) {
            bulk_wait_read_1();  // the previous piece's store has read its stage
            issue(issued++);
        }
    }
    if (!ok) {
        atomicExch(flag, 1);
        for (long long j = c; j < issued; ++j) {
            const unsigned long long k = seq + (unsigned long long)j;
            mbar_wait(&bar[k % S::ring], unsigned((k / S::ring) & 1));
        }
    }
    bulk_wait_read_0();  // stages free for the next tile
    seq += (unsigned long long)issued;
    for (long long b = body; b < nbytes; ++b) d[b] = s[b];
    return ok;
}

// Row-form gather / scatter over outputs (gather) or inputs (scatter)
// [first, first + cnt) in words of V, m words per struct given at run time
// (so one mover serves every width).  Each warp pass moves U chunks of 32
// structs; a chunk's m rounds run in groups of G (loads of the group, then its
// stores).  Round k, lane l: word q = l + 32k of the chunk, i.e. word q % m of
// struct q / m, whose index comes from that struct's lane by one shuffle.  m is
// uniform across the warp, so the guarded shuffles are too.
template <class S, typename V, int U, int G, bool GATHER>
__device__ __forceinline__ void tile_index_rows(const V* src, V* dst, const int* idx, long long bound, long long first,
                                                long long cnt, int m, bool hint) {
    const int tid = opaque_tid();
    const int lane = tid & 31, warp = tid >> 5;
    const long long end = first + cnt;
    for (long long base = first + warp * 32 * U; base < end; base += S::warps * 32 * U) {
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

// Gather / scatter of the structs [first, first + cnt) of the contiguous side
// staged through shared memory with cp.async.  Gather: the warps issue
// asynchronous word copies from the random source rows straight into a
// shared-memory buffer (no registers hold the data in flight, so far more of
// it can be), then write the buffer out to the contiguous destination with
// coalesced stores.  Scatter: the contiguous source piece is copied in the
// same way, then each word is stored to its random destination row from
// shared memory (stores need no registers held in flight either).  Two
// buffers of S::piece bytes alternate, so the next piece's copies are in
// flight while the current one is written.  Word q of a piece (words of
// sizeof(V)) belongs to struct q / m; the piece's indices are staged in
// shared memory first (one coalesced read), invalid ones marked -1.  PF is
// the L2 prefetch size the random row copies ask for on a miss: 0 the
// context's fetch granularity, 64 or 128 bytes (GB300s differ in their
// default, and the best size depends on the struct width).
template <int PF>
__device__ __forceinline__ void cp_async_word(void* smem, const void* gmem, int bytes) {
    const unsigned s = smem_addr(smem);
    if (PF == 64) {
        if (bytes == 16)
            asm volatile("cp.async.cg.shared.global.L2::64B [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
        else if (bytes == 8)
            asm volatile("cp.async.ca.shared.global.L2::64B [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
        else
            asm volatile("cp.async.ca.shared.global.L2::64B [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
    } else if (PF == 128) {
        if (bytes == 16)
            asm volatile("cp.async.cg.shared.global.L2::128B [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
        else if (bytes == 8)
            asm volatile("cp.async.ca.shared.global.L2::128B [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
        else
            asm volatile("cp.async.ca.shared.global.L2::128B [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
    } else {
        if (bytes == 16)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
        else if (bytes == 8)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
    }
}

// Waits until at most n of this thread's cp.async groups are pending.
__device__ __forceinline__ void cp_async_wait_pending(int n) {
    if (n <= 0)
        asm volatile("cp.async.wait_group 0;" ::: "memory");
    else if (n == 1)
        asm volatile("cp.async.wait_group 1;" ::: "memory");
    else if (n == 2)
        asm volatile("cp.async.wait_group 2;" ::: "memory");
    else
        asm volatile("cp.async.wait_group 3;" ::: "memory");
}

// Copies `bytes` (a multiple of sizeof(V)) of a contiguous range from global to
// shared memory with cp.async, 16 bytes a copy when both ends are 16-byte
// aligned (a scatter's source piece: 2 % faster scatters than copies of V).
template <class S, typename V>
__device__ __forceinline__ void cp_async_range(V* smem, const V* gmem, int bytes, int tid) {
    if (((reinterpret_cast<uintptr_t>(smem) | reinterpret_cast<uintptr_t>(gmem)) & 15u) == 0) {
        const int n16 = bytes >> 4;
        for (int k = tid; k < n16; k += S::block)
            cp_async_word<0>(reinterpret_cast<uint4*>(smem) + k, reinterpret_cast<const uint4*>(gmem) + k, 16);
        const int done = (n16 << 4) / int(sizeof(V));
        const int tail = bytes / int(sizeof(V)) - done;
        if (tid < tail) cp_async_word<0>(smem + done + tid, gmem + done + tid, int(sizeof(V)));
    } else {
        const int words = bytes / int(sizeof(V));
        for (int q = tid; q < words; q += S::block) cp_async_word<0>(smem + q, gmem + q, int(sizeof(V)));
    }
}

template <class S, typename V, bool GATHER, int PF>
__device__ void tile_index_staged(const V* src, V* dst, const int* idx, long long bound, long long first,
                                  long long cnt, int m, unsigned char* stage, int* s_idx) {
    constexpr int D = 2;
    const int tid = opaque_tid();
    // structs per piece: a multiple of 32 that fits the buffer and the index slots
    int per = (S::piece / int(sizeof(V))) / m / 32 * 32;
    if (per > S::idx_slots) per = S::idx_slots;
    // q / m for q < 2^12 and m <= 16 as a multiply and shift (exact there)
    const unsigned inv_m = (65536u + unsigned(m) - 1) / unsigned(m);
    const long long pieces = (cnt + per - 1) / per;
    auto issue = [&](long long p) {
        const int b = int(p % D);
        V* buf = reinterpret_cast<V*>(stage + b * S::piece);
        int* ix = s_idx + b * S::idx_slots;
        const long long base = first + p * per;
        const int n_here = int(cnt - p * per < per ? cnt - p * per : per);
        const int words = n_here * m;
        if (GATHER) {
            for (int j = tid; j < n_here; j += S::block) {
                const int v = __ldcs(idx + base + j);
                ix[j] = (v >= 0 && (long long)v < bound) ? v : -1;
            }
            __syncthreads();  // the copies below read the staged indices
            for (int q = tid; q < words; q += S::block) {
                const int j = int((unsigned(q) * inv_m) >> 16);
                const int v = ix[j];
                if (v >= 0) cp_async_word<PF>(buf + q, src + (long long)v * m + (q - j * m), int(sizeof(V)));
            }
        } else {  // raw indices and source words, both read after the wait's barrier
            cp_async_range<S>(ix, idx + base, n_here * 4, tid);
            cp_async_range<S>(buf, src + base * m, words * int(sizeof(V)), tid);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    auto drain = [&](long long p) {
        const int b = int(p % D);
        const V* buf = reinterpret_cast<const V*>(stage + b * S::piece);
        const int* ix = s_idx + b * S::idx_slots;
        const long long base = first + p * per;
        const int n_here = int(cnt - p * per < per ? cnt - p * per : per);
        const int words = n_here * m;
        for (int q = tid; q < words; q += S::block) {
            const int j = int((unsigned(q) * inv_m) >> 16);
            const int v = ix[j];
            if (v < 0 || (!GATHER && (long long)v >= bound)) continue;  // gather slots hold -1 when invalid
            if (GATHER)
                __stcs(dst + base * m + q, buf[q]);
            else
                dst[(long long)v * m + (q - j * m)] = buf[q];
        }
    };
    for (long long p = 0; p < D - 1 && p < pieces; ++p) issue(p);
    for (long long p = 0; p < pieces; ++p) {
        // buffer (p + D - 1) % D was drained in the previous iteration
        if (p + D - 1 < pieces) issue(p + D - 1);
        // groups committed: min(p + D, pieces); piece p's must be complete
        const long long later = pieces - 1 - p;
        cp_async_wait_pending(later < D - 1 ? int(later) : D - 1);
        __syncthreads();
        drain(p);
        __syncthreads();  // buffer and index slots are refilled by issue(p + D)
    }
}

template <class S, bool GATHER>
__device__ __forceinline__ void tile_index(const BatchTask& t, long long first, long long cnt) {
    const int m = t.words * 4 >> t.word_log2;
    if (t.word_log2 == 4)
        tile_index_rows<S, uint4, 2, 2, GATHER>(reinterpret_cast<const uint4*>(t.src), reinterpret_cast<uint4*>(t.dst),
                                             t.idx, t.bound, first, cnt, m, t.index_mode == 1);
    else if (t.word_log2 == 3)
        tile_index_rows<S, uint2, 2, 4, GATHER>(reinterpret_cast<const uint2*>(t.src), reinterpret_cast<uint2*>(t.dst),
                                             t.idx, t.bound, first, cnt, m, t.index_mode == 1);
    else
        tile_index_rows<S, unsigned, 2, 4, GATHER>(reinterpret_cast<const unsigned*>(t.src),
                                                reinterpret_cast<unsigned*>(t.dst), t.idx, t.bound, first, cnt, m,
                                                t.index_mode == 1);
}

template <class S, bool GATHER, int PF>
__device__ __forceinline__ void tile_staged_pf(const BatchTask& t, long long first, long long cnt, int m,
                                               unsigned char* stage, int* s_idx) {
    if (t.word_log2 == 4)
        tile_index_staged<S, uint4, GATHER, PF>(reinterpret_cast<const uint4*>(t.src), reinterpret_cast<uint4*>(t.dst),
                                                t.idx, t.bound, first, cnt, m, stage, s_idx);
    else if (t.word_log2 == 3)
        tile_index_staged<S, uint2, GATHER, PF>(reinterpret_cast<const uint2*>(t.src), reinterpret_cast<uint2*>(t.dst),
                                                t.idx, t.bound, first, cnt, m, stage, s_idx);
    else
        tile_index_staged<S, unsigned, GATHER, PF>(reinterpret_cast<const unsigned*>(t.src),
                                                   reinterpret_cast<unsigned*>(t.dst), t.idx, t.bound, first, cnt, m,
                                                   stage, s_idx);
}

// index_mode 2: staged with the context's fetch size; 3 / 4 (gathers): with
// the 64 / 128-byte L2 prefetch-size hint.  In the 4-block build, which has no
// register-held movers, index_mode 0 / 1 (register rows, plain or with the
// 64-byte hint) are staged the same way: plain, or with the 64-byte hint.
template <class S>
__device__ __forceinline__ void tile_staged(const BatchTask& t, long long first, long long cnt, unsigned char* stage,
                                            int* s_idx) {
    const int m = t.words * 4 >> t.word_log2;
    if (t.op != TRV_OP_GATHER)
        tile_staged_pf<S, false, 0>(t, first, cnt, m, stage, s_idx);
    else if (t.index_mode == 3 || t.index_mode == 1)
        tile_staged_pf<S, true, 64>(t, first, cnt, m, stage, s_idx);
    else if (t.index_mode == 4)
        tile_staged_pf<S, true, 128>(t, first, cnt, m, stage, s_idx);
    else
        tile_staged_pf<S, true, 0>(t, first, cnt, m, stage, s_idx);
}

// Task of tile number `tile`: the last k with prefix[k] <= tile (tasks without
// tiles repeat a prefix value and are skipped).  One warp searches, 32 probes
// per round (3 dependent loads for 4096 tasks instead of 12).
__device__ __forceinline__ int find_task(const long long* __restrict__ prefix, int ntasks, long long tile) {
    const int lane = opaque_tid() & 31;
    int lo = 0, hi = ntasks;  // prefix[lo] <= tile < prefix[hi]
    while (hi - lo > 1) {
        const int step = (hi - lo + 31) >> 5;
        const int p = lo + (lane + 1) * step;
        const bool le = p < hi && __ldg(prefix + p) <= tile;  // true on a prefix of the lanes
        const int k = __popc(__ballot_sync(0xFFFFFFFFu, le));
        const int next_hi = lo + (k + 1) * step;
        lo += k * step;
        hi = next_hi < hi ? next_hi : hi;
    }
    return lo;
}

// The persistent kernel in launch shape S (Shape2 / Shape4): the batch
// options or the autotuner pick one.
template <class S>
__global__ void __launch_bounds__(S::block, S::minb)
batch_kernel(const BatchTask* __restrict__ tasks, int ntasks, const long long* __restrict__ tile_prefix,
             unsigned long long* counter, int* flag) {
    __shared__ long long s_tile;
    __shared__ long long s_begin, s_end;  // tile range of task s_lo
    __shared__ int s_lo;
    __shared__ __align__(8) unsigned long long s_bar[S::ring];
    extern __shared__ __align__(128) unsigned char s_stage[];  // S::dyn_smem bytes
    int* s_idx = reinterpret_cast<int*>(s_stage + 2 * S::piece);
    unsigned long long seq = 0;  // thread 0: bulk loads issued so far
    if (threadIdx.x == 0) {
        for (int k = 0; k < S::ring; ++k) mbar_init(&s_bar[k], 1);
        fence_mbarrier_init();
        s_begin = 0;
        s_end = 0;  // no task found yet
        s_lo = 0;
    }
    __syncthreads();
    const long long total = tile_prefix[ntasks];
    for (;;) {
        // Warp 0 takes the next tile and, unless it lies in the task of the
        // block's previous tile, finds its task; the other warps wait at the
        // barrier and read the result.
        if (threadIdx.x < 32) {
            const int lane = opaque_tid() & 31;
            long long tile = 0;
            if (lane == 0) tile = (long long)atomicAdd(counter, 1ull);
            tile = __shfl_sync(0xFFFFFFFFu, tile, 0);
            if (tile < total && !(tile >= s_begin && tile < s_end)) {
                const int lo = find_task(tile_prefix, ntasks, tile);
                __syncwarp();  // every lane has read s_begin / s_end
                if (lane == 0) {
                    s_lo = lo;
                    s_begin = __ldg(tile_prefix + lo);
                    s_end = __ldg(tile_prefix + lo + 1);
                }
            }
            if (lane == 0) s_tile = tile;
        }
        __syncthreads();
        const long long tile = s_tile;
        const int lo = s_lo;
        const long long begin = s_begin;
        __syncthreads();  // read before warp 0 writes the next tile's
        if (tile >= total) break;
        const BatchTask& t = tasks[lo];
        const long long first = (tile - begin) * t.tile_structs;
        const long long cnt = t.n - first < t.tile_structs ? t.n - first : t.tile_structs;
        const long long w = 4ll * t.words;
        if (t.op == TRV_OP_COPY) {
            const unsigned char* cs = t.src + first * w;
            unsigned char* cd = t.dst + first * w;
            const bool bulk = t.copy_bulk != 0 &&
                              ((reinterpret_cast<uintptr_t>(cs) | reinterpret_cast<uintptr_t>(cd)) & 15u) == 0 &&
                              cnt * w >= 16;
            if (bulk) {
                if (threadIdx.x == 0) tile_copy_bulk<S>(cs, cd, cnt * w, s_stage, s_bar, seq, flag);
            } else {
                tile_copy_flat<S>(cs, cd, cnt * w);
            }
        } else if constexpr (S::minb == 2) {
            // the 128-register build: rows staged through shared memory, or
            // held in registers (index_mode 0 / 1)
            if (t.index_mode >= 2)
                tile_staged<S>(t, first, cnt, s_stage, s_idx);
            else if (t.op == TRV_OP_GATHER)
                tile_index<S, true>(t, first, cnt);
            else
                tile_index<S, false>(t, first, cnt);
        } else {
            // The 64-register build stages every gather and scatter row
            // through shared memory: compiling the register-held movers into it
            // as well made it spill (456 bytes a thread) in every path, and
            // without them the 4096-array batch runs 21.32 instead of 22.22 ms
            // (its gathers 10.90 instead of 11.73 ms).
            tile_staged<S>(t, first, cnt, s_stage, s_idx);
        }
    }
}

template <class S>
bool shape_setup(int* per_sm) {
    return cudaFuncSetAttribute(batch_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::dyn_smem) ==
               cudaSuccess &&
           cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, batch_kernel<S>, S::block, S::dyn_smem) ==
               cudaSuccess &&
           *per_sm >= 1;
}

template <class S>
cudaError_t launch_shape(const BatchTask* tasks, int ntasks, const long long* tile_prefix,
                         unsigned long long* counter, int grid, int* flag, cudaStream_t st) {
    batch_kernel<S><<<grid, S::block, S::dyn_smem, st>>>(tasks, ntasks, tile_prefix, counter, flag);
    return cudaGetLastError();
}

}  // namespace

// Per device: the kernels' dynamic shared memory limit raised to their
// staging buffers (once) and their resident blocks with that memory.
int batch_grid(int blocks_per_sm) {
    static std::mutex mu;
    static int resident[64][2] = {};
    DeviceInfo& d = device_info();
    if (d.device < 0 || d.device >= 64) return 0;
    const int which = blocks_per_sm == 2 ? 0 : 1;
    std::lock_guard<std::mutex> g(mu);
    if (!resident[d.device][0]) {
        int r[2] = {0, 0};
        if (!shape_setup<Shape2>(&r[0]) || !shape_setup<Shape4>(&r[1])) {
            cudaGetLastError();
            return 0;
        }
        for (int k = 0; k < 2; ++k) resident[d.device][k] = r[k] * d.sm_count;
    }
    return resident[d.device][which];
}

cudaError_t launch_batch_kernel(const BatchTask* tasks, int ntasks, const long long* tile_prefix,
                                unsigned long long* counter, int grid, int blocks_per_sm, cudaStream_t st) {
    int* flag = device_flag();
    if (!flag) return cudaErrorMemoryAllocation;
    if (blocks_per_sm == 2) return launch_shape<Shape2>(tasks, ntasks, tile_prefix, counter, grid, flag, st);
    return launch_shape<Shape4>(tasks, ntasks, tile_prefix, counter, grid, flag, st);
}

}  // namespace trv
