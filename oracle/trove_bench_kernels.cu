// Trove-API kernels in the style of the reference's own tests — TEST
// INFRASTRUCTURE ONLY (parity tests and comparison baseline, never the product).
//
// The same source is compiled against two header trees by
// oracle/build_oracle.py:
//   * the reference's trove/ (in place, read-only) -> oracle/_ref/*.cubin,
//     so the reference Trove runs on the same GB300 as this library, and
//   * this repository's include/trove -> oracle/_build/*.cubin, which shows
//     that kernels written for the reference recompile unchanged.
// Kernel bodies follow tests/benchmark.cu:52-128 (shfl and direct store,
// load+sum, gather, scatter) and tests/block.cu:13-54 (block write/copy).
// Every kernel has C linkage: <kind>_<words>, e.g. shfl_gather_12.
//
// TILE_SIZE is the reference's own build knob (tests/Makefile): the tile of
// load/store_warp_contiguous and of the block interface.  build_oracle.py
// compiles this file at TILE_SIZE 32, 16, 8, 4 and 2 for both trees.  The
// kernels beyond the reference's tests exercise the rest of its public API
// on the GPU: warp_load / warp_store / uncoalesced_store (memory.h),
// warp_converged<N> and thread_tile<N> (warp.h), warps with inactive lanes
// through coalesced_ptr (the load/store cascade of aos.h), and, built only
// against this repository's headers (TRV_OWN_TREE), coalesced_ptr
// reference-to-reference assignment, which the reference's ptr.h does not
// compile.
#include <trove/aos.h>
#include <trove/block.h>
#include <trove/ptr.h>

#ifndef TILE_SIZE
#define TILE_SIZE 32
#endif

namespace {

template <typename T>
__device__ __forceinline__ unsigned first_word(const T& v) {
    unsigned w;
    memcpy(&w, &v, 4);
    return w;
}

// Which threads of the partial-warp kernels leave first: (lane_hash % 100) <
// pct.  A 32-bit multiply-xorshift mix; the tests restate it on the host.
__device__ __forceinline__ unsigned lane_hash(unsigned i, unsigned seed) {
    unsigned x = i * 0x9E3779B1u + seed;
    x ^= x >> 15;
    x *= 0x85EBCA6Bu;
    x ^= x >> 13;
    return x;
}

}  // namespace

#ifdef TRV_OWN_TREE
// D[i] = S[idx[i]] and D[idx[i]] = S[i] through two coalesced_refs: the
// reference-to-reference assignment of ptr.h (a load, then a store).
#define TRV_REFREF_KERNELS(S)                                                                       \
    extern "C" __global__ void refref_gather_##S(const int* indices, aos_##S* raw_s, aos_##S* raw_r) { \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        trove::coalesced_ptr<aos_##S> s(raw_s);                                                     \
        trove::coalesced_ptr<aos_##S> r(raw_r);                                                     \
        r[i] = s[indices[i]];                                                                       \
    }                                                                                               \
    extern "C" __global__ void refref_scatter_##S(const int* indices, aos_##S* raw_s, aos_##S* raw_r) { \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        trove::coalesced_ptr<aos_##S> s(raw_s);                                                     \
        trove::coalesced_ptr<aos_##S> r(raw_r);                                                     \
        r[indices[i]] = s[i];                                                                       \
    }
#else
#define TRV_REFREF_KERNELS(S)
#endif

// warp_converged<N> for N = 32, 16, 8, 4, 2 in warps whose active lanes are
// masks[warp]: each active lane writes bit k for the k-th N (out[i], 0xFF
// stays where the lane was inactive).
extern "C" __global__ void converged_probe(const unsigned* masks, unsigned char* out) {
    int i = threadIdx.x + blockDim.x * blockIdx.x;
    unsigned mask = masks[i >> 5];
    if (!((mask >> (i & 31)) & 1u)) return;
    out[i] = (unsigned char)((trove::warp_converged<32>() ? 1 : 0) | (trove::warp_converged<16>() ? 2 : 0) |
                             (trove::warp_converged<8>() ? 4 : 0) | (trove::warp_converged<4>() ? 8 : 0) |
                             (trove::warp_converged<2>() ? 16 : 0));
}

// thread_tile<N>: rank, size and a shuffle from rank (rank + 3) % N, for
// N = 32, 16, 8, 4, 2 (out[5 * i + k]).
template <int N>
__device__ __forceinline__ int tile_probe_one(int v) {
    trove::thread_tile<N> t;
    int got = t.shfl(v, int((t.id() + 3) % N));
    return got * 1024 + int(t.id()) * 32 + int(t.size());
}

extern "C" __global__ void tile_shfl_probe(int* out) {
    int i = threadIdx.x + blockDim.x * blockIdx.x;
    int v = i * 7 + 1;
    out[5 * i + 0] = tile_probe_one<32>(v);
    out[5 * i + 1] = tile_probe_one<16>(v);
    out[5 * i + 2] = tile_probe_one<8>(v);
    out[5 * i + 3] = tile_probe_one<4>(v);
    out[5 * i + 4] = tile_probe_one<2>(v);
}

#define TRV_BENCH_KERNELS(S)                                                                        \
    typedef trove::array<int, S> aos_##S;                                                           \
    /* tests/benchmark.cu:52-61 */                                                                  \
    extern "C" __global__ void shfl_store_##S(aos_##S* r) {                                        \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        aos_##S data = trove::counting_array<aos_##S>::impl(i * S);                                \
        trove::store_warp_contiguous<TILE_SIZE>(data, r + i);                                      \
    }                                                                                               \
    /* tests/benchmark.cu:74-80 */                                                                  \
    extern "C" __global__ void shfl_load_##S(aos_##S* s, int* r) {                                 \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        aos_##S data = trove::load_warp_contiguous<TILE_SIZE>(s + i);                              \
        r[i] = trove::sum(data);                                                                    \
    }                                                                                               \
    /* contiguous copy through the low-level API, one struct per thread */                         \
    extern "C" __global__ void shfl_copy_##S(const aos_##S* s, aos_##S* r) {                       \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        aos_##S data = trove::load_warp_contiguous<TILE_SIZE>(s + i);                              \
        trove::store_warp_contiguous<TILE_SIZE>(data, r + i);                                      \
    }                                                                                               \
    extern "C" __global__ void direct_copy_##S(const aos_##S* s, aos_##S* r) {                     \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        r[i] = s[i];                                                                                \
    }                                                                                               \
    /* tests/benchmark.cu:90-128 */                                                                 \
    extern "C" __global__ void shfl_gather_##S(const int* indices, aos_##S* raw_s, aos_##S* raw_r) { \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        int index = indices[i];                                                                     \
        trove::coalesced_ptr<aos_##S> s(raw_s);                                                     \
        trove::coalesced_ptr<aos_##S> r(raw_r);                                                     \
        aos_##S data = s[index];                                                                    \
        r[i] = data;                                                                                \
    }                                                                                               \
    extern "C" __global__ void shfl_scatter_##S(const int* indices, aos_##S* raw_s, aos_##S* raw_r) { \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        int index = indices[i];                                                                     \
        trove::coalesced_ptr<aos_##S> s(raw_s);                                                     \
        trove::coalesced_ptr<aos_##S> r(raw_r);                                                     \
        aos_##S data = s[i];                                                                        \
        r[index] = data;                                                                            \
    }                                                                                               \
    extern "C" __global__ void direct_gather_##S(const int* indices, aos_##S* s, aos_##S* r) {     \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        r[i] = s[indices[i]];                                                                       \
    }                                                                                               \
    extern "C" __global__ void direct_scatter_##S(const int* indices, aos_##S* s, aos_##S* r) {    \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        r[indices[i]] = s[i];                                                                       \
    }                                                                                               \
    /* tests/block.cu:13-54, any length l (grid-stride, converged check) */                        \
    extern "C" __global__ void block_write_##S(int* r, int l) {                                    \
        for (int index = threadIdx.x + blockIdx.x * blockDim.x; index < l;                         \
             index += gridDim.x * blockDim.x) {                                                     \
            aos_##S d = trove::counting_array<aos_##S>::impl(S * index);                           \
            if (trove::warp_converged<TILE_SIZE>())                                                \
                trove::store_array_warp_contiguous<S, TILE_SIZE>(r, index, d);                     \
            else                                                                                    \
                trove::store_array(r, index, d);                                                    \
        }                                                                                           \
    }                                                                                               \
    extern "C" __global__ void block_copy_##S(const int* x, int* r, int l) {                       \
        for (int index = threadIdx.x + blockIdx.x * blockDim.x; index < l;                         \
             index += gridDim.x * blockDim.x) {                                                     \
            if (trove::warp_converged<TILE_SIZE>()) {                                               \
                aos_##S d = trove::load_array_warp_contiguous<S, TILE_SIZE>(x, index);             \
                trove::store_array_warp_contiguous<S, TILE_SIZE>(r, index, d);                     \
            } else {                                                                                \
                aos_##S d = trove::load_array<S>(x, index);                                        \
                trove::store_array(r, index, d);                                                    \
            }                                                                                       \
        }                                                                                           \
    }                                                                                               \
    /* copy with a data-dependent early exit between load and store */                             \
    extern "C" __global__ void exit_copy_##S(const aos_##S* s, aos_##S* r, long long n,            \
                                             unsigned modulus) {                                    \
        long long i = threadIdx.x + (long long)blockDim.x * blockIdx.x;                            \
        if (i >= n) return;                                                                         \
        aos_##S v = trove::warp_converged<TILE_SIZE>() ? trove::load_warp_contiguous<TILE_SIZE>(s + i) \
                                                       : s[i];                                      \
        if (modulus != 0u && first_word(v) % modulus == modulus - 1u) return;                      \
        if (trove::warp_converged<TILE_SIZE>())                                                     \
            trove::store_warp_contiguous<TILE_SIZE>(v, r + i);                                     \
        else                                                                                        \
            r[i] = v;                                                                               \
    }                                                                                               \
    /* memory.h: each warp's S*32 words read as warp_load(p, lane, 32) (the volatile overload in \
       odd warps), written back with warp_store(a, q, lane, 32) and, per thread, with            \
       uncoalesced_store(a, u + S*i) */                                                            \
    extern "C" __global__ void memory_rw_##S(const int* s, int* r, int* u) {                       \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        int lane = i & 31;                                                                          \
        long long base = (long long)(i >> 5) * 32 * S;                                             \
        typedef trove::array<int, S> words;                                                         \
        words a = ((i >> 5) & 1) ? trove::warp_load<words>((const volatile int*)(s + base), lane, 32) \
                                 : trove::warp_load<words>(s + base, lane, 32);                    \
        trove::warp_store(a, r + base, lane, 32);                                                   \
        if ((i >> 5) & 1)                                                                           \
            trove::uncoalesced_store(a, (volatile int*)(u + (long long)S * i));                    \
        else                                                                                        \
            trove::uncoalesced_store(a, u + (long long)S * i);                                      \
    }                                                                                               \
    /* coalesced_ptr on warps with inactive lanes: a lane whose hash falls below pct % leaves  \
       first, so load/store see partial warps (the reference's 16/8/4/2-lane cascade) */        \
    extern "C" __global__ void partial_gather_##S(const int* indices, aos_##S* raw_s, aos_##S* raw_r, \
                                                  unsigned pct, unsigned seed) {                    \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        if (lane_hash(unsigned(i), seed) % 100u < pct) return;                                      \
        int index = indices[i];                                                                     \
        trove::coalesced_ptr<aos_##S> s(raw_s);                                                     \
        trove::coalesced_ptr<aos_##S> r(raw_r);                                                     \
        aos_##S data = s[index];                                                                    \
        r[i] = data;                                                                                \
    }                                                                                               \
    extern "C" __global__ void partial_copy_##S(aos_##S* raw_s, aos_##S* raw_r, unsigned pct,      \
                                                unsigned seed) {                                    \
        int i = threadIdx.x + blockDim.x * blockIdx.x;                                             \
        if (lane_hash(unsigned(i), seed) % 100u < pct) return;                                      \
        trove::coalesced_ptr<aos_##S> s(raw_s);                                                     \
        trove::coalesced_ptr<aos_##S> r(raw_r);                                                     \
        aos_##S data = s[i];                                                                        \
        r[i] = data;                                                                                \
    }                                                                                               \
    TRV_REFREF_KERNELS(S)

TRV_BENCH_KERNELS(1)
TRV_BENCH_KERNELS(2)
TRV_BENCH_KERNELS(3)
TRV_BENCH_KERNELS(4)
TRV_BENCH_KERNELS(5)
TRV_BENCH_KERNELS(6)
TRV_BENCH_KERNELS(7)
TRV_BENCH_KERNELS(8)
TRV_BENCH_KERNELS(9)
TRV_BENCH_KERNELS(10)
TRV_BENCH_KERNELS(11)
TRV_BENCH_KERNELS(12)
TRV_BENCH_KERNELS(13)
TRV_BENCH_KERNELS(14)
TRV_BENCH_KERNELS(15)
TRV_BENCH_KERNELS(16)
// 80 B = 5 x int4 (odd), 96 B = 6 x int4 (composite), 132 B = 33 words (more
// words than lanes: per-thread)
TRV_BENCH_KERNELS(20)
TRV_BENCH_KERNELS(24)
TRV_BENCH_KERNELS(33)
