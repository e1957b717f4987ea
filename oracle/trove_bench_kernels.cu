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

}  // namespace

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
            if (trove::warp_converged())                                                           \
                trove::store_array_warp_contiguous<S, TILE_SIZE>(r, index, d);                     \
            else                                                                                    \
                trove::store_array(r, index, d);                                                    \
        }                                                                                           \
    }                                                                                               \
    extern "C" __global__ void block_copy_##S(const int* x, int* r, int l) {                       \
        for (int index = threadIdx.x + blockIdx.x * blockDim.x; index < l;                         \
             index += gridDim.x * blockDim.x) {                                                     \
            if (trove::warp_converged()) {                                                          \
                aos_##S d = trove::load_array_warp_contiguous<S, TILE_SIZE>(x, index);             \
                trove::store_array_warp_contiguous(r, index, d);                                   \
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
        aos_##S v = trove::warp_converged() ? trove::load_warp_contiguous<TILE_SIZE>(s + i) : s[i]; \
        if (modulus != 0u && first_word(v) % modulus == modulus - 1u) return;                      \
        if (trove::warp_converged())                                                                \
            trove::store_warp_contiguous<TILE_SIZE>(v, r + i);                                     \
        else                                                                                        \
            r[i] = v;                                                                               \
    }

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
