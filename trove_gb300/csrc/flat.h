// Launchers of the width-agnostic kernels in flat.cu and bulk.cu.
#pragma once

#include <cuda_runtime.h>

namespace trv {

// Seeded synthetic inputs.  Word k of the stream for `seed` is the high half
// of splitmix64's finaliser applied to k * 0x9E3779B97F4A7C15 +
// seed * 0xD1B54A32D192ED03 + 1: counter-based, so any word can be computed
// alone, on the host or the device.
__host__ __device__ inline unsigned long long stream_mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ inline unsigned stream_word(unsigned long long seed, unsigned long long k) {
    return (unsigned)(stream_mix64(k * 0x9E3779B97F4A7C15ull + seed * 0xD1B54A32D192ED03ull + 1ull) >> 32);
}
// Uniform draw in [0, bound) from word k (multiply-high).
__host__ __device__ inline unsigned stream_bounded(unsigned long long seed, unsigned long long k, unsigned bound) {
    return (unsigned)(((unsigned long long)stream_word(seed, k) * bound) >> 32);
}

void launch_fill_u32(unsigned* dst, long long nwords, unsigned long long seed, int grid, cudaStream_t st);
void launch_uniform_indices(int* idx, long long n, unsigned bound, unsigned long long seed, int grid,
                            cudaStream_t st);
void launch_run_indices(int* idx, long long n, unsigned long long seed, int grid, cudaStream_t st);

// Flat copy of nbytes: `head` leading bytes (< vec_bytes) bring both pointers
// to vec_bytes alignment, the rest moves as vec_bytes vectors.
void launch_flat_copy(const void* src, void* dst, long long nbytes, int vec_bytes, int head, int unroll,
                      int grid, cudaStream_t st);
const void* flat_copy_func(int vec_bytes, int unroll);

void launch_gather_bytes(const void* src, long long src_n, const int* idx, void* dst, long long n,
                         unsigned width, int grid, cudaStream_t st);
void launch_scatter_bytes(const void* src, const int* idx, void* dst, long long dst_n, long long n,
                          unsigned width, int grid, cudaStream_t st);

}  // namespace trv
