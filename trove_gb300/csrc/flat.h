// Launchers of the width-agnostic kernels in flat.cu and bulk.cu.
#pragma once

#include <cuda_runtime.h>

namespace trv {

void launch_fill_u32(unsigned* dst, long long nwords, unsigned long long seed, int grid, cudaStream_t st);
void launch_uniform_indices(int* idx, long long n, unsigned bound, unsigned long long seed, int grid,
                            cudaStream_t st);

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
