// TMA bulk-copy path (bulk.cu).
#pragma once

#include <cuda_runtime.h>

namespace trv {

// The bulk engine needs src and dst equal modulo 16.
bool bulk_copy_supported(const void* src, const void* dst);
int bulk_copy_smem_bytes(int chunk);
const void* bulk_copy_func();
// chunk: bytes per stage, a multiple of 16.  flag: device int set to 1 if a
// wait ran out of polls.
cudaError_t launch_bulk_copy(const void* src, void* dst, long long nbytes, int chunk, int grid, int* flag,
                             cudaStream_t st);

}  // namespace trv
