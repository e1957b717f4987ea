// TMA bulk-copy path (bulk.cu).
#pragma once

#include <cuda_runtime.h>

namespace trv {

// The bulk engine needs src and dst equal modulo 16.
bool bulk_copy_supported(const void* src, const void* dst);
int bulk_copy_smem_bytes(int chunk);
const void* bulk_copy_func();
// Poll budget of the copy loop's waits (0xFFFFFFFF: the default, about a
// second); the drain after a timeout always uses the default.  Test hook.
void set_bulk_wait_polls(unsigned polls);
// chunk: bytes per stage, a multiple of 16.  flag: device int set to 1 if a
// wait ran out of polls.
cudaError_t launch_bulk_copy(const void* src, void* dst, long long nbytes, int chunk, int grid, int* flag,
                             cudaStream_t st);

}  // namespace trv
