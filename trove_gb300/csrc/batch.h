// Device task table of the batched persistent kernel (batch.cu) and its
// host-side launcher.
#pragma once

#include <cuda_runtime.h>

namespace trv {

struct alignas(16) BatchTask {
    const unsigned char* src;
    unsigned char* dst;
    const int* idx;
    long long n;      // structs (copy) or indices (gather / scatter)
    long long bound;  // gather: source length; scatter: destination length
    int op;           // TRV_OP_*
    int words;        // struct width / 4
    int tile_structs; // structs per tile, a multiple of 32
    int variant;      // copy tasks: TRV_PATH_VECTOR or TRV_PATH_WARP
};

const void* batch_kernel_func();
cudaError_t launch_batch_kernel(const BatchTask* tasks, int ntasks, const long long* tile_prefix,
                                unsigned long long* counter, int grid, cudaStream_t st);
int batch_block_threads();

}  // namespace trv
