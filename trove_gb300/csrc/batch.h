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
    int word_log2;    // gather / scatter: log2 of the word moved per lane (2, 3 or 4)
    int l2_hint;      // gather: 1 = random loads carry the 64-byte L2 prefetch-size hint,
                      // 2 = rows staged through shared memory with cp.async
    int copy_bulk;    // copy: 1 = TMA bulk tiles where 16-byte aligned, 0 = flat vector tiles
};

// blocks_per_sm: 2 or 4 (the register budget the kernel was built for).
const void* batch_kernel_func(int blocks_per_sm);
cudaError_t launch_batch_kernel(const BatchTask* tasks, int ntasks, const long long* tile_prefix,
                                unsigned long long* counter, int grid, int blocks_per_sm, cudaStream_t st);
int batch_block_threads();
// Dynamic shared memory of each batch kernel block (its TMA copy stages).
int batch_dynamic_smem();

}  // namespace trv
