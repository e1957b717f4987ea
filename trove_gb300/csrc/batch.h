// Device task table of the batched persistent kernel (batch.cu), its
// host-side launcher and the tile planner shared by every batch front end
// (trv_batch_create, trv_batch_run_static, the server).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "trove_gb300.h"

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
    int index_mode;   // gather / scatter: 0 = rows held in registers, 1 = the same with the 64-byte
                      // L2 prefetch-size hint on random loads (gather), 2 = rows staged through
                      // shared memory with cp.async, 3 / 4 = staged with the 64 / 128-byte hint
                      // (gather)
    int copy_bulk;    // copy: 1 = TMA bulk tiles where 16-byte aligned, 0 = flat vector tiles
};

// Per-task choices that are not in the task itself.
struct TaskPlan {
    int tile_bytes;           // tile size in bytes of structs (rounded to 32 structs)
    int gather_policy;        // 1 plain, 4 64-byte L2 prefetch-size hint, 5 staged through shared
                              // memory, 6 / 7 staged with the 64 / 128-byte hint
    int scatter_policy;       // 1 plain, 5 staged through shared memory
    int copy_bulk;            // copy tiles through the TMA bulk engine where aligned
};

// Fills one task-table entry from a validated task; returns its tile count.
long long plan_task(int op, uint32_t width, uint64_t n, uint64_t bound, const void* src, void* dst,
                    const int32_t* idx, const TaskPlan& p, BatchTask* d);

// Option checks shared by trv_batch_create and trv_batch_run_static.
int check_batch_options(const trv_batch_options* opt);

// Validates `count` tasks and fills the task table, the running tile count
// (prefix[count + 1]), the algorithmic bytes and the register budget.
int plan_batch(const trv_task* tasks, uint64_t count, const trv_batch_options* opt, BatchTask* out,
               long long* prefix, uint64_t* bytes, int* blocks_per_sm);

// Resident blocks of the batch kernel on the current device at a register
// budget of blocks_per_sm (2 or 4), 0 if it cannot be set up.  The first call
// on a device also raises the kernels' dynamic shared memory limit (their
// staging buffers exceed the default 48 KiB): make it before any capture.
int batch_grid(int blocks_per_sm);
cudaError_t launch_batch_kernel(const BatchTask* tasks, int ntasks, const long long* tile_prefix,
                                unsigned long long* counter, int grid, int blocks_per_sm, cudaStream_t st);

}  // namespace trv
