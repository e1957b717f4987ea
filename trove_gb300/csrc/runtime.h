// Shared host-side runtime state of the library: per-device properties,
// launch-shape helpers and the thread-local CUDA error slot.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <exception>

#include "trove_gb300.h"

namespace trv {

struct DeviceInfo {
    std::atomic<bool> ready{false};
    int device = 0;
    int sm_count = 1;
    int* flag = nullptr;  // device int: set by kernels whose bounded waits give up
};

// Properties of the calling thread's current device (cached).
DeviceInfo& device_info();

// The current device's error flag (a device variable found on first use),
// or nullptr if it cannot be found.
int* device_flag();

// Resident blocks of `func` at `block` threads across the whole GPU.
int resident_blocks(const void* func, int block);

// Blocks for work_items items at items_per_block each, capped at the
// resident-block count (a persistent, grid-stride launch); `requested` > 0
// overrides.
int grid_for(const void* func, long long work_items, int items_per_block, int block, int requested);

// True, with the grid, when a launch of one 32*unroll-struct chunk per warp
// applies (no grid requested, and the grid fits).
bool one_chunk_per_warp(long long n, int unroll, int requested, int* grid);

int unroll_slot(int unroll);
int default_unroll(unsigned width);

// Runs an entry point's body so that no C++ exception crosses the C ABI.  The
// only exceptions the host code can meet are failed allocations of its host
// containers and of the server's dispatcher thread: both report
// TRV_ERR_OUT_OF_MEMORY.
template <typename F>
int32_t no_throw(F&& body) noexcept {
    try {
        return body();
    } catch (...) {
        return TRV_ERR_OUT_OF_MEMORY;
    }
}

// Records a CUDA error for trv_last_cuda_error() and returns TRV_ERR_CUDA.
int cuda_fail(cudaError_t e);
// cudaGetLastError() folded into a trv_status.
int check_launch();

}  // namespace trv
