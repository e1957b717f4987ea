// trv_batch_run_static: the batched kernel without any device allocation.
//
// trv_batch_create allocates the batch's task table, tile prefix and work
// counter with cudaMalloc.  Some callers cannot do that: cudaMalloc
// synchronizes the whole device, which stalls latency-critical loops that
// share the GPU with other streams, and processes whose device memory is
// reserved up front by another allocator (a framework's pool, a fixed arena)
// may have nothing left for a stray cudaMalloc, or must not fragment it.
// This entry point keeps those three tables in one file-scope __device__
// array instead, so a call allocates nothing on the device; the caller still
// provides every input and output array.
//
// Limits and sharing:
//  - at most kStaticMaxTasks tasks per call (larger batches are rejected with
//    TRV_ERR_UNSUPPORTED before anything is enqueued);
//  - the array is one per device, held by every process that loads the
//    library until it exits (about 300 KB), and shared by all calls on that
//    device: a call rewrites it and clears the work counter on its stream, so
//    two calls whose work overlaps on the GPU (different streams, or threads
//    without ordering) race on it and must be serialized by the caller;
//  - the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (once per device, that device current); make that
//    first call before any stream capture begins.  The address is cached for
//    the life of the process: after cudaDeviceReset the device's next
//    context places the array elsewhere, so a process that resets a device
//    must not call this entry point on that device again;
//  - the task table and tile prefix are planned in host memory that lives
//    only for the duration of the call and are copied to the array with
//    cudaMemcpyAsync from that pageable memory, which may make the host wait
//    for the stream's earlier work before the copy starts.  For the same
//    reason a stream that is being captured is refused (TRV_ERR_UNSUPPORTED):
//    a captured copy would read the freed host plan on every replay;
//  - opt->grid_blocks, when positive, is used as the grid as given (a grid
//    above the device's limit fails the launch with TRV_ERR_CUDA), and a
//    current device index of 64 or more is refused with TRV_ERR_UNSUPPORTED.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "batch.h"
#include "runtime.h"
#include "trove_gb300.h"

namespace trv {
namespace {

constexpr int kStaticMaxTasks = TRV_STATIC_BATCH_MAX_TASKS;
constexpr size_t kTaskBytes = sizeof(BatchTask) * kStaticMaxTasks;
constexpr size_t kPrefixOffset = (kTaskBytes + 255) / 256 * 256;
constexpr size_t kPrefixBytes = sizeof(long long) * (kStaticMaxTasks + 1);
constexpr size_t kCounterOffset = (kPrefixOffset + kPrefixBytes + 255) / 256 * 256;
constexpr size_t kScratchBytes = kCounterOffset + 256;

// Task table | tile prefix | work counter, each 256-byte aligned.
static __device__ __align__(256) unsigned char g_batch_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[64] = {};

// Device address of g_batch_scratch on the current device (resolved once).
int scratch_for_current_device(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e);
    if (dev < 0 || dev >= 64) return TRV_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_batch_scratch);
        if (e != cudaSuccess) return cuda_fail(e);
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return TRV_OK;
}

}  // namespace
}  // namespace trv

using namespace trv;

static int32_t batch_run_static_impl(const trv_task* tasks, uint64_t count, const trv_batch_options* opt,
                                        void* stream) {
    if (count > 0 && !tasks) return TRV_ERR_INVALID_ARGUMENT;
    if (count > uint64_t(kStaticMaxTasks)) return TRV_ERR_UNSUPPORTED;
    const int orc = check_batch_options(opt);
    if (orc != TRV_OK) return orc;
    std::vector<BatchTask> host(count);
    std::vector<long long> prefix(count + 1);
    int blocks_per_sm = 4;
    const int rc = plan_batch(tasks, count, opt, host.data(), prefix.data(), nullptr, &blocks_per_sm);
    if (rc != TRV_OK) return rc;
    if (count == 0 || prefix[count] == 0) return TRV_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &capture);
    if (e != cudaSuccess) return cuda_fail(e);
    if (capture != cudaStreamCaptureStatusNone) return TRV_ERR_UNSUPPORTED;
    unsigned char* scratch = nullptr;
    const int src = scratch_for_current_device(&scratch);
    if (src != TRV_OK) return src;
    const int resident = batch_grid(blocks_per_sm);
    if (resident < 1) return TRV_ERR_CUDA;
    BatchTask* d_tasks = reinterpret_cast<BatchTask*>(scratch);
    long long* d_prefix = reinterpret_cast<long long*>(scratch + kPrefixOffset);
    unsigned long long* d_counter = reinterpret_cast<unsigned long long*>(scratch + kCounterOffset);
    e = cudaMemcpyAsync(d_tasks, host.data(), sizeof(BatchTask) * count, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_prefix, prefix.data(), sizeof(long long) * (count + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_fail(e);
    int grid = (opt && opt->grid_blocks > 0) ? opt->grid_blocks : resident;
    if (prefix[count] < grid) grid = int(prefix[count]);
    e = launch_batch_kernel(d_tasks, int(count), d_prefix, d_counter, grid, blocks_per_sm, st);
    return e == cudaSuccess ? TRV_OK : cuda_fail(e);
}

extern "C" int32_t trv_batch_run_static(const trv_task* tasks, uint64_t count, const trv_batch_options* opt,
                                        void* stream) {
    return no_throw([&] { return batch_run_static_impl(tasks, count, opt, stream); });
}
