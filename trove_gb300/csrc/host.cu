// trv_copy_host: the host-buffer form of trv_copy.
//
// When the GPU can address both host buffers — page-locked (pinned) memory,
// or any memory on systems whose GPU walks the host page tables (Grace with
// NVLink-C2C) — the copy kernel reads and writes them directly: one pass
// over the CPU-GPU link in each direction at once, measured at the link's
// bidirectional limit on GB300 (340 GB/s of copy vs 255 GB/s staged).
// Otherwise the array moves through device staging in chunks on three
// streams, so the host->device copy of one chunk, the copy kernel of the
// previous one and the device->host copy of the one before that overlap (the
// two copy directions use separate engines).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "runtime.h"
#include "trove_gb300.h"

namespace trv {
namespace {

constexpr int kStages = 3;
constexpr uint64_t kChunkBytes = uint64_t(64) << 20;

struct Staging {
    std::mutex mu;
    bool ready = false;
    void* src[kStages] = {};
    void* dst[kStages] = {};
    cudaStream_t st[kStages] = {};
};

constexpr int kMaxDevices = 64;

// The current device's staging, or nullptr past the first kMaxDevices devices.
Staging* staging_for_device() {
    static Staging per_device[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return dev >= 0 && dev < kMaxDevices ? &per_device[dev] : nullptr;
}

// Waits for every stage's stream, so no copy still reads or writes the
// caller's buffers once the call returns; the first error wins.
int drain(Staging& s, int rc) {
    for (int j = 0; j < kStages; ++j) {
        const cudaError_t e = cudaStreamSynchronize(s.st[j]);
        if (e != cudaSuccess && rc == TRV_OK) rc = cuda_fail(e);
    }
    return rc;
}

int prepare(Staging& s) {
    if (s.ready) return TRV_OK;
    for (int k = 0; k < kStages; ++k) {
        cudaError_t e = cudaMalloc(&s.src[k], kChunkBytes);
        if (e == cudaSuccess) e = cudaMalloc(&s.dst[k], kChunkBytes);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s.st[k], cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            for (int j = 0; j <= k; ++j) {
                if (s.src[j]) cudaFree(s.src[j]);
                if (s.dst[j]) cudaFree(s.dst[j]);
                if (s.st[j]) cudaStreamDestroy(s.st[j]);
                s.src[j] = s.dst[j] = nullptr;
                s.st[j] = nullptr;
            }
            cudaGetLastError();
            return e == cudaErrorMemoryAllocation ? TRV_ERR_OUT_OF_MEMORY : cuda_fail(e);
        }
    }
    s.ready = true;
    return TRV_OK;
}

// Device-usable addresses of two host buffers when the kernel can access them
// directly: page-locked memory mapped into the device's address space, or
// pageable memory on a device that uses the host page tables.
bool direct_access(const void* src, void* dst, const void** dsrc, void** ddst) {
    cudaPointerAttributes as{}, ad{};
    const bool known = cudaPointerGetAttributes(&as, src) == cudaSuccess &&
                       cudaPointerGetAttributes(&ad, dst) == cudaSuccess;
    cudaGetLastError();
    if (known && as.type == cudaMemoryTypeHost && ad.type == cudaMemoryTypeHost && as.devicePointer &&
        ad.devicePointer) {
        *dsrc = as.devicePointer;
        *ddst = ad.devicePointer;
        return true;
    }
    int dev = 0, pageable = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (known && pageable == 1 && as.type == cudaMemoryTypeUnregistered && ad.type == cudaMemoryTypeUnregistered) {
        *dsrc = src;
        *ddst = dst;
        return true;
    }
    return false;
}

}  // namespace
}  // namespace trv

using namespace trv;

extern "C" int32_t trv_copy_host(void* dst_host, const void* src_host, uint64_t n, uint32_t width) {
    if (width == 0 || n > (uint64_t(1) << 62) / width) return TRV_ERR_INVALID_ARGUMENT;
    if (n == 0) return TRV_OK;
    if (!dst_host || !src_host) return TRV_ERR_INVALID_ARGUMENT;
    Staging* sp = staging_for_device();
    if (!sp) return TRV_ERR_UNSUPPORTED;
    Staging& s = *sp;
    std::lock_guard<std::mutex> guard(s.mu);
    const void* dsrc = nullptr;
    void* ddst = nullptr;
    if (direct_access(src_host, dst_host, &dsrc, &ddst)) {
        cudaStream_t st = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e);
        int rc = trv_copy(ddst, dsrc, n, width, st);
        e = cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
        if (rc != TRV_OK) return rc;
        return e == cudaSuccess ? TRV_OK : cuda_fail(e);
    }
    int rc = prepare(s);
    if (rc != TRV_OK) return rc;
    // Whole structs per chunk, so each chunk is a valid trv_copy.
    uint64_t per_chunk = kChunkBytes / width;
    if (per_chunk == 0) return TRV_ERR_UNSUPPORTED;  // one struct larger than a chunk
    const unsigned char* in = static_cast<const unsigned char*>(src_host);
    unsigned char* out = static_cast<unsigned char*>(dst_host);
    int k = 0;
    for (uint64_t first = 0; first < n; first += per_chunk, k = (k + 1) % kStages) {
        const uint64_t cnt = n - first < per_chunk ? n - first : per_chunk;
        const uint64_t off = first * width, bytes = cnt * width;
        cudaStream_t st = s.st[k];
        cudaError_t e = cudaMemcpyAsync(s.src[k], in + off, bytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return drain(s, cuda_fail(e));
        rc = trv_copy(s.dst[k], s.src[k], cnt, width, st);
        if (rc != TRV_OK) return drain(s, rc);
        e = cudaMemcpyAsync(out + off, s.dst[k], bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return drain(s, cuda_fail(e));
    }
    return drain(s, TRV_OK);
}
