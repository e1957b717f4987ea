// TRV_PATH_BULK: long contiguous copies through the TMA bulk-copy engine.
//
// One thread per CTA drives a ring of kStages shared-memory buffers:
//   load chunk c:  cp.async.bulk.shared::cluster.global ... complete_tx on
//                  the stage's mbarrier;
//   store chunk c: after the mbarrier phase completes,
//                  cp.async.bulk.global.shared::cta.bulk_group from the
//                  stage, one bulk group per chunk;
//   refill:        once the previous chunk's store has finished reading its
//                  stage (cp.async.bulk.wait_group.read 1) that stage loads
//                  chunk c - 1 + kStages.
// So kStages - 1 loads and up to two stores are in flight per SM with a
// single issuing thread and no register traffic.  Chunks are dealt to CTAs
// round-robin.  Both pointers must share their address modulo 16 (the bulk
// engine's alignment unit); the unaligned head and sub-16-byte tail are
// copied by CTA 0 with plain loads.
//
// Every mbarrier wait is bounded: after kSpinLimit polls the CTA records an
// error in the library's device flag, drains what it has in flight (again
// bounded) and returns, so a stuck transfer can never hang the GPU.
#include <cuda_runtime.h>
#include <stdint.h>

#include "bulk.h"
#include "tma.cuh"

namespace trv {
namespace {

constexpr int kStages = 4;

__global__ void __launch_bounds__(32)
bulk_copy_kernel(const unsigned char* __restrict__ src, unsigned char* __restrict__ dst, long long nbytes, int head,
                 int chunk, int* flag, unsigned polls) {
    extern __shared__ __align__(128) unsigned char stage_mem[];
    __shared__ __align__(8) unsigned long long bar[kStages];

    // plain-load edges: [0, head) and the sub-16-byte tail
    const long long body = ((nbytes - head) / 16) * 16;
    if (blockIdx.x == 0) {
        for (int t = threadIdx.x; t < head; t += blockDim.x) dst[t] = src[t];
        for (long long t = head + body + threadIdx.x; t < nbytes; t += blockDim.x) dst[t] = src[t];
    }
    if (threadIdx.x != 0 || body == 0) return;

    const unsigned char* s = src + head;
    unsigned char* d = dst + head;
    const long long nchunks = (body + chunk - 1) / chunk;
    const long long mine = nchunks > blockIdx.x ? (nchunks - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (mine == 0) return;

    for (int k = 0; k < kStages; ++k) mbar_init(&bar[k], 1);
    fence_mbarrier_init();

    auto chunk_bytes = [&](long long c) -> unsigned {
        const long long off = c * chunk;
        return static_cast<unsigned>(body - off < chunk ? body - off : chunk);
    };
    auto issue_load = [&](long long k) {  // k-th chunk of this CTA
        const long long c = blockIdx.x + k * (long long)gridDim.x;
        const int st = int(k % kStages);
        const unsigned bytes = chunk_bytes(c);
        mbar_expect_tx(&bar[st], bytes);
        bulk_load(stage_mem + (size_t)st * chunk, s + c * chunk, bytes, &bar[st]);
    };

    const long long prologue = mine < kStages ? mine : kStages;
    for (long long k = 0; k < prologue; ++k) issue_load(k);
    long long issued = prologue;

    bool ok = true;
    long long k = 0;
    for (; k < mine; ++k) {
        const int st = int(k % kStages);
        if (!mbar_wait(&bar[st], unsigned((k / kStages) & 1), polls)) {
            ok = false;
            break;
        }
        fence_proxy_async_shared();
        const long long c = blockIdx.x + k * (long long)gridDim.x;
        bulk_store(d + c * chunk, stage_mem + (size_t)st * chunk, chunk_bytes(c));
        if (k >= 1 && issued < mine) {
            bulk_wait_read_1();  // the previous chunk's store has read its stage
            issue_load(issued++);
        }
    }
    if (!ok) {
        atomicExch(flag, 1);
        // drain every load still in flight, including the one that timed out
        // (bounded), so no transfer targets this CTA's shared memory after it
        // exits
        for (long long j = k; j < issued; ++j) mbar_wait(&bar[j % kStages], unsigned((j / kStages) & 1));
    }
    bulk_wait_all();
}

}  // namespace

bool bulk_copy_supported(const void* src, const void* dst) {
    return ((reinterpret_cast<uintptr_t>(src) ^ reinterpret_cast<uintptr_t>(dst)) & 15u) == 0;
}

int bulk_copy_smem_bytes(int chunk) { return kStages * chunk; }

namespace {
unsigned g_main_polls = kSpinLimit;
}

void set_bulk_wait_polls(unsigned polls) { g_main_polls = polls == 0xFFFFFFFFu ? kSpinLimit : polls; }

cudaError_t launch_bulk_copy(const void* src, void* dst, long long nbytes, int chunk, int grid, int* flag,
                             cudaStream_t st) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(src);
    int head = int((16 - (a & 15u)) & 15u);
    if (head > nbytes) head = int(nbytes);
    const int smem = bulk_copy_smem_bytes(chunk);
    cudaError_t e = cudaFuncSetAttribute(bulk_copy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    bulk_copy_kernel<<<grid, 32, smem, st>>>(static_cast<const unsigned char*>(src), static_cast<unsigned char*>(dst),
                                             nbytes, head, chunk, flag, g_main_polls);
    return cudaGetLastError();
}

const void* bulk_copy_func() { return (const void*)&bulk_copy_kernel; }

}  // namespace trv
