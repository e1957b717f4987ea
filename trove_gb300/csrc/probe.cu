// trv_probe_block_gather: the memory system's ceiling for a random gather.
//
// A gather dst[i] = src[idx[i]] of `width`-byte rows must read, for every
// index, the DRAM blocks its row overlaps; how fast that can go on a given
// GPU is a property of the memory system (DRAM row activations, L2 fetch
// size), not of a gather kernel.  This probe measures it with the most
// favourable access shape there is: for each index it reads every
// block_bytes-aligned block its row overlaps as whole 16-byte vectors, the
// lanes of a warp covering each block together (one sector group per block
// and instruction), all of a warp's loads issued before any is used; it reads
// the indices sequentially and writes n * width bytes sequentially, as a
// gather does.  What it writes is a fold of the blocks, not the rows: only the
// traffic matters.  Block sizes 32 / 64 / 128 with a matching L2
// prefetch-size hint (none / 64 B / 128 B) bracket what the L2 fetches on a
// miss.  No reference counterpart.
#include <cuda_runtime.h>

#include <cstdint>

#include "runtime.h"
#include "trove_gb300.h"

namespace trv {
namespace {

// Predicated 16-byte load (v keeps its value where `on` is 0).  Every load
// and every fold step is a volatile asm statement, so the compiler keeps
// them in program order: all of a warp's loads are issued before the first
// fold consumes one, which keeps K loads per lane in flight.
template <int HINT>
__device__ __forceinline__ void load_block_vec(uint4& v, const uint4* p, unsigned on) {
    if constexpr (HINT == 64) {
        asm volatile("{ .reg .pred q; setp.ne.u32 q, %5, 0; @q ld.global.L2::64B.v4.u32 {%0, %1, %2, %3}, [%4]; }"
                     : "+r"(v.x), "+r"(v.y), "+r"(v.z), "+r"(v.w)
                     : "l"(p), "r"(on));
    } else if constexpr (HINT == 128) {
        asm volatile("{ .reg .pred q; setp.ne.u32 q, %5, 0; @q ld.global.L2::128B.v4.u32 {%0, %1, %2, %3}, [%4]; }"
                     : "+r"(v.x), "+r"(v.y), "+r"(v.z), "+r"(v.w)
                     : "l"(p), "r"(on));
    } else {
        asm volatile("{ .reg .pred q; setp.ne.u32 q, %5, 0; @q ld.global.v4.u32 {%0, %1, %2, %3}, [%4]; }"
                     : "+r"(v.x), "+r"(v.y), "+r"(v.z), "+r"(v.w)
                     : "l"(p), "r"(on));
    }
}

__device__ __forceinline__ void fold(uint4& f, const uint4& v) {
    asm volatile("xor.b32 %0, %0, %4; xor.b32 %1, %1, %5; xor.b32 %2, %2, %6; xor.b32 %3, %3, %7;"
                 : "+r"(f.x), "+r"(f.y), "+r"(f.z), "+r"(f.w)
                 : "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w));
}

// One warp per 32 rows (n is a multiple of 32).  K = vector slots per row:
// the most blocks a row can overlap times the vectors per block.  Round r,
// lane l: slot q = l + 32 r -> row q / K, its block (q % K) / (B / 16) past
// the row's first, vector (q % K) % (B / 16) of that block; slots past the
// row's last block stay idle.
template <int B, int K, int HINT>
__global__ void __launch_bounds__(256) block_gather_kernel(uint4* __restrict__ dst, const unsigned char* __restrict__ src,
                                                           unsigned long long src_n, const int* __restrict__ idx,
                                                           unsigned long long n, unsigned width) {
    constexpr int VPB = B / 16;
    const unsigned long long warp = (blockIdx.x * 256ull + threadIdx.x) >> 5;
    const int lane = int(threadIdx.x & 31);
    const unsigned long long i0 = warp * 32ull;
    if (i0 >= n) return;
    const int my = idx[i0 + lane];
    uint4 v[K];
#pragma unroll
    for (int r = 0; r < K; ++r) {
        const int q = lane + 32 * r;
        const int j = q / K;
        const int slot = q - j * K;
        const int row = __shfl_sync(0xFFFFFFFFu, my, j);
        const unsigned long long start = (unsigned long long)(unsigned)row * width;
        const unsigned long long b0 = start / B;
        const unsigned long long b1 = (start + width - 1) / B;
        const unsigned long long blk = b0 + slot / VPB;
        const bool on = row >= 0 && (unsigned long long)row < src_n && blk <= b1;
        v[r] = make_uint4(0u, 0u, 0u, 0u);
        load_block_vec<HINT>(v[r], reinterpret_cast<const uint4*>(src + (on ? blk * B : 0)) + (slot % VPB),
                             on ? 1u : 0u);
    }
    uint4 f = make_uint4(unsigned(lane), 0u, 0u, 0u);
#pragma unroll
    for (int r = 0; r < K; ++r) fold(f, v[r]);
    // the warp's 32 rows are 32 * width bytes = 2 * width vectors at byte i0 * width
    uint4* out = dst + (i0 * width) / 16;
    for (int k = lane; k < int(2 * width); k += 32) out[k] = f;
}

template <int B, int HINT>
int launch_for_block(void* dst, const void* src, uint64_t src_n, const int32_t* idx, uint64_t n, uint32_t width,
                     cudaStream_t st) {
    // most B-byte blocks a 4-byte-aligned row of `width` bytes overlaps
    const int nb = int((width - 1) / B) + 2;
    const int k = nb * (B / 16);
    const unsigned long long warps = n / 32;
    const unsigned grid = unsigned((warps + 7) / 8);
    auto d = static_cast<uint4*>(dst);
    auto s = static_cast<const unsigned char*>(src);
    switch (k) {
        case 4: block_gather_kernel<B, 4, HINT><<<grid, 256, 0, st>>>(d, s, src_n, idx, n, width); break;
        case 6: block_gather_kernel<B, 6, HINT><<<grid, 256, 0, st>>>(d, s, src_n, idx, n, width); break;
        case 8: block_gather_kernel<B, 8, HINT><<<grid, 256, 0, st>>>(d, s, src_n, idx, n, width); break;
        case 10: block_gather_kernel<B, 10, HINT><<<grid, 256, 0, st>>>(d, s, src_n, idx, n, width); break;
        case 12: block_gather_kernel<B, 12, HINT><<<grid, 256, 0, st>>>(d, s, src_n, idx, n, width); break;
        case 16: block_gather_kernel<B, 16, HINT><<<grid, 256, 0, st>>>(d, s, src_n, idx, n, width); break;
        default: return TRV_ERR_UNSUPPORTED;
    }
    return check_launch();
}

}  // namespace
}  // namespace trv

using namespace trv;

extern "C" int32_t trv_probe_block_gather(void* dst, const void* src, uint64_t src_n, const int32_t* idx,
                                          uint64_t n, uint32_t width, uint32_t block_bytes, int32_t l2_hint,
                                          void* stream) {
    if (n == 0) return TRV_OK;
    if (!dst || !src || !idx) return TRV_ERR_INVALID_ARGUMENT;
    if (n % 32 != 0 || n >= (1ull << 31) || width == 0 || width % 4 != 0 || width > 128)
        return TRV_ERR_INVALID_ARGUMENT;
    if (src_n > (1ull << 31) || src_n * width > (1ull << 40)) return TRV_ERR_INVALID_ARGUMENT;
    if (block_bytes != 32 && block_bytes != 64 && block_bytes != 128) return TRV_ERR_UNSUPPORTED;
    if (l2_hint != 0 && l2_hint != 64 && l2_hint != 128) return TRV_ERR_UNSUPPORTED;
    // whole aligned blocks are read: the source must start on a block boundary,
    // and its last block must lie inside the caller's allocation (src_n rows
    // rounded up to a block)
    if (reinterpret_cast<uintptr_t>(src) % block_bytes != 0 || reinterpret_cast<uintptr_t>(dst) % 16 != 0)
        return TRV_ERR_MISALIGNED;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
#define TRV_PROBE_CASE(B)                                                                                  \
    if (block_bytes == B) {                                                                                \
        if (l2_hint == 64) return launch_for_block<B, 64>(dst, src, src_n, idx, n, width, st);           \
        if (l2_hint == 128) return launch_for_block<B, 128>(dst, src, src_n, idx, n, width, st);         \
        return launch_for_block<B, 0>(dst, src, src_n, idx, n, width, st);                               \
    }
    TRV_PROBE_CASE(32)
    TRV_PROBE_CASE(64)
    TRV_PROBE_CASE(128)
#undef TRV_PROBE_CASE
    return TRV_ERR_UNSUPPORTED;
}
