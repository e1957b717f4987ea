// Width-agnostic kernels: the flat vector copy (TRV_PATH_VECTOR), the TMA
// bulk copy (TRV_PATH_BULK), byte-wise gather/scatter for widths the struct
// kernels do not cover, and the seeded input generator.
#include <cuda_runtime.h>
#include <stdint.h>

#include "flat.h"

namespace trv {

// ---- seeded input stream (stream_word, flat.h) --------------------------
__global__ void fill_u32_kernel(unsigned* __restrict__ dst, long long nwords, unsigned long long seed) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nwords; k += stride)
        dst[k] = stream_word(seed, (unsigned long long)k);
}

void launch_fill_u32(unsigned* dst, long long nwords, unsigned long long seed, int grid, cudaStream_t st) {
    fill_u32_kernel<<<grid, 256, 0, st>>>(dst, nwords, seed);
}

// idx[i] = stream_bounded(seed, i, bound): n indices uniform in [0, bound).
__global__ void uniform_indices_kernel(int* __restrict__ idx, long long n, unsigned bound, unsigned long long seed) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
        idx[k] = (int)stream_bounded(seed, (unsigned long long)k, bound);
}

void launch_uniform_indices(int* idx, long long n, unsigned bound, unsigned long long seed, int grid,
                            cudaStream_t st) {
    uniform_indices_kernel<<<grid, 256, 0, st>>>(idx, n, bound, seed);
}

// Run pattern over n >= 32 indices: output chunk c (32 aligned outputs) is,
// when bit 0 of word 2c is set, a run start + 0..31 with start drawn from
// word 2c + 1 over [0, n - 32]; otherwise 32 independent draws over [0, n)
// from the stream seed ^ 0x5bd1e995 at the output's own position.  Every
// output depends only on its chunk, so one thread per output.
__global__ void run_indices_kernel(int* __restrict__ idx, long long n, unsigned long long seed) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const unsigned long long c = (unsigned long long)k >> 5;
        if (stream_word(seed, 2 * c) & 1u)
            idx[k] = (int)(stream_bounded(seed, 2 * c + 1, (unsigned)(n - 31)) + (unsigned)(k & 31));
        else
            idx[k] = (int)stream_bounded(seed ^ 0x5bd1e995ull, (unsigned long long)k, (unsigned)n);
    }
}

void launch_run_indices(int* idx, long long n, unsigned long long seed, int grid, cudaStream_t st) {
    run_indices_kernel<<<grid, 256, 0, st>>>(idx, n, seed);
}

// ---- flat vector copy ----------------------------------------------------
// Copies nbytes from s to d.  The first `head` bytes bring both pointers to
// V alignment; the aligned middle moves as V vectors, U per thread per pass
// (all U loads issued before the stores); block 0 also copies the head and
// the sub-vector tail byte by byte.
template <typename V, int U>
__global__ void __launch_bounds__(256)
flat_copy_kernel(const unsigned char* __restrict__ s, unsigned char* __restrict__ d, long long nbytes,
                 int head) {
    const long long body = (nbytes - head) / (long long)sizeof(V);
    const V* __restrict__ sv = reinterpret_cast<const V*>(s + head);
    V* __restrict__ dv = reinterpret_cast<V*>(d + head);
    const long long step = (long long)gridDim.x * blockDim.x * U;
    for (long long base = (long long)blockIdx.x * blockDim.x * U + threadIdx.x; base < body; base += step) {
        V r[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long k = base + (long long)u * blockDim.x;
            if (k < body) r[u] = __ldg(sv + k);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long k = base + (long long)u * blockDim.x;
            if (k < body) __stcs(dv + k, r[u]);
        }
    }
    if (blockIdx.x == 0) {
        const long long tail_begin = head + body * (long long)sizeof(V);
        if ((long long)threadIdx.x < head) d[threadIdx.x] = s[threadIdx.x];
        const long long t = tail_begin + threadIdx.x;
        if (t < nbytes) d[t] = s[t];
    }
}

template <typename V, int U>
static void launch_flat_v(const unsigned char* s, unsigned char* d, long long nbytes, int head, int grid,
                          cudaStream_t st) {
    flat_copy_kernel<V, U><<<grid, 256, 0, st>>>(s, d, nbytes, head);
}

const void* flat_copy_func(int vec_bytes, int unroll) {
#define TRV_FLAT_FUNC(V, U) \
    if (sizeof(V) == (size_t)vec_bytes && U == unroll) return (const void*)&flat_copy_kernel<V, U>;
    TRV_FLAT_FUNC(uint4, 1) TRV_FLAT_FUNC(uint4, 2) TRV_FLAT_FUNC(uint4, 4) TRV_FLAT_FUNC(uint4, 8)
    TRV_FLAT_FUNC(uint2, 1) TRV_FLAT_FUNC(uint2, 2) TRV_FLAT_FUNC(uint2, 4) TRV_FLAT_FUNC(uint2, 8)
    TRV_FLAT_FUNC(unsigned, 1) TRV_FLAT_FUNC(unsigned, 2) TRV_FLAT_FUNC(unsigned, 4) TRV_FLAT_FUNC(unsigned, 8)
    TRV_FLAT_FUNC(unsigned char, 1) TRV_FLAT_FUNC(unsigned char, 2) TRV_FLAT_FUNC(unsigned char, 4)
    TRV_FLAT_FUNC(unsigned char, 8)
#undef TRV_FLAT_FUNC
    return nullptr;
}

void launch_flat_copy(const void* src, void* dst, long long nbytes, int vec_bytes, int head, int unroll, int grid,
                      cudaStream_t st) {
    const unsigned char* s = static_cast<const unsigned char*>(src);
    unsigned char* d = static_cast<unsigned char*>(dst);
#define TRV_FLAT_CASE(V)                                                  \
    switch (unroll) {                                                     \
        case 1: launch_flat_v<V, 1>(s, d, nbytes, head, grid, st); break; \
        case 2: launch_flat_v<V, 2>(s, d, nbytes, head, grid, st); break; \
        case 4: launch_flat_v<V, 4>(s, d, nbytes, head, grid, st); break; \
        default: launch_flat_v<V, 8>(s, d, nbytes, head, grid, st); break; \
    }
    switch (vec_bytes) {
        case 16: TRV_FLAT_CASE(uint4) break;
        case 8: TRV_FLAT_CASE(uint2) break;
        case 4: TRV_FLAT_CASE(unsigned) break;
        default: TRV_FLAT_CASE(unsigned char) break;
    }
#undef TRV_FLAT_CASE
}

// ---- byte-wise gather / scatter for widths outside 4..64 step 4 ----------
__global__ void gather_bytes_kernel(const unsigned char* __restrict__ s, long long src_n,
                                    const int* __restrict__ idx, unsigned char* __restrict__ d, long long n,
                                    unsigned width) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int j = idx[i];
        if (j < 0 || (long long)j >= src_n) continue;
        const unsigned char* p = s + (long long)j * width;
        unsigned char* q = d + i * (long long)width;
        for (unsigned b = 0; b < width; ++b) q[b] = p[b];
    }
}

__global__ void scatter_bytes_kernel(const unsigned char* __restrict__ s, const int* __restrict__ idx,
                                     unsigned char* __restrict__ d, long long dst_n, long long n,
                                     unsigned width) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int j = idx[i];
        if (j < 0 || (long long)j >= dst_n) continue;
        const unsigned char* p = s + i * (long long)width;
        unsigned char* q = d + (long long)j * width;
        for (unsigned b = 0; b < width; ++b) q[b] = p[b];
    }
}

void launch_gather_bytes(const void* src, long long src_n, const int* idx, void* dst, long long n,
                         unsigned width, int grid, cudaStream_t st) {
    gather_bytes_kernel<<<grid, 256, 0, st>>>(static_cast<const unsigned char*>(src), src_n, idx,
                                              static_cast<unsigned char*>(dst), n, width);
}

void launch_scatter_bytes(const void* src, const int* idx, void* dst, long long dst_n, long long n,
                          unsigned width, int grid, cudaStream_t st) {
    scatter_bytes_kernel<<<grid, 256, 0, st>>>(static_cast<const unsigned char*>(src), idx,
                                               static_cast<unsigned char*>(dst), dst_n, n, width);
}

}  // namespace trv
