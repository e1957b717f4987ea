// Kernel templates of the C ABI.  Every struct-typed kernel moves
// trove::array<unsigned, S> (S = width / 4) through this library's device API
// (include/trove), so the library's host entry points run exactly the code a
// user kernel written against that API would run.
//
// Work decomposition: a warp owns chunks of 32*U consecutive structs; within
// a chunk lane l owns structs base + u*32 + l (u < U).  All U loads of a
// chunk are issued before its U stores, which keeps U structs per lane in
// flight (the memory-level parallelism HBM needs: ~5 MB in flight chip-wide
// at 6.8 TB/s).  By default the grid has one chunk per warp and the kernels
// have no loop (measured on GB300 a few percent faster than a persistent
// grid-stride grid, and free of the loop's registers); grid-stride forms
// serve a grid chosen through trv_launch.grid_blocks.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <trove/aos.h>
#include <trove/block.h>
#include <trove/ptr.h>

namespace trv {

template <int S>
using aos = trove::array<unsigned, S>;

enum Api { API_WARP = 0, API_BLOCK = 1, API_DIRECT = 2 };

template <int S>
__device__ __forceinline__ bool exits(const aos<S>& v, unsigned modulus) {
    return modulus != 0u && (v.head % modulus) == modulus - 1u;
}

// Load/store of struct i when the caller's warp is converged and its lanes
// address consecutive structs.
template <int S, int API>
__device__ __forceinline__ aos<S> load_conv(const aos<S>* src, long long i) {
    if constexpr (API == API_WARP)
        return trove::load_warp_contiguous(src + i);
    else if constexpr (API == API_BLOCK)
        return trove::load_array_warp_contiguous<S>(reinterpret_cast<const unsigned*>(src), i);
    else
        return src[i];
}

template <int S, int API>
__device__ __forceinline__ void store_conv(aos<S>* dst, long long i, const aos<S>& v) {
    if constexpr (API == API_WARP)
        trove::store_warp_contiguous(v, dst + i);
    else if constexpr (API == API_BLOCK)
        trove::store_array_warp_contiguous(reinterpret_cast<unsigned*>(dst), i, v);
    else
        dst[i] = v;
}

// The same when the warp is not converged.
template <int S, int API>
__device__ __forceinline__ aos<S> load_div(const aos<S>* src, long long i) {
    if constexpr (API == API_BLOCK)
        return trove::load_array<S>(reinterpret_cast<const unsigned*>(src), i);
    else if constexpr (API == API_WARP)
        return trove::detail::divergent_load(src + i);
    else
        return src[i];
}

template <int S, int API>
__device__ __forceinline__ void store_div(aos<S>* dst, long long i, const aos<S>& v) {
    if constexpr (API == API_BLOCK)
        trove::store_array(reinterpret_cast<unsigned*>(dst), i, v);
    else if constexpr (API == API_WARP)
        trove::detail::divergent_store(v, dst + i);
    else
        dst[i] = v;
}

template <int S, int API>
__device__ __forceinline__ aos<S> load_any(const aos<S>* src, long long i) {
    if constexpr (API == API_DIRECT) return src[i];
    if (trove::warp_converged()) return load_conv<S, API>(src, i);
    return load_div<S, API>(src, i);
}

template <int S, int API>
__device__ __forceinline__ void store_any(aos<S>* dst, long long i, const aos<S>& v) {
    if constexpr (API == API_DIRECT) {
        dst[i] = v;
    } else {
        if (trove::warp_converged())
            store_conv<S, API>(dst, i, v);
        else
            store_div<S, API>(dst, i, v);
    }
}

struct WarpGrid {
    int lane;
    long long warp, warps;
    __device__ __forceinline__ WarpGrid() {
        lane = int(threadIdx.x & 31u);
        warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        warps = ((long long)gridDim.x * blockDim.x) >> 5;
    }
};

// dst[i] = src[i], optionally skipping structs whose first word hits the
// early-exit predicate (EXIT).  Full chunks are warp-uniform, so their loads
// run with all 32 lanes; stores after an exit see a partial warp and fall back.
// The one partial chunk at the end of the array is plain per-lane struct
// copies: its transposing form would be a second inlined copy of the tile
// schedule, and every register that copy holds lowers the occupancy of the
// whole kernel.
//
// LOOP = false: the grid has one chunk per warp (the default launch) and the
// kernel has no loop.  The grid-stride loop's 64-bit induction state costs
// 4-8 registers per thread, enough to push narrow structs at U = 1 from 24
// to 32+ registers and below full occupancy (2048 threads per SM), which is
// where a one-chunk kernel gets its loads in flight.  LOOP = true serves
// caller-chosen and persistent grids.
template <int S, int U, int API, bool EXIT>
__device__ __forceinline__ void copy_chunk(const aos<S>* __restrict__ src, aos<S>* __restrict__ dst, long long n,
                                           unsigned modulus, long long base, int lane) {
    constexpr int CH = 32 * U;
    if (base + CH <= n) {
        aos<S> v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = load_conv<S, API>(src, base + u * 32 + lane);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (!EXIT || !exits(v[u], modulus)) {
                if constexpr (EXIT)
                    store_any<S, API>(dst, base + u * 32 + lane, v[u]);
                else
                    store_conv<S, API>(dst, base + u * 32 + lane, v[u]);
            }
        }
    } else {
#pragma unroll 1
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + lane;
            if (i < n) {
                const aos<S> v = src[i];
                if (!EXIT || !exits(v, modulus)) dst[i] = v;
            }
        }
    }
}

template <int S, int U, int API, bool EXIT, bool LOOP>
__global__ void __launch_bounds__(256) copy_kernel(const aos<S>* __restrict__ src, aos<S>* __restrict__ dst,
                                                   long long n, unsigned modulus) {
    const WarpGrid g;
    constexpr int CH = 32 * U;
    if constexpr (LOOP) {
        for (long long base = g.warp * CH; base < n; base += g.warps * CH)
            copy_chunk<S, U, API, EXIT>(src, dst, n, modulus, base, g.lane);
    } else {
        const long long base = g.warp * CH;
        if (base < n) copy_chunk<S, U, API, EXIT>(src, dst, n, modulus, base, g.lane);
    }
}

// MODE 0: coalesced_ptr (trove::load / trove::store); MODE 1: compiler
// direct.  Index loads of a chunk are coalesced; every load of the chunk is
// issued before its stores.
enum { MODE_COALESCED = 0, MODE_DIRECT = 1 };

template <int S, int U, int MODE>
__global__ void __launch_bounds__(256)
gather_kernel(const aos<S>* __restrict__ src, long long src_n, const int* __restrict__ idx,
              aos<S>* __restrict__ dst, long long n) {
    const WarpGrid g;
    constexpr int CH = 32 * U;
    trove::coalesced_ptr<aos<S> > S_(const_cast<aos<S>*>(src));
    trove::coalesced_ptr<aos<S> > D_(dst);
    for (long long base = g.warp * CH; base < n; base += g.warps * CH) {
        int id[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + g.lane;
            id[u] = i < n ? __ldg(idx + i) : -1;
        }
        aos<S> v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (id[u] >= 0 && (long long)id[u] < src_n) {
                if constexpr (MODE == MODE_COALESCED)
                    v[u] = S_[id[u]];
                else
                    v[u] = src[id[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + g.lane;
            if (id[u] >= 0 && (long long)id[u] < src_n) {
                if constexpr (MODE == MODE_COALESCED)
                    D_[i] = v[u];
                else
                    dst[i] = v[u];
            }
        }
    }
}

template <int S, int U, int MODE>
__global__ void __launch_bounds__(256)
scatter_kernel(const aos<S>* __restrict__ src, const int* __restrict__ idx, aos<S>* __restrict__ dst,
               long long dst_n, long long n) {
    const WarpGrid g;
    constexpr int CH = 32 * U;
    trove::coalesced_ptr<aos<S> > S_(const_cast<aos<S>*>(src));
    trove::coalesced_ptr<aos<S> > D_(dst);
    for (long long base = g.warp * CH; base < n; base += g.warps * CH) {
        int id[U];
        aos<S> v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + g.lane;
            id[u] = i < n ? __ldg(idx + i) : -1;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + g.lane;
            if (i < n) {
                if constexpr (MODE == MODE_COALESCED)
                    v[u] = S_[i];
                else
                    v[u] = src[i];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (id[u] >= 0 && (long long)id[u] < dst_n) {
                if constexpr (MODE == MODE_COALESCED)
                    D_[id[u]] = v[u];
                else
                    dst[id[u]] = v[u];
            }
        }
    }
}

// ---- cache policies of the row-form kernels ----------------------------
// 0: default (read-only path for loads, plain stores)
// 1: the index stream and the contiguous side are streamed (evict-first), so
//    L2 keeps the random side's sectors: structs narrower than a 32-byte
//    sector share sectors, and a sector that stays in L2 is fetched once
// 2: as 1, and the random side bypasses L1 (L2 only)
// 3: as 1, and the random side is marked evict-last in L2
// 4: as 1, and random-side loads carry a 64-byte L2 prefetch-size hint
__device__ __forceinline__ unsigned long long l2_evict_last_policy() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ int ld_index(const int* p, int policy) { return policy ? __ldcs(p) : __ldg(p); }

__device__ __forceinline__ uint4 ld_hint(const uint4* p, unsigned long long pol) {
    uint4 v;
    asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ uint2 ld_hint(const uint2* p, unsigned long long pol) {
    uint2 v;
    asm volatile("ld.global.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(v.x), "=r"(v.y) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ unsigned ld_hint(const unsigned* p, unsigned long long pol) {
    unsigned v;
    asm volatile("ld.global.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_hint(uint4* p, uint4 v, unsigned long long pol) {
    asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "r"(v.x), "r"(v.y),
                 "r"(v.z), "r"(v.w), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void st_hint(uint2* p, uint2 v, unsigned long long pol) {
    asm volatile("st.global.L2::cache_hint.v2.u32 [%0], {%1, %2}, %3;" ::"l"(p), "r"(v.x), "r"(v.y), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void st_hint(unsigned* p, unsigned v, unsigned long long pol) {
    asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

// Random-side loads with a 64-byte L2 prefetch-size hint: on a miss L2 is
// asked for the 64-byte half line holding the word instead of the whole
// 128-byte line.
__device__ __forceinline__ uint4 ld_pf64(const uint4* p) {
    uint4 v;
    asm volatile("ld.global.nc.L2::64B.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}
__device__ __forceinline__ uint2 ld_pf64(const uint2* p) {
    uint2 v;
    asm volatile("ld.global.nc.L2::64B.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ unsigned ld_pf64(const unsigned* p) {
    unsigned v;
    asm volatile("ld.global.nc.L2::64B.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// The same with a 128-byte prefetch-size hint: a miss fetches the whole
// 128-byte line, whose neighbouring structs a narrow gather over a source
// near the L2 size often reads while the line is still cached.
__device__ __forceinline__ uint4 ld_pf128(const uint4* p) {
    uint4 v;
    asm volatile("ld.global.nc.L2::128B.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}
__device__ __forceinline__ uint2 ld_pf128(const uint2* p) {
    uint2 v;
    asm volatile("ld.global.nc.L2::128B.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ unsigned ld_pf128(const unsigned* p) {
    unsigned v;
    asm volatile("ld.global.nc.L2::128B.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

template <typename V>
__device__ __forceinline__ V ld_random(const V* p, int policy, unsigned long long pol) {
    if (policy == 5) return ld_pf128(p);
    if (policy == 4) return ld_pf64(p);
    if (policy == 3) return ld_hint(p, pol);
    if (policy == 2) return __ldcg(p);
    return __ldg(p);
}
template <typename V>
__device__ __forceinline__ V ld_contig(const V* p, int policy) {
    return policy ? __ldcs(p) : __ldg(p);
}
template <typename V>
__device__ __forceinline__ void st_random(V* p, V v, int policy, unsigned long long pol) {
    if (policy == 3)
        st_hint(p, v, pol);
    else if (policy == 2)
        __stcg(p, v);
    else
        *p = v;
}
template <typename V>
__device__ __forceinline__ void st_contig(V* p, V v, int policy) {
    if (policy)
        __stcs(p, v);
    else
        *p = v;
}

// Row-form gather / scatter (TRV_PATH_WARP for index ops).  The C ABI knows
// both sides of the operation, and one side is contiguous, so no struct ever
// needs to sit in one lane: the warp moves 32 structs as m = 4S/sizeof(V)
// rounds of 32 words V.  In round k lane l carries word q = l + 32k of the
// chunk, i.e. word q % m of struct j = q / m, whose index comes from lane j
// by one 32-bit shuffle.  Gather: the random side is the load (adjacent lanes
// read adjacent words of one struct in the same instruction), the store lands
// at word q of the contiguous destination chunk (fully coalesced).  Scatter is
// the mirror image.  No transposes, no 64-bit pointer broadcasts.
template <int S, typename V, int U>
__global__ void __launch_bounds__(256)
gather_rows_kernel(const V* __restrict__ src, long long src_n, const int* __restrict__ idx, V* __restrict__ dst,
                   long long n, int policy) {
    constexpr int m = S * 4 / int(sizeof(V));
    const WarpGrid g;
    constexpr int CH = 32 * U;
    const unsigned long long pol = policy == 3 ? l2_evict_last_policy() : 0ull;
    for (long long base = g.warp * CH; base < n; base += g.warps * CH) {
        int id[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + g.lane;
            const int v = i < n ? ld_index(idx + i, policy) : -1;
            id[u] = (v >= 0 && (long long)v < src_n) ? v : -1;
        }
        V val[U][m];
        int from[U][m];
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int k = 0; k < m; ++k) {
                const int q = g.lane + 32 * k;
                const int j = q / m;
                from[u][k] = __shfl_sync(0xFFFFFFFFu, id[u], j);
                if (from[u][k] >= 0) val[u][k] = ld_random(src + (long long)from[u][k] * m + (q - j * m), policy, pol);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int k = 0; k < m; ++k)
                if (from[u][k] >= 0) st_contig(dst + (base + u * 32) * m + g.lane + 32 * k, val[u][k], policy);
        }
    }
}

template <int S, typename V, int U>
__global__ void __launch_bounds__(256)
scatter_rows_kernel(const V* __restrict__ src, const int* __restrict__ idx, V* __restrict__ dst, long long dst_lo,
                    long long dst_hi, long long n, int policy) {
    constexpr int m = S * 4 / int(sizeof(V));
    const WarpGrid g;
    constexpr int CH = 32 * U;
    const unsigned long long pol = policy == 3 ? l2_evict_last_policy() : 0ull;
    for (long long base = g.warp * CH; base < n; base += g.warps * CH) {
        int id[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long i = base + u * 32 + g.lane;
            const int v = i < n ? ld_index(idx + i, policy) : -1;
            id[u] = ((long long)v >= dst_lo && (long long)v < dst_hi) ? v : -1;  // dst_lo >= 0
        }
        V val[U][m];
        int to[U][m];
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int k = 0; k < m; ++k) {
                const int q = g.lane + 32 * k;
                to[u][k] = __shfl_sync(0xFFFFFFFFu, id[u], q / m);
                if (to[u][k] >= 0) val[u][k] = ld_contig(src + (base + u * 32) * m + q, policy);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int k = 0; k < m; ++k) {
                const int q = g.lane + 32 * k;
                if (to[u][k] >= 0) st_random(dst + (long long)to[u][k] * m + (q - (q / m) * m), val[u][k], policy, pol);
            }
        }
    }
}

// Row-form gather / scatter with the word count m given at run time: one
// kernel per word type serves every width that is a multiple of 4 bytes,
// including structs wider than the per-width tables cover (> 64 bytes).  Same
// scheme as the compile-time kernels above; the m rounds of a chunk run in
// groups of G so the live registers stay bounded for any m.
template <typename V, int G, bool GATHER>
__global__ void __launch_bounds__(256)
index_rows_rt_kernel(const V* __restrict__ src, const int* __restrict__ idx, V* __restrict__ dst, long long bound,
                     long long n, int m, int policy) {
    const WarpGrid g;
    const unsigned long long pol = policy == 3 ? l2_evict_last_policy() : 0ull;
    for (long long base = g.warp * 32; base < n; base += g.warps * 32) {
        const long long i = base + g.lane;
        const int v = i < n ? ld_index(idx + i, policy) : -1;
        const int id = (v >= 0 && (long long)v < bound) ? v : -1;
        for (int k0 = 0; k0 < m; k0 += G) {
            V val[G];
            int other[G];
#pragma unroll
            for (int t = 0; t < G; ++t) {
                const int k = k0 + t;
                other[t] = -1;
                if (k < m) {  // m is uniform: the whole warp takes the same branch
                    const int q = g.lane + 32 * k;
                    const int j = q / m;
                    other[t] = __shfl_sync(0xFFFFFFFFu, id, j);
                    if (other[t] >= 0)
                        val[t] = GATHER ? ld_random(src + (long long)other[t] * m + (q - j * m), policy, pol)
                                        : ld_contig(src + base * m + q, policy);
                }
            }
#pragma unroll
            for (int t = 0; t < G; ++t) {
                if (other[t] < 0) continue;
                const int q = g.lane + 32 * (k0 + t);
                if (GATHER)
                    st_contig(dst + base * m + q, val[t], policy);
                else
                    st_random(dst + (long long)other[t] * m + (q % m), val[t], policy, pol);
            }
        }
    }
}

// AoS <-> SoA for structs of S 32-bit fields: field j of struct i sits at
// aos[i].word(j) and soa[j * n + i].  The AoS side moves through the device
// API (load/store_warp_contiguous: coalesced rounds + transpose); the SoA side
// is S coalesced 32-bit streams, one per field.
// One chunk of 32*U structs; the partial chunk at the end moves per lane.
template <int S, int U>
__device__ __forceinline__ void aos_to_soa_chunk(const aos<S>* __restrict__ src, unsigned* __restrict__ dst,
                                                 long long n, long long base, int lane) {
    constexpr int CH = 32 * U;
    aos<S> v[U];
    const bool full = base + CH <= n;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const long long i = base + u * 32 + lane;
        if (full)
            v[u] = trove::load_warp_contiguous(src + i);
        else if (i < n)
            v[u] = src[i];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const long long i = base + u * 32 + lane;
        if (!full && i >= n) continue;
        const trove::detail::regs<unsigned, S> w = trove::detail::to_regs(v[u]);
#pragma unroll
        for (int j = 0; j < S; ++j) __stcs(dst + (long long)j * n + i, w.v[j]);
    }
}

template <int S, int U>
__device__ __forceinline__ void soa_to_aos_chunk(const unsigned* __restrict__ src, aos<S>* __restrict__ dst,
                                                 long long n, long long base, int lane) {
    constexpr int CH = 32 * U;
    const bool full = base + CH <= n;
    trove::detail::regs<unsigned, S> w[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const long long i = base + u * 32 + lane;
        if (full || i < n) {
#pragma unroll
            for (int j = 0; j < S; ++j) w[u].v[j] = __ldcs(src + (long long)j * n + i);
        }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const long long i = base + u * 32 + lane;
        const aos<S> v = trove::detail::from_regs(w[u]);
        if (full)
            trove::store_warp_contiguous(v, dst + i);
        else if (i < n)
            dst[i] = v;
    }
}

// LOOP as for copy_kernel: false = one chunk per warp (the default grid).
template <int S, int U, bool LOOP>
__global__ void __launch_bounds__(256)
aos_to_soa_kernel(const aos<S>* __restrict__ src, unsigned* __restrict__ dst, long long n) {
    const WarpGrid g;
    constexpr int CH = 32 * U;
    if constexpr (LOOP) {
        for (long long base = g.warp * CH; base < n; base += g.warps * CH)
            aos_to_soa_chunk<S, U>(src, dst, n, base, g.lane);
    } else {
        const long long base = g.warp * CH;
        if (base < n) aos_to_soa_chunk<S, U>(src, dst, n, base, g.lane);
    }
}

template <int S, int U, bool LOOP>
__global__ void __launch_bounds__(256)
soa_to_aos_kernel(const unsigned* __restrict__ src, aos<S>* __restrict__ dst, long long n) {
    const WarpGrid g;
    constexpr int CH = 32 * U;
    if constexpr (LOOP) {
        for (long long base = g.warp * CH; base < n; base += g.warps * CH)
            soa_to_aos_chunk<S, U>(src, dst, n, base, g.lane);
    } else {
        const long long base = g.warp * CH;
        if (base < n) soa_to_aos_chunk<S, U>(src, dst, n, base, g.lane);
    }
}

}  // namespace trv
