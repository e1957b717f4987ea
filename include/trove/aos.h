// Low-level AoS API: warp-contiguous loads and stores, and the converged /
// divergent load() and store() used by coalesced_ptr.
//
// Interface of the reference trove/aos.h:66-105 (load_warp_contiguous,
// store_warp_contiguous) and :258-290 (load, store), plus the dispatch traits
// detail::size_in_range / use_shfl / use_direct (:40-61).
//
// load_warp_contiguous<n>(p): the caller's tile of n lanes is converged and
// lane i passes p_0 + i.  The tile reads its n*sizeof(T) bytes as m
// coalesced rounds of a word type U, then transposes rows to columns in
// registers (transpose.h).  U is the widest of int4 / int2 / int that divides
// sizeof(T); when the tile's start address is not aligned to U (checked at
// run time, uniform across the tile) every lane moves its own struct with
// the widest words its address allows.  One-word structs and structs of more
// words than the tile has lanes are read per lane.
//
// load(p) / store(v, p) take any pointers.  On a fully converged warp, a
// broadcast of lane 0's pointer and one __ballot_sync tell whether the
// pointers are consecutive:
// if so the warp-contiguous path runs; if not, structs of 2..32 words move as
// cooperative rounds (each struct read by adjacent lanes in one instruction)
// plus a transpose, and one-word structs move per lane.  A partial warp moves
// every struct per lane with the widest aligned words.
#pragma once

#include <trove/detail/dismember.h>
#include <trove/detail/fallback.h>
#include <trove/memory.h>
#include <trove/transpose.h>
#include <trove/utility.h>
#include <trove/warp.h>

namespace trove {
namespace detail {

template <typename T, std::size_t tile_size>
struct size_in_range {
    typedef typename dismember_type<T>::type U;
    static const int size = aliased_size<T, U>::value;
    static const bool value = (size > 1) && (size <= int(tile_size));
};

template <typename T, std::size_t tile_size>
struct use_shfl {
    static const bool value =
        size_multiple_power_of_two<T, 2>::value && size_in_range<T, tile_size>::value;
};

template <typename T, std::size_t tile_size>
struct use_direct {
    static const bool value = !use_shfl<T, tile_size>::value;
};

template <std::size_t n, typename U, typename T>
TROVE_D T tile_load_as(const T* src, int lane) {
    constexpr int m = aliased_size<T, U>::value;
    if constexpr (m == 1 || m > int(n)) {
        return load_words<T, U>(src);
    } else {
        const U* base = reinterpret_cast<const U*>(src - lane);
        regs<U, m> r;
#pragma unroll
        for (int k = 0; k < m; ++k) r.v[k] = base[lane + k * int(n)];
        r2c_block(r, thread_tile<n>());
        return fuse_regs<T>(r);
    }
}

template <std::size_t n, typename U, typename T>
TROVE_D void tile_store_as(const T& data, T* dst, int lane) {
    constexpr int m = aliased_size<T, U>::value;
    if constexpr (m == 1 || m > int(n)) {
        store_words<T, U>(data, dst);
    } else {
        U* base = reinterpret_cast<U*>(dst - lane);
        regs<U, m> r = lyse_regs<U>(data);
        c2r_block(r, thread_tile<n>());
#pragma unroll
        for (int k = 0; k < m; ++k) base[lane + k * int(n)] = r.v[k];
    }
}

// Only the widest word's tile schedule is compiled in.  A tile whose start is
// not aligned to that word (possible when alignof(T) is smaller) moves per
// lane instead: the same bytes, less coalesced, and no second transposition
// schedule holding registers in every kernel that uses this path (a second
// and third schedule raised a 64-byte copy kernel from 32 to 47 registers).
template <std::size_t n, typename T>
TROVE_D T contiguous_load(const T* src) {
    if constexpr (sizeof(T) % 4 != 0) {
        return *src;
    } else {
        typedef typename dismember_type<T>::type Umax;
        const int lane = int(lane_id() & unsigned(n - 1));
        if constexpr (alignof(T) >= sizeof(Umax)) {
            return tile_load_as<n, Umax>(src, lane);
        } else {
            const std::uintptr_t base = reinterpret_cast<std::uintptr_t>(src - lane);
            if ((base & (sizeof(Umax) - 1)) == 0) return tile_load_as<n, Umax>(src, lane);
            return divergent_load(src);
        }
    }
}

template <std::size_t n, typename T>
TROVE_D void contiguous_store(const T& data, T* dst) {
    if constexpr (sizeof(T) % 4 != 0) {
        *dst = data;
    } else {
        typedef typename dismember_type<T>::type Umax;
        const int lane = int(lane_id() & unsigned(n - 1));
        if constexpr (alignof(T) >= sizeof(Umax)) {
            tile_store_as<n, Umax>(data, dst, lane);
        } else {
            const std::uintptr_t base = reinterpret_cast<std::uintptr_t>(dst - lane);
            if ((base & (sizeof(Umax) - 1)) == 0) return tile_store_as<n, Umax>(data, dst, lane);
            divergent_store(data, dst);
        }
    }
}

// Warp-cooperative access to 32 unrelated structs (one pointer per lane),
// in units of U, m = sizeof(T) / sizeof(U) words per struct.  The 32 structs
// form a 32 x m block of words in lane order; round k (k < m) has lane l move
// word q = l + 32k of that block: word q % m of the struct whose pointer lane
// q / m broadcasts.  Lanes reading the same struct read adjacent words in the
// same instruction, so every struct costs one sector group per round instead
// of m separate per-lane accesses; the rounds are the row form of the
// transposition, which converts them to one struct per lane (and back for
// stores).
// The random-row loads of gather_rows_load carry a 64-byte L2 prefetch-size
// hint for structs of 20 bytes and more (otherwise they are ordinary coherent
// loads): on a miss, L2 fetches the 64-byte half line holding the word instead
// of a whole 128-byte line on GPUs whose default fetch is a whole line, which
// halves the DRAM bytes read for structs scattered at random.  Measured on a
// GB300 through coalesced_ptr gathers of 2^24 structs: runs of 32 +4.5 to
// +11 % from 20 bytes up, permutations +2.5 to +6.6 % from 28 bytes up, but
// 12-byte permutations -7.5 %, so narrower structs keep plain loads.
TROVE_D int load_row_word(const int* p) {
#if defined(__CUDA_ARCH__)
    int v;
    asm volatile("ld.global.L2::64B.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
#else
    return *p;
#endif
}
TROVE_D int2 load_row_word(const int2* p) {
#if defined(__CUDA_ARCH__)
    int2 v;
    asm volatile("ld.global.L2::64B.v2.b32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p) : "memory");
    return v;
#else
    return *p;
#endif
}
TROVE_D int4 load_row_word(const int4* p) {
#if defined(__CUDA_ARCH__)
    int4 v;
    asm volatile("ld.global.L2::64B.v4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
#else
    return *p;
#endif
}

template <typename U, typename T>
TROVE_D T gather_rows_load(const T* src) {
    constexpr int m = aliased_size<T, U>::value;
    const int lane = int(lane_id());
    regs<U, m> r;
#pragma unroll
    for (int k = 0; k < m; ++k) {
        const int q = lane + 32 * k;
        const int j = q / m;
        const T* pj = shfl_any(src, j, 0xFFFFFFFFu, 32);
        const U* w = reinterpret_cast<const U*>(pj) + (q - j * m);
        if constexpr (sizeof(T) >= 20)
            r.v[k] = load_row_word(w);
        else
            r.v[k] = *w;
    }
    r2c_block(r, thread_tile<32>());
    return fuse_regs<T>(r);
}

template <typename U, typename T>
TROVE_D void scatter_rows_store(const T& data, T* dst) {
    constexpr int m = aliased_size<T, U>::value;
    const int lane = int(lane_id());
    regs<U, m> r = lyse_regs<U>(data);
    c2r_block(r, thread_tile<32>());
#pragma unroll
    for (int k = 0; k < m; ++k) {
        const int q = lane + 32 * k;
        const int j = q / m;
        T* pj = shfl_any(dst, j, 0xFFFFFFFFu, 32);
        reinterpret_cast<U*>(pj)[q - j * m] = r.v[k];
    }
}

// Widest word that divides sizeof(T) and that every lane's pointer is aligned
// to, as log2 of its size (2, 3 or 4); 0 when some pointer is not 4-byte
// aligned.  One vote, converged warp only.
template <typename T>
TROVE_D int warp_word_log2(const void* p) {
    typedef typename dismember_type<T>::type Umax;
    const unsigned a = unsigned(reinterpret_cast<std::uintptr_t>(p));
    const unsigned any = __reduce_or_sync(0xFFFFFFFFu, a & 15u);
    if (sizeof(Umax) == 16 && (any & 15u) == 0) return 4;
    if (sizeof(Umax) >= 8 && (any & 7u) == 0) return 3;
    return (any & 3u) == 0 ? 2 : 0;
}

// Converged-warp load of 32 arbitrary structs.  When every pointer is aligned
// to the struct's widest word U: a one-word struct is one vector access per
// lane, a 2..32-word struct moves as cooperative rounds of U.  Less aligned
// pointers use the widest word they allow.
template <typename T>
TROVE_D T warp_gather_load(const T* src) {
    typedef typename dismember_type<T>::type Umax;
    constexpr int mmax = aliased_size<T, Umax>::value;
    const int lg = warp_word_log2<T>(src);
    if (lg == floor_log2(int(sizeof(Umax)))) {
        if constexpr (mmax == 1) return divergent_load(src);
        if constexpr (mmax >= 2 && mmax <= 32) return gather_rows_load<Umax>(src);
    }
    if constexpr (sizeof(T) % 8 == 0 && sizeof(T) / 8 >= 2 && sizeof(T) / 8 <= 32)
        if (lg >= 3) return gather_rows_load<int2>(src);
    if constexpr (sizeof(T) / 4 >= 2 && sizeof(T) / 4 <= 32)
        if (lg >= 2) return gather_rows_load<int>(src);
    return divergent_load(src);
}

template <typename T>
TROVE_D void warp_scatter_store(const T& data, T* dst) {
    typedef typename dismember_type<T>::type Umax;
    constexpr int mmax = aliased_size<T, Umax>::value;
    const int lg = warp_word_log2<T>(dst);
    if (lg == floor_log2(int(sizeof(Umax)))) {
        if constexpr (mmax == 1) return divergent_store(data, dst);
        if constexpr (mmax >= 2 && mmax <= 32) return scatter_rows_store<Umax>(data, dst);
    }
    if constexpr (sizeof(T) % 8 == 0 && sizeof(T) / 8 >= 2 && sizeof(T) / 8 <= 32)
        if (lg >= 3) return scatter_rows_store<int2>(data, dst);
    if constexpr (sizeof(T) / 4 >= 2 && sizeof(T) / 4 <= 32)
        if (lg >= 2) return scatter_rows_store<int>(data, dst);
    divergent_store(data, dst);
}

// For a fully converged warp: do lanes 0..31 address consecutive structs in
// lane order?  Lane 0's address is broadcast and one __ballot_sync checks
// every lane against it (cheaper than a match over 32 distinct addresses,
// which the random case would pay on every access).
template <typename T>
TROVE_D bool warp_consecutive(const T* p) {
    const unsigned long long a = static_cast<unsigned long long>(reinterpret_cast<std::uintptr_t>(p));
    const unsigned long long a0 = __shfl_sync(0xFFFFFFFFu, a, 0);
    const bool mine = a == a0 + static_cast<unsigned long long>(lane_id()) * sizeof(T);
    return __ballot_sync(0xFFFFFFFFu, mine) == 0xFFFFFFFFu;
}

}  // namespace detail

template <std::size_t tile_size = WARP_SIZE, typename T>
TROVE_D T load_warp_contiguous(const T* src) {
    return detail::contiguous_load<tile_size>(src);
}

template <std::size_t tile_size = WARP_SIZE, typename T>
TROVE_D void store_warp_contiguous(const T& data, T* dest) {
    detail::contiguous_store<tile_size>(data, dest);
}

template <typename T>
TROVE_D T load(const T* src) {
    // A struct of one widest word is one access per lane whether or not the
    // warp's pointers are consecutive: no vote needed.
    if constexpr (sizeof(T) % 4 == 0 && sizeof(T) != sizeof(typename detail::dismember_type<T>::type)) {
        if (warp_converged()) {
            if (detail::warp_consecutive(src)) return detail::contiguous_load<WARP_SIZE>(src);
            return detail::warp_gather_load(src);
        }
    }
    return detail::divergent_load(src);
}

template <typename T>
TROVE_D void store(const T& data, T* dest) {
    if constexpr (sizeof(T) % 4 == 0 && sizeof(T) != sizeof(typename detail::dismember_type<T>::type)) {
        if (warp_converged()) {
            if (detail::warp_consecutive(dest))
                detail::contiguous_store<WARP_SIZE>(data, dest);
            else
                detail::warp_scatter_store(data, dest);
            return;
        }
    }
    detail::divergent_store(data, dest);
}

}  // namespace trove
