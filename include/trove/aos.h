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
// sizeof(T) AND that the tile's start address is aligned to, checked at run
// time (uniform across the tile, so it costs one branch).  One-word structs
// and structs of more words than the tile has lanes are read per lane.
//
// load(p) / store(v, p) take any pointers: when the whole warp is converged
// and its pointers are consecutive (one __match_any_sync on p - lane) they
// take the warp-contiguous path; otherwise every lane moves its own struct
// with the widest aligned words (sector-minimal per-thread access, no
// shuffles, no pointer broadcast).
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

template <std::size_t n, typename T>
TROVE_D T contiguous_load(const T* src) {
    if constexpr (sizeof(T) % 4 != 0) {
        return *src;
    } else {
        typedef typename dismember_type<T>::type Umax;
        const int lane = int(lane_id() & unsigned(n - 1));
        const std::uintptr_t base = reinterpret_cast<std::uintptr_t>(src - lane);
        if constexpr (sizeof(Umax) == 16) {
            if ((base & 15) == 0) return tile_load_as<n, int4>(src, lane);
        }
        if constexpr (sizeof(Umax) >= 8) {
            if ((base & 7) == 0) return tile_load_as<n, int2>(src, lane);
        }
        if constexpr (alignof(T) < 4) {
            if ((base & 3) != 0) return *src;
        }
        return tile_load_as<n, int>(src, lane);
    }
}

template <std::size_t n, typename T>
TROVE_D void contiguous_store(const T& data, T* dst) {
    if constexpr (sizeof(T) % 4 != 0) {
        *dst = data;
    } else {
        typedef typename dismember_type<T>::type Umax;
        const int lane = int(lane_id() & unsigned(n - 1));
        const std::uintptr_t base = reinterpret_cast<std::uintptr_t>(dst - lane);
        if constexpr (sizeof(Umax) == 16) {
            if ((base & 15) == 0) return tile_store_as<n, int4>(data, dst, lane);
        }
        if constexpr (sizeof(Umax) >= 8) {
            if ((base & 7) == 0) return tile_store_as<n, int2>(data, dst, lane);
        }
        if constexpr (alignof(T) < 4) {
            if ((base & 3) != 0) {
                *dst = data;
                return;
            }
        }
        tile_store_as<n, int>(data, dst, lane);
    }
}

// For a fully converged warp: do lanes 0..31 address consecutive structs in
// lane order?  Lanes agree on p - lane exactly when they do.
template <typename T>
TROVE_D bool warp_consecutive(const T* p) {
    const unsigned long long key =
        static_cast<unsigned long long>(reinterpret_cast<std::uintptr_t>(p)) -
        static_cast<unsigned long long>(lane_id()) * sizeof(T);
    return __match_any_sync(0xFFFFFFFFu, key) == 0xFFFFFFFFu;
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
    if constexpr (sizeof(T) % 4 == 0) {
        if (warp_converged() && detail::warp_consecutive(src))
            return detail::contiguous_load<WARP_SIZE>(src);
    }
    return detail::divergent_load(src);
}

template <typename T>
TROVE_D void store(const T& data, T* dest) {
    if constexpr (sizeof(T) % 4 == 0) {
        if (warp_converged() && detail::warp_consecutive(dest)) {
            detail::contiguous_store<WARP_SIZE>(data, dest);
            return;
        }
    }
    detail::divergent_store(data, dest);
}

}  // namespace trove
