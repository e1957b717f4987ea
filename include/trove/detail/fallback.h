// Per-lane ("divergent") struct loads and stores that need no other lane.
//
// Interface of the reference trove/detail/fallback.h:67-129
// (divergent_load, divergent_store).  The reference picks the word type from
// sizeof(T) alone and so assumes the pointer is aligned to that word; here the
// widest word is chosen from the pointer's actual alignment at run time
// (16, 8 or 4 bytes), which moves the same bytes with the fewest sectors-worth
// of instructions and never issues a misaligned vector access.  Sizes that
// are not a multiple of 4 bytes, and pointers below 4-byte alignment, are
// accessed as the struct itself (the compiler then honours alignof(T)).
#pragma once

#include <trove/detail/dismember.h>

namespace trove {
namespace detail {

template <typename T, typename U>
TROVE_D T load_words(const T* src) {
    constexpr int m = aliased_size<T, U>::value;
    const U* p = reinterpret_cast<const U*>(src);
    regs<U, m> r;
#pragma unroll
    for (int k = 0; k < m; ++k) r.v[k] = p[k];
    return fuse_regs<T>(r);
}

template <typename T, typename U>
TROVE_D void store_words(const T& data, T* dst) {
    constexpr int m = aliased_size<T, U>::value;
    U* p = reinterpret_cast<U*>(dst);
    const regs<U, m> r = lyse_regs<U>(data);
#pragma unroll
    for (int k = 0; k < m; ++k) p[k] = r.v[k];
}

template <typename T>
TROVE_D T divergent_load(const T* src) {
    if constexpr (sizeof(T) % 4 != 0) {
        return *src;
    } else {
        typedef typename dismember_type<T>::type Umax;
        const std::uintptr_t a = reinterpret_cast<std::uintptr_t>(src);
        if constexpr (sizeof(Umax) == 16) {
            if ((a & 15) == 0) return load_words<T, int4>(src);
        }
        if constexpr (sizeof(Umax) >= 8) {
            if ((a & 7) == 0) return load_words<T, int2>(src);
        }
        if constexpr (alignof(T) < 4) {
            if ((a & 3) != 0) return *src;
        }
        return load_words<T, int>(src);
    }
}

template <typename T>
TROVE_D void divergent_store(const T& data, T* dst) {
    if constexpr (sizeof(T) % 4 != 0) {
        *dst = data;
    } else {
        typedef typename dismember_type<T>::type Umax;
        const std::uintptr_t a = reinterpret_cast<std::uintptr_t>(dst);
        if constexpr (sizeof(Umax) == 16) {
            if ((a & 15) == 0) return store_words<T, int4>(data, dst);
        }
        if constexpr (sizeof(Umax) >= 8) {
            if ((a & 7) == 0) return store_words<T, int2>(data, dst);
        }
        if constexpr (alignof(T) < 4) {
            if ((a & 3) != 0) {
                *dst = data;
                return;
            }
        }
        store_words<T, int>(data, dst);
    }
}

}  // namespace detail
}  // namespace trove
