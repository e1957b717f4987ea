// Warp tiles and convergence tests.
//
// Interface of the reference trove/warp.h:34-93: WARP_SIZE, WARP_CONVERGED,
// log2, thread_tile<N> (shfl, size, log_size, mask, id) and
// warp_converged<N>().  thread_tile is written directly on the sm_103a warp
// intrinsics: a tile of N lanes is the aligned group of N lanes that holds the
// caller, and its shuffles name exactly those lanes in their member mask, so a
// tile may run while the rest of the warp is elsewhere.
#pragma once

#include <trove/detail/config.h>

namespace trove {

enum { WARP_SIZE = 32, WARP_CONVERGED = 0xFFFFFFFF };

TROVE_CX std::size_t log2(std::size_t n) { return n < 2 ? 0 : 1 + log2(n / 2); }

namespace detail {

// Member mask of the aligned group of n lanes that contains the caller.
template <std::size_t n>
TROVE_D unsigned group_mask() {
    if constexpr (n >= 32) {
        return 0xFFFFFFFFu;
    } else {
        const unsigned lane = lane_id();
        return ((1u << n) - 1u) << (lane & ~unsigned(n - 1));
    }
}

// Shuffle of any trivially copyable value, 32 bits at a time.
template <typename T>
TROVE_D T shfl_any(const T& t, int src, unsigned mask, int width) {
    constexpr int nw = int((sizeof(T) + 3) / 4);
    unsigned w[nw];
    std::memcpy(w, &t, sizeof(T));
#pragma unroll
    for (int k = 0; k < nw; ++k) w[k] = __shfl_sync(mask, w[k], src, width);
    T r;
    std::memcpy(&r, w, sizeof(T));
    return r;
}

}  // namespace detail

template <std::size_t threads>
struct thread_tile {
    static_assert(threads >= 1 && threads <= 32 && (threads & (threads - 1)) == 0,
                  "a thread_tile is a power-of-two group of at most 32 lanes");

    TROVE_D thread_tile() {}

    template <typename T>
    TROVE_D T shfl(const T& t, const int& i) const {
        return detail::shfl_any(t, i, detail::group_mask<threads>(), int(threads));
    }

    TROVE_HD static constexpr int size() { return int(threads); }
    TROVE_HD static constexpr int log_size() { return int(log2(threads)); }
    TROVE_HD static constexpr int mask() { return int(threads) - 1; }
    TROVE_D int id() const { return int(detail::lane_id() & unsigned(threads - 1)); }
    TROVE_D unsigned member_mask() const { return detail::group_mask<threads>(); }
};

// True when every lane of the caller's aligned group of warp_size lanes is
// active (for warp_size == 32: the whole warp).
template <std::size_t warp_size = WARP_SIZE>
TROVE_D bool warp_converged() {
    const unsigned gm = detail::group_mask<warp_size>();
    return (__activemask() & gm) == gm;
}

}  // namespace trove
