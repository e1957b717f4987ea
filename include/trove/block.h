// Block interface: each thread loads or stores an array<T, s> at index idx
// of an array of T viewed as consecutive s-element blocks.
//
// Interface of the reference trove/block.h:35-65.  The *_warp_contiguous
// forms need a converged tile whose lanes pass consecutive idx; load_array /
// store_array are the per-thread forms for any other case (a partial warp,
// scattered idx).  The per-thread forms here pick the widest word the
// address is aligned to instead of the compiler's alignof(T)-sized accesses.
#pragma once

#include <trove/aos.h>
#include <trove/warp.h>

namespace trove {

template <int s, std::size_t tile_size = WARP_SIZE, typename T, typename I>
TROVE_D array<T, s> load_array_warp_contiguous(const T* src, const I& idx) {
    return load_warp_contiguous<tile_size>(reinterpret_cast<const array<T, s>*>(src) + idx);
}

template <int s, typename T, typename I>
TROVE_D array<T, s> load_array(const T* src, const I& idx) {
    return detail::divergent_load(reinterpret_cast<const array<T, s>*>(src) + idx);
}

template <int s, std::size_t tile_size = WARP_SIZE, typename T, typename I>
TROVE_D void store_array_warp_contiguous(T* dest, const I& idx, const array<T, s>& src) {
    store_warp_contiguous<tile_size>(src, reinterpret_cast<array<T, s>*>(dest) + idx);
}

template <int s, typename T, typename I>
TROVE_D void store_array(T* dest, const I& idx, const array<T, s>& src) {
    detail::divergent_store(src, reinterpret_cast<array<T, s>*>(dest) + idx);
}

}  // namespace trove
