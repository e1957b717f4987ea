// Strided per-lane array loads and stores.
//
// Interface of the reference trove/memory.h:136-168:
//  - warp_load<Array>(p, offset, stride)[k] == p[offset + k * stride];
//  - warp_store(a, p, offset, stride) writes p[offset + k * stride] = a[k];
//  - uncoalesced_store(a, p, stride) writes p[k] = a[k].  As in the
//    reference, the stride argument is accepted and not used.
// With offset = lane and stride = tile size every round is one coalesced
// access of the whole tile.
#pragma once

#include <trove/array.h>
#include <trove/detail/regs.h>

namespace trove {

template <typename Array>
TROVE_HD void warp_store(const Array& t, typename Array::head_type* ptr, int offset, int stride) {
    typedef typename Array::head_type U;
    const detail::regs<U, Array::size> r = detail::to_regs(t);
#pragma unroll
    for (int k = 0; k < Array::size; ++k) ptr[offset + k * stride] = r.v[k];
}

template <typename Array>
TROVE_HD Array warp_load(const typename Array::head_type* ptr, int offset, int stride) {
    typedef typename Array::head_type U;
    detail::regs<U, Array::size> r;
#pragma unroll
    for (int k = 0; k < Array::size; ++k) r.v[k] = ptr[offset + k * stride];
    return detail::from_regs(r);
}

template <typename Array>
TROVE_HD Array warp_load(const volatile typename Array::head_type* ptr, int offset, int stride) {
    typedef typename Array::head_type U;
    detail::regs<U, Array::size> r;
#pragma unroll
    for (int k = 0; k < Array::size; ++k) r.v[k] = ptr[offset + k * stride];
    return detail::from_regs(r);
}

template <typename Array>
TROVE_HD void uncoalesced_store(const Array& t, typename Array::head_type* ptr, int stride = 1) {
    (void)stride;
    typedef typename Array::head_type U;
    const detail::regs<U, Array::size> r = detail::to_regs(t);
#pragma unroll
    for (int k = 0; k < Array::size; ++k) ptr[k] = r.v[k];
}

template <typename Array>
TROVE_HD void uncoalesced_store(const Array& t, volatile typename Array::head_type* ptr,
                                int stride = 1) {
    (void)stride;
    typedef typename Array::head_type U;
    const detail::regs<U, Array::size> r = detail::to_regs(t);
#pragma unroll
    for (int k = 0; k < Array::size; ++k) ptr[k] = r.v[k];
}

}  // namespace trove
