// trove::rotate(t, a) — rotate an array left by a runtime amount:
// result[j] = t[(j + a) mod m], for 0 <= a < m.
// Interface and semantics of the reference trove/rotate.h:111-115.  Like the
// reference it decomposes a into its bits, one stage per power of two below
// m, so only the low ceil(log2 m) bits of a are looked at.
#pragma once

#include <trove/array.h>
#include <trove/detail/regs.h>

namespace trove {

template <typename T, int i>
TROVE_HD array<T, i> rotate(const array<T, i>& t, int a) {
    detail::regs<T, i> r = detail::to_regs(t);
    detail::rotate_regs(r, a);
    return detail::from_regs(r);
}

}  // namespace trove
