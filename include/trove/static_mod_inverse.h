// static_mod_inverse<a, m>::value — the r in [1, m) with (r * a) % m == 1,
// or -1 when a has no inverse modulo m.  Interface of the reference
// trove/static_mod_inverse.h:32-52; computed with a constexpr search.
#pragma once

#include <trove/detail/config.h>

namespace trove {

namespace detail {
TROVE_CX int mod_inverse_search(int a, int m) {
    for (int r = 1; r < m; ++r)
        if ((r * a) % m == 1) return r;
    return -1;
}
}  // namespace detail

template <int a, int m, int r = 1>
struct static_mod_inverse {
    static const int value = detail::mod_inverse_search(a, m);
};

}  // namespace trove
