// static_gcd<u, v>::value — greatest common divisor at compile time.
// Interface of the reference trove/static_gcd.h:59-75 (`::value`); computed
// here with a constexpr Euclid loop.  gcd(0, v) == v.
#pragma once

#include <trove/detail/config.h>

namespace trove {

namespace detail {
TROVE_CX int euclid_gcd(int u, int v) {
    while (v != 0) {
        int r = u % v;
        u = v;
        v = r;
    }
    return u < 0 ? -u : u;
}
}  // namespace detail

template <int u, int v>
struct static_gcd {
    static const int value = detail::euclid_gcd(u, v);
};

}  // namespace trove
