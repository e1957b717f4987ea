// A flat register block `regs<T, m>` and conversions to and from
// trove::array.  The transposition and memory code works on this flat form:
// every index into `v` is a compile-time constant after unrolling, so the
// block lives in registers.
#pragma once

#include <utility>

#include <trove/array.h>

namespace trove {
namespace detail {

template <typename T, int m>
struct regs {
    T v[m];
};

template <typename T, int m, std::size_t... I>
TROVE_HD regs<T, m> to_regs_impl(const array<T, m>& a, std::index_sequence<I...>) {
    return regs<T, m>{{get<static_cast<int>(I)>(a)...}};
}

template <typename T, int m>
TROVE_HD regs<T, m> to_regs(const array<T, m>& a) {
    return to_regs_impl(a, std::make_index_sequence<m>());
}

template <typename T, int m, std::size_t... I>
TROVE_HD array<T, m> from_regs_impl(const regs<T, m>& r, std::index_sequence<I...>) {
    return make_array<T>(r.v[I]...);
}

template <typename T, int m>
TROVE_HD array<T, m> from_regs(const regs<T, m>& r) {
    return from_regs_impl(r, std::make_index_sequence<m>());
}

// In-place left rotation by a runtime amount: v'[j] = v[(j + a) mod m] for
// 0 <= a < m.  A barrel shifter: one stage of m selects per bit of a, no
// dynamic register indexing (which would spill to local memory).
template <typename T, int m>
TROVE_HD void rotate_regs(regs<T, m>& r, int a) {
#pragma unroll
    for (int b = 1; b < m; b <<= 1) {
        const bool take = (a & b) != 0;
        regs<T, m> t = r;
#pragma unroll
        for (int j = 0; j < m; ++j) r.v[j] = take ? t.v[(j + b) % m] : t.v[j];
    }
}

}  // namespace detail
}  // namespace trove
