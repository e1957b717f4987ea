// Compile-time helpers of the device API.
//
// Same names and members as the reference (trove/utility.h:33-159):
// counting_array, sum, static_log, is_power_of_two, is_odd, value_if,
// value_identity, inverse, null_type, cons_c, static_range, enable_if and
// size_multiple_power_of_two.  Test kernels and the width-sweep drivers use
// counting_array, sum, static_range and null_type directly.
#pragma once

#include <trove/array.h>

namespace trove {

// counting_array<array<T, s>>::impl(v, i) == {v, v+i, v+2i, ...}.
template <typename Array>
struct counting_array {};

template <typename T, int s>
struct counting_array<array<T, s> > {
    TROVE_HD static array<T, s> impl(T v = 0, T i = 1) {
        return array<T, s>(v, counting_array<array<T, s - 1> >::impl(v + i, i));
    }
};

template <typename T>
struct counting_array<array<T, 1> > {
    TROVE_HD static array<T, 1> impl(T v = 0, T i = 1) {
        (void)i;
        return array<T, 1>(v);
    }
};

namespace detail {
template <typename T, int s>
struct array_sum {
    TROVE_HD static T add(const array<T, s>& a, T acc) {
        return array_sum<T, s - 1>::add(a.tail, acc + a.head);
    }
};
template <typename T>
struct array_sum<T, 1> {
    TROVE_HD static T add(const array<T, 1>& a, T acc) { return acc + a.head; }
};
}  // namespace detail

// Left-to-right sum of the elements, starting from 0.
template <typename T, int s>
TROVE_HD T sum(const array<T, s>& a) {
    return detail::array_sum<T, s>::add(a, T(0));
}

namespace detail {
TROVE_CX int floor_log2(int m) { return m <= 1 ? 0 : 1 + floor_log2(m >> 1); }
}  // namespace detail

// floor(log2(m)); taking the log of 0 is a compile error.
template <int m>
struct static_log {
    static_assert(m > 0, "static_log of 0");
    static const int value = detail::floor_log2(m);
};

template <int m>
struct is_power_of_two {
    static const bool value = (m & (m - 1)) == 0;
};

template <int m>
struct is_odd {
    static const bool value = (m & 1) == 1;
};

template <bool cond, typename T, typename Then, typename Else>
struct value_if {
    static const T value = Then::value;
};

template <typename T, typename Then, typename Else>
struct value_if<false, T, Then, Else> {
    static const T value = Else::value;
};

template <typename T, T x>
struct value_identity {
    static const T value = x;
};

// Smallest p >= start with Fn<p>::value == x (linear search at compile time).
template <typename T, template <T> class Fn, T x, T p = 0>
struct inverse {
    static const T value =
        value_if<Fn<p>::value == x, T, value_identity<T, p>, inverse<T, Fn, x, p + 1> >::value;
};

struct null_type {};

template <typename T, T i, typename Tail = null_type>
struct cons_c {
    static const T head = i;
    typedef Tail tail;
};

// Type list k, k+1, ..., l (inclusive), terminated by null_type.
template <int k, int l>
struct static_range {
    static const int head = k;
    typedef static_range<k + 1, l> tail;
};

template <int f>
struct static_range<f, f> {
    static const int head = f;
    typedef null_type tail;
};

template <bool b, typename T = void>
struct enable_if {
    typedef T type;
};

template <typename T>
struct enable_if<false, T> {};

// True when sizeof(T) is a multiple of 2^p.
template <typename T, int p>
struct size_multiple_power_of_two {
    static const bool value = (sizeof(T) & ((std::size_t(1) << p) - 1)) == 0;
};

}  // namespace trove
