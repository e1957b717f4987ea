// trove::array<T, m> — a fixed-length value array indexed at compile time.
//
// Device API type of the AoS library.  Keeps the interface of the reference
// (trove/array.h:32-200): the recursive `head`/`tail` members, `size`,
// `value_type`, `get<i>`, `make_array` (variadic and from a C array) and
// `make_carray`, so kernels written against that interface recompile
// unchanged.  The layout is head-first, so an `array<T, m>` occupies exactly
// m consecutive T in memory (this is what lets the block interface cast a
// `T*` to `array<T, s>*`).  Copy construction and assignment are the
// compiler's, which keeps the type trivially copyable.
#pragma once

#include <trove/detail/config.h>

namespace trove {

template <typename T, int m>
struct array {
    typedef T value_type;
    typedef T head_type;
    typedef array<T, m - 1> tail_type;
    static const int size = m;

    head_type head;
    tail_type tail;

    TROVE_HD array() : head(), tail() {}
    TROVE_HD array(head_type h, const tail_type& t) : head(h), tail(t) {}
    array(const array&) = default;
    array& operator=(const array&) = default;

    TROVE_HD bool operator==(const array& o) const {
        return head == o.head && tail == o.tail;
    }
    TROVE_HD bool operator!=(const array& o) const { return !(*this == o); }
};

template <typename T>
struct array<T, 1> {
    typedef T value_type;
    typedef T head_type;
    static const int size = 1;

    head_type head;

    TROVE_HD array() : head() {}
    TROVE_HD array(head_type h) : head(h) {}
    array(const array&) = default;
    array& operator=(const array&) = default;

    TROVE_HD bool operator==(const array& o) const { return head == o.head; }
    TROVE_HD bool operator!=(const array& o) const { return !(*this == o); }
};

template <typename T>
struct array<T, 0> {};

namespace detail {

// Walks i links down the tail chain.
template <int i>
struct array_at {
    template <typename T, int m>
    TROVE_HD static T& ref(array<T, m>& a) { return array_at<i - 1>::ref(a.tail); }
    template <typename T, int m>
    TROVE_HD static T val(const array<T, m>& a) { return array_at<i - 1>::val(a.tail); }
};

template <>
struct array_at<0> {
    template <typename T, int m>
    TROVE_HD static T& ref(array<T, m>& a) { return a.head; }
    template <typename T, int m>
    TROVE_HD static T val(const array<T, m>& a) { return a.head; }
};

}  // namespace detail

template <int i, typename T, int m>
TROVE_HD T& get(array<T, m>& a) {
    static_assert(i >= 0 && i < m, "trove::get index out of range");
    return detail::array_at<i>::ref(a);
}

template <int i, typename T, int m>
TROVE_HD T get(const array<T, m>& a) {
    static_assert(i >= 0 && i < m, "trove::get index out of range");
    return detail::array_at<i>::val(a);
}

template <typename T>
TROVE_HD array<T, 0> make_array() {
    return array<T, 0>();
}

template <typename T>
TROVE_HD array<T, 1> make_array(T a0) {
    return array<T, 1>(a0);
}

template <typename T, typename... Rest>
TROVE_HD array<T, 1 + sizeof...(Rest)> make_array(T a0, Rest... rest) {
    return array<T, 1 + sizeof...(Rest)>(a0, make_array<T>(static_cast<T>(rest)...));
}

namespace detail {

template <typename T, int s>
struct from_c_array {
    TROVE_HD static array<T, s> build(const T* c) {
        return array<T, s>(c[0], from_c_array<T, s - 1>::build(c + 1));
    }
    TROVE_HD static void spill(const array<T, s>& a, T* c) {
        c[0] = a.head;
        from_c_array<T, s - 1>::spill(a.tail, c + 1);
    }
};

template <typename T>
struct from_c_array<T, 1> {
    TROVE_HD static array<T, 1> build(const T* c) { return array<T, 1>(c[0]); }
    TROVE_HD static void spill(const array<T, 1>& a, T* c) { c[0] = a.head; }
};

}  // namespace detail

// Builds an array from the first s elements of a C array.
template <typename T, int s>
TROVE_HD array<T, s> make_array(T cary[s]) {
    return detail::from_c_array<T, s>::build(cary);
}

// Writes the s elements of an array into a C array.
template <typename T, int s>
TROVE_HD void make_carray(const array<T, s>& ary, T result[s]) {
    detail::from_c_array<T, s>::spill(ary, result);
}

}  // namespace trove
