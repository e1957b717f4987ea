// Splitting a struct into machine words and back.
//
// Interface of the reference trove/detail/dismember.h:37-129:
//  - dismember_type<T>::type is the widest of int4 / int2 / int whose size
//    divides sizeof(T), or char when sizeof(T) is not a multiple of 4;
//  - aliased_size<T, U>::value == sizeof(T) / sizeof(U);
//  - lyse<U>(t) splits t into an array<U, m>, fuse<T>(a) puts it back.
// The split is a byte copy, so it is exact for any trivially copyable T.
// (The reference asserts divisibility with a thrust macro; this header uses
// static_assert and has no thrust dependency.)
#pragma once

#include <trove/array.h>
#include <trove/detail/regs.h>
#include <trove/utility.h>

namespace trove {
namespace detail {

template <typename T,
          bool by4 = size_multiple_power_of_two<T, 2>::value,
          bool by8 = size_multiple_power_of_two<T, 3>::value,
          bool by16 = size_multiple_power_of_two<T, 4>::value>
struct dismember_type {
    typedef char type;
};
template <typename T>
struct dismember_type<T, true, false, false> {
    typedef int type;
};
template <typename T>
struct dismember_type<T, true, true, false> {
    typedef int2 type;
};
template <typename T>
struct dismember_type<T, true, true, true> {
    typedef int4 type;
};

template <typename T, typename U>
struct aliased_size {
    static_assert(sizeof(T) % sizeof(U) == 0, "word type must divide the struct");
    static const int value = int(sizeof(T) / sizeof(U));
};

template <typename U, typename T>
TROVE_HD regs<U, aliased_size<T, U>::value> lyse_regs(const T& in) {
    regs<U, aliased_size<T, U>::value> r;
    std::memcpy(r.v, &in, sizeof(T));
    return r;
}

template <typename T, typename U, int m>
TROVE_HD T fuse_regs(const regs<U, m>& r) {
    static_assert(sizeof(U) * m == sizeof(T), "word block must match the struct");
    T out;
    std::memcpy(&out, r.v, sizeof(T));
    return out;
}

template <typename U, typename T>
TROVE_HD array<U, aliased_size<T, U>::value> lyse(const T& in) {
    return from_regs(lyse_regs<U>(in));
}

template <typename T, typename U>
TROVE_HD T fuse(const array<U, aliased_size<T, U>::value>& in) {
    return fuse_regs<T>(to_regs(in));
}

}  // namespace detail
}  // namespace trove
