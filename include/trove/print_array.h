// operator<< for trove::array (host-side debugging): elements separated by
// single spaces.  Interface of the reference trove/print_array.h:34-45.
#pragma once

#include <iostream>

#include <trove/array.h>

namespace trove {

template <typename T>
std::ostream& operator<<(std::ostream& strm, const array<T, 1>& ary) {
    return strm << ary.head;
}

template <typename T, int s>
std::ostream& operator<<(std::ostream& strm, const array<T, s>& ary) {
    strm << ary.head << " ";
    return strm << ary.tail;
}

}  // namespace trove
