// High-level interface: coalesced_ptr<T> wraps a T* so that plain reads and
// writes through it (`T v = p[i]; q[j] = v;`) use trove::load / trove::store.
//
// Interface of the reference trove/ptr.h:34-90 (coalesced_ref,
// coalesced_ptr).  Assigning one reference to another (`q[j] = p[i]`) is a
// load followed by a store; the reference's version of that operator calls a
// dispatch overload that does not exist and so fails to compile when used.
#pragma once

#include <trove/aos.h>

namespace trove {
namespace detail {

template <typename T>
struct coalesced_ref {
    T* m_ptr;
    TROVE_D explicit coalesced_ref(T* ptr) : m_ptr(ptr) {}

    TROVE_D operator T() const { return trove::load(static_cast<const T*>(m_ptr)); }

    TROVE_D coalesced_ref& operator=(const T& data) {
        trove::store(data, m_ptr);
        return *this;
    }

    TROVE_D coalesced_ref& operator=(const coalesced_ref& other) {
        const T data = trove::load(static_cast<const T*>(other.m_ptr));
        trove::store(data, m_ptr);
        return *this;
    }
};

}  // namespace detail

template <typename T>
struct coalesced_ptr {
    T* m_ptr;
    TROVE_D coalesced_ptr(T* ptr) : m_ptr(ptr) {}
    TROVE_D detail::coalesced_ref<T> operator*() { return detail::coalesced_ref<T>(m_ptr); }
    template <typename I>
    TROVE_D detail::coalesced_ref<T> operator[](const I& idx) {
        return detail::coalesced_ref<T>(m_ptr + idx);
    }
    TROVE_D operator T*() { return m_ptr; }
};

}  // namespace trove
