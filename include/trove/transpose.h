// Register-only warp transposition between "rows" and "columns".
//
// A tile of n lanes holds an n x m block of words W[0 .. n*m).
//  - Row form (what m coalesced rounds of loads produce): lane L, register k
//    holds W[k*n + L].
//  - Column form (one struct per lane): lane l, register j holds W[l*m + j].
// r2c_warp_transpose turns row form into column form; c2r_warp_transpose is
// its inverse.  These are the semantics of the reference entry points
// trove/transpose.h:638-696, which implement the register-level C2R/R2C
// decomposition of Catanzaro, Keller and Garland, "A Decomposition for
// In-place Matrix Transposition" (PPoPP 2014).
//
// Schedule used here (one derivation for every m <= n, n a power of two).
// Let g = gcd(m, n), n' = n/g, a_l = l / n' and gamma_L = (-L) mod m.
//  R2C: in shuffle step s (0 <= s < m) lane l reads lane
//       src_s(l) = (l*m + (s + a_l) mod m) mod n and receives the word for its
//       column slot (s + a_l) mod m.  For fixed s this is a bijection of lanes.
//       Lane L must then publish its register pi((s + gamma_L) mod m), where
//       pi is a permutation fixed at compile time.  So a lane
//         1. renames registers by pi              (free: static),
//         2. rotates left by gamma_L              (barrel shifter),
//         3. does m shuffles,
//         4. rotates left by (m - a_l) mod m      (only when g > 1).
//  C2R runs the same schedule backwards: rotate by a_l, m shuffles from the
//       inverse lanes, rotate by L mod m, rename by pi^-1.
// For odd m (g == 1) a_l == 0 and one rotation per direction remains; the
// shuffle sources reduce to (l*m + s) mod n and ((L - s) * m^-1) mod n.
#pragma once

#include <utility>

#include <trove/array.h>
#include <trove/detail/regs.h>
#include <trove/static_gcd.h>
#include <trove/static_mod_inverse.h>
#include <trove/utility.h>
#include <trove/warp.h>

namespace trove {
namespace detail {

template <int n, int m>
struct tx_shape {
    static_assert(n >= 1 && (n & (n - 1)) == 0, "tile size must be a power of two");
    static_assert(m >= 1 && m <= n, "transposition needs 1 <= m <= tile size");
    static constexpr int g = euclid_gcd(n, m);
    static constexpr int ng = n / g;
    static constexpr int mg = m / g;
    static constexpr int log_g = floor_log2(g);
    static constexpr int log_ng = floor_log2(ng);
    // n'^-1 mod m' (m' is odd or 1) and, for odd m, m^-1 mod n.
    static constexpr int ng_inv = mg > 1 ? mod_inverse_search(ng % mg, mg) : 0;
    static constexpr int m_inv = (g == 1 && n > 1) ? mod_inverse_search(m % n, n) : 1;

    // Register published by lane 0 in R2C step x.
    TROVE_CX static int pi(int x) {
        for (int l = 0; l < n; ++l) {
            const int j = (x + l / ng) % m;
            const int w = l * m + j;
            if (w % n == 0) return w / n;
        }
        return -1;
    }
    TROVE_CX static int pi_inv(int k) {
        for (int x = 0; x < m; ++x)
            if (pi(x) == k) return x;
        return -1;
    }

    // R2C: lane this step's word comes from (receiver l, step s).
    TROVE_HD static int r2c_source(int l, int s) {
        int j = s + (l >> log_ng);
        if (j >= m) j -= m;
        return (l * m + j) & (n - 1);
    }

    // C2R: lane that sends to receiver L in step s (inverse of r2c_source).
    TROVE_HD static int c2r_source(int L, int s) {
        if (g == 1) return ((L - s) * m_inv) & (n - 1);
        const int t = (L - s) & (g - 1);
        if (g == m) return (t << log_ng) + (L >> log_g);
        int j = s + t;
        if (j >= m) j -= m;
        const int e = (j - L) >> log_g;  // exact: j == L (mod g)
        const int v = ((e + mg * ng) * ng_inv) % mg;
        const int u = L + n * v;
        return (t << log_ng) + (u - j) / m;
    }

    TROVE_HD static int sender_rotation(int L) { return (m - L % m) % m; }
    TROVE_HD static int lane_offset(int l) { return l >> log_ng; }
};

template <typename T, int m, int n, std::size_t... X>
TROVE_HD regs<T, m> rename_by_pi(const regs<T, m>& r, std::index_sequence<X...>) {
    return regs<T, m>{{r.v[std::integral_constant<int, tx_shape<n, m>::pi(int(X))>::value]...}};
}

template <typename T, int m, int n, std::size_t... X>
TROVE_HD regs<T, m> rename_by_pi_inv(const regs<T, m>& r, std::index_sequence<X...>) {
    return regs<T, m>{{r.v[std::integral_constant<int, tx_shape<n, m>::pi_inv(int(X))>::value]...}};
}

// Row form -> column form.  `src_lane[s]` and `rot` are the values that
// r2c_compute_indices produces for this lane.
template <typename Tile, typename T, int m>
TROVE_D void r2c_regs(regs<T, m>& r, const int (&src_lane)[m], int rot, const Tile& tile) {
    if constexpr (m > 1) {
        typedef tx_shape<Tile::size(), m> S;
        regs<T, m> p = rename_by_pi<T, m, Tile::size()>(r, std::make_index_sequence<m>());
        rotate_regs(p, rot);
#pragma unroll
        for (int s = 0; s < m; ++s) r.v[s] = tile.shfl(p.v[s], src_lane[s]);
        if constexpr (S::g > 1) {
            const int a = S::lane_offset(tile.id());
            rotate_regs(r, a == 0 ? 0 : m - a);
        }
    }
}

// Column form -> row form.  `src_lane[s]` and `rot` come from
// c2r_compute_indices.
template <typename Tile, typename T, int m>
TROVE_D void c2r_regs(regs<T, m>& r, const int (&src_lane)[m], int rot, const Tile& tile) {
    if constexpr (m > 1) {
        typedef tx_shape<Tile::size(), m> S;
        if constexpr (S::g > 1) rotate_regs(r, S::lane_offset(tile.id()));
        regs<T, m> x;
#pragma unroll
        for (int s = 0; s < m; ++s) x.v[s] = tile.shfl(r.v[s], src_lane[s]);
        rotate_regs(x, rot);
        r = rename_by_pi_inv<T, m, Tile::size()>(x, std::make_index_sequence<m>());
    }
}

template <typename Tile, int m>
TROVE_D void r2c_schedule(int (&src_lane)[m], int& rot, const Tile& tile) {
    typedef tx_shape<Tile::size(), m> S;
    const int l = tile.id();
#pragma unroll
    for (int s = 0; s < m; ++s) src_lane[s] = S::r2c_source(l, s);
    rot = S::sender_rotation(l);
}

template <typename Tile, int m>
TROVE_D void c2r_schedule(int (&src_lane)[m], int& rot, const Tile& tile) {
    typedef tx_shape<Tile::size(), m> S;
    const int L = tile.id();
#pragma unroll
    for (int s = 0; s < m; ++s) src_lane[s] = S::c2r_source(L, s);
    rot = L % m;
}

// Whole transposes of a register block, schedule computed in place.
template <typename Tile, typename T, int m>
TROVE_D void r2c_block(regs<T, m>& r, const Tile& tile) {
    int src_lane[m];
    int rot;
    r2c_schedule<Tile, m>(src_lane, rot, tile);
    r2c_regs(r, src_lane, rot, tile);
}

template <typename Tile, typename T, int m>
TROVE_D void c2r_block(regs<T, m>& r, const Tile& tile) {
    int src_lane[m];
    int rot;
    c2r_schedule<Tile, m>(src_lane, rot, tile);
    c2r_regs(r, src_lane, rot, tile);
}

template <typename A, int i, std::size_t... I>
TROVE_HD void fill_indices(array<int, i>& out, const A& a, std::index_sequence<I...>) {
    out = make_array<int>(a[I]...);
}

}  // namespace detail

// Per-lane shuffle sources and rotation for a C2R transpose of i words.
template <typename Tile, int i>
TROVE_D void c2r_compute_indices(array<int, i>& indices, int& rotation, const Tile& tile) {
    int src_lane[i];
    detail::c2r_schedule<Tile, i>(src_lane, rotation, tile);
    detail::fill_indices(indices, src_lane, std::make_index_sequence<i>());
}

template <typename Tile, typename T, int i>
TROVE_D void c2r_warp_transpose(array<T, i>& src, const array<int, i>& indices, int rotation,
                                const Tile& tile) {
    detail::regs<int, i> idx = detail::to_regs(indices);
    detail::regs<T, i> r = detail::to_regs(src);
    detail::c2r_regs(r, idx.v, rotation, tile);
    src = detail::from_regs(r);
}

template <typename Tile, typename T, int i>
TROVE_D void c2r_warp_transpose(array<T, i>& src, const Tile& tile) {
    detail::regs<T, i> r = detail::to_regs(src);
    detail::c2r_block(r, tile);
    src = detail::from_regs(r);
}

// Per-lane shuffle sources and rotation for an R2C transpose of i words.
template <typename Tile, int i>
TROVE_D void r2c_compute_indices(array<int, i>& indices, int& rotation, const Tile& tile) {
    int src_lane[i];
    detail::r2c_schedule<Tile, i>(src_lane, rotation, tile);
    detail::fill_indices(indices, src_lane, std::make_index_sequence<i>());
}

template <typename Tile, typename T, int i>
TROVE_D void r2c_warp_transpose(array<T, i>& src, const array<int, i>& indices, int rotation,
                                const Tile& tile) {
    detail::regs<int, i> idx = detail::to_regs(indices);
    detail::regs<T, i> r = detail::to_regs(src);
    detail::r2c_regs(r, idx.v, rotation, tile);
    src = detail::from_regs(r);
}

template <typename Tile, typename T, int i>
TROVE_D void r2c_warp_transpose(array<T, i>& src, const Tile& tile) {
    detail::regs<T, i> r = detail::to_regs(src);
    detail::r2c_block(r, tile);
    src = detail::from_regs(r);
}

}  // namespace trove
