// Instantiates every struct-typed kernel for one width, TRV_WIDTH words
// (compiled once per width so the build parallelises across widths).
#include "kernels.cuh"
#include "ops.h"

#ifndef TRV_WIDTH
#error "compile with -DTRV_WIDTH=<words per struct>"
#endif

namespace trv {
namespace {

constexpr int S = TRV_WIDTH;

template <int U, int API, bool EXIT, bool LOOP>
void launch_copy(const CopyArgs& a, int grid, int block, cudaStream_t st) {
    copy_kernel<S, U, API, EXIT, LOOP><<<grid, block, 0, st>>>(static_cast<const aos<S>*>(a.src),
                                                               static_cast<aos<S>*>(a.dst), a.n, a.modulus);
}

template <int U, int MODE>
void launch_gather(const IndexArgs& a, int grid, int block, cudaStream_t st) {
    gather_kernel<S, U, MODE><<<grid, block, 0, st>>>(static_cast<const aos<S>*>(a.src), a.bound, a.idx,
                                                      static_cast<aos<S>*>(a.dst), a.n);
}

template <int U, int MODE>
void launch_scatter(const IndexArgs& a, int grid, int block, cudaStream_t st) {
    scatter_kernel<S, U, MODE><<<grid, block, 0, st>>>(static_cast<const aos<S>*>(a.src), a.idx,
                                                       static_cast<aos<S>*>(a.dst), a.bound, a.n);
}

// Unroll actually built for table slot k (1, 2, 4, 8): a lane keeps at most
// 32 words of payload in flight, so wide structs reuse the largest fitting
// unroll in the upper slots (bounded registers and build time).
constexpr int unroll_for(int k) {
    int u = 1 << k;
    while (u > 1 && u * S > 32) u >>= 1;
    return u;
}

template <int API, bool EXIT, bool LOOP, int k>
CopyKernel copy_entry() {
    constexpr int U = unroll_for(k);
    return {&launch_copy<U, API, EXIT, LOOP>, (const void*)&copy_kernel<S, U, API, EXIT, LOOP>};
}

// Widest word dividing the struct: 16, 8 or 4 bytes.
constexpr int kWideWord = (S % 4 == 0) ? 16 : (S % 2 == 0) ? 8 : 4;
template <int B>
struct word_of;
template <>
struct word_of<16> {
    typedef uint4 type;
};
template <>
struct word_of<8> {
    typedef uint2 type;
};
template <>
struct word_of<4> {
    typedef unsigned type;
};

template <typename V, int U>
void launch_gather_rows(const IndexArgs& a, int grid, int block, cudaStream_t st) {
    gather_rows_kernel<S, V, U><<<grid, block, 0, st>>>(static_cast<const V*>(a.src), a.bound, a.idx,
                                                        static_cast<V*>(a.dst), a.n, a.policy);
}

template <typename V, int U>
void launch_scatter_rows(const IndexArgs& a, int grid, int block, cudaStream_t st) {
    scatter_rows_kernel<S, V, U><<<grid, block, 0, st>>>(static_cast<const V*>(a.src), a.idx,
                                                         static_cast<V*>(a.dst), a.lo, a.bound, a.n, a.policy);
}

template <typename V, int k>
void rows_entries(IndexKernel& g, IndexKernel& s) {
    constexpr int U = unroll_for(k);
    g = {&launch_gather_rows<V, U>, (const void*)&gather_rows_kernel<S, V, U>};
    s = {&launch_scatter_rows<V, U>, (const void*)&scatter_rows_kernel<S, V, U>};
}

template <typename V>
void fill_rows(IndexKernel (&g)[kUnrolls], IndexKernel (&s)[kUnrolls]) {
    rows_entries<V, 0>(g[0], s[0]);
    rows_entries<V, 1>(g[1], s[1]);
    rows_entries<V, 2>(g[2], s[2]);
    rows_entries<V, 3>(g[3], s[3]);
}

template <int U, bool LOOP>
void launch_aos_to_soa(const CopyArgs& a, int grid, int block, cudaStream_t st) {
    aos_to_soa_kernel<S, U, LOOP><<<grid, block, 0, st>>>(static_cast<const aos<S>*>(a.src),
                                                          static_cast<unsigned*>(a.dst), a.n);
}

template <int U, bool LOOP>
void launch_soa_to_aos(const CopyArgs& a, int grid, int block, cudaStream_t st) {
    soa_to_aos_kernel<S, U, LOOP><<<grid, block, 0, st>>>(static_cast<const unsigned*>(a.src),
                                                          static_cast<aos<S>*>(a.dst), a.n);
}

template <int k, bool LOOP>
void layout_entries(CopyKernel& to_soa, CopyKernel& to_aos) {
    constexpr int U = unroll_for(k);
    to_soa = {&launch_aos_to_soa<U, LOOP>, (const void*)&aos_to_soa_kernel<S, U, LOOP>};
    to_aos = {&launch_soa_to_aos<U, LOOP>, (const void*)&soa_to_aos_kernel<S, U, LOOP>};
}

template <int API, bool EXIT, bool LOOP>
void fill_copy(CopyKernel (&row)[kUnrolls]) {
    row[0] = copy_entry<API, EXIT, LOOP, 0>();
    row[1] = copy_entry<API, EXIT, LOOP, 1>();
    row[2] = copy_entry<API, EXIT, LOOP, 2>();
    row[3] = copy_entry<API, EXIT, LOOP, 3>();
}

template <int MODE, int k>
IndexKernel gather_entry() {
    constexpr int U = unroll_for(k);
    return {&launch_gather<U, MODE>, (const void*)&gather_kernel<S, U, MODE>};
}

template <int MODE, int k>
IndexKernel scatter_entry() {
    constexpr int U = unroll_for(k);
    return {&launch_scatter<U, MODE>, (const void*)&scatter_kernel<S, U, MODE>};
}

template <int MODE>
void fill_index(IndexKernel (&g)[kUnrolls], IndexKernel (&s)[kUnrolls]) {
    g[0] = gather_entry<MODE, 0>();
    g[1] = gather_entry<MODE, 1>();
    g[2] = gather_entry<MODE, 2>();
    g[3] = gather_entry<MODE, 3>();
    s[0] = scatter_entry<MODE, 0>();
    s[1] = scatter_entry<MODE, 1>();
    s[2] = scatter_entry<MODE, 2>();
    s[3] = scatter_entry<MODE, 3>();
}

WidthOps make_ops() {
    WidthOps ops;
    fill_copy<API_WARP, false, false>(ops.copy[API_WARP]);
    fill_copy<API_BLOCK, false, false>(ops.copy[API_BLOCK]);
    fill_copy<API_DIRECT, false, false>(ops.copy[API_DIRECT]);
    fill_copy<API_WARP, true, false>(ops.copy_exit[API_WARP]);
    fill_copy<API_BLOCK, true, false>(ops.copy_exit[API_BLOCK]);
    fill_copy<API_WARP, false, true>(ops.copy_grid[API_WARP]);
    fill_copy<API_BLOCK, false, true>(ops.copy_grid[API_BLOCK]);
    fill_copy<API_DIRECT, false, true>(ops.copy_grid[API_DIRECT]);
    fill_copy<API_WARP, true, true>(ops.copy_exit_grid[API_WARP]);
    fill_copy<API_BLOCK, true, true>(ops.copy_exit_grid[API_BLOCK]);
    fill_index<MODE_COALESCED>(ops.gather[MODE_COALESCED], ops.scatter[MODE_COALESCED]);
    fill_index<MODE_DIRECT>(ops.gather[MODE_DIRECT], ops.scatter[MODE_DIRECT]);
    fill_rows<typename word_of<kWideWord>::type>(ops.gather_rows[0], ops.scatter_rows[0]);
    fill_rows<unsigned>(ops.gather_rows[1], ops.scatter_rows[1]);
    ops.rows_word_bytes = kWideWord;
    for (int k = 0; k < kUnrolls; ++k) ops.built_unroll[k] = unroll_for(k);
    layout_entries<0, false>(ops.aos_to_soa[0], ops.soa_to_aos[0]);
    layout_entries<1, false>(ops.aos_to_soa[1], ops.soa_to_aos[1]);
    layout_entries<2, false>(ops.aos_to_soa[2], ops.soa_to_aos[2]);
    layout_entries<3, false>(ops.aos_to_soa[3], ops.soa_to_aos[3]);
    layout_entries<0, true>(ops.aos_to_soa_grid[0], ops.soa_to_aos_grid[0]);
    layout_entries<1, true>(ops.aos_to_soa_grid[1], ops.soa_to_aos_grid[1]);
    layout_entries<2, true>(ops.aos_to_soa_grid[2], ops.soa_to_aos_grid[2]);
    layout_entries<3, true>(ops.aos_to_soa_grid[3], ops.soa_to_aos_grid[3]);
    return ops;
}

}  // namespace

template <>
const WidthOps& width_ops<S>() {
    static const WidthOps ops = make_ops();
    return ops;
}

}  // namespace trv
