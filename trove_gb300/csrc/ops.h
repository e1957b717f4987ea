// Per-width kernel tables.  width_ops.cu is compiled once per struct width
// S = 1..16 words (-DTRV_WIDTH=S) and fills one WidthOps; the C ABI looks the
// table up by width and picks an entry by path and unroll.
#pragma once

#include <cuda_runtime.h>

namespace trv {

// Unroll factors offered (structs per lane per pass); index = log2(unroll).
constexpr int kUnrolls = 4;  // 1, 2, 4, 8

struct CopyArgs {
    const void* src;
    void* dst;
    long long n;
    unsigned modulus;
};

struct IndexArgs {
    const void* src;
    void* dst;
    const int* idx;
    long long n;
    long long bound;  // src_n for gather, dst_n for scatter
    int policy;       // cache policy of the row-form kernels
    long long lo = 0; // row-form scatter: only destinations in [lo, bound) are written
};

template <typename Args>
struct Kernel {
    void (*launch)(const Args&, int grid, int block, cudaStream_t);
    const void* func;  // for occupancy queries
};

typedef Kernel<CopyArgs> CopyKernel;
typedef Kernel<IndexArgs> IndexKernel;

struct WidthOps {
    // One chunk of 32*unroll structs per warp, no loop: the default grid.
    CopyKernel copy[3][kUnrolls];       // [API_WARP, API_BLOCK, API_DIRECT][unroll]
    CopyKernel copy_exit[2][kUnrolls];  // [API_WARP, API_BLOCK][unroll]
    // Grid-stride forms of the same, for caller-chosen and persistent grids.
    CopyKernel copy_grid[3][kUnrolls];
    CopyKernel copy_exit_grid[2][kUnrolls];
    IndexKernel gather[2][kUnrolls];    // [MODE_COALESCED, MODE_DIRECT][unroll]
    IndexKernel scatter[2][kUnrolls];
    // Row-form kernels: [0] the widest word dividing the width, [1] 4-byte words.
    IndexKernel gather_rows[2][kUnrolls];
    IndexKernel scatter_rows[2][kUnrolls];
    int rows_word_bytes;  // size of the word used by slot [0]
    // Unroll actually built in each slot (wide structs cap it: a lane keeps
    // at most 32 words in flight); grids are sized from this, not from the
    // unroll the caller asked for.
    int built_unroll[kUnrolls];
    CopyKernel aos_to_soa[kUnrolls];  // one chunk per warp
    CopyKernel soa_to_aos[kUnrolls];
    CopyKernel aos_to_soa_grid[kUnrolls];  // grid-stride forms
    CopyKernel soa_to_aos_grid[kUnrolls];
};

// Row-form gather / scatter with a run-time word count (rows_rt.cu), for any
// width that is a multiple of 4 bytes.  word_bytes: 16, 8 or 4.
void launch_index_rows_rt(bool gather, int word_bytes, const IndexArgs& a, int m, int grid, cudaStream_t st);
const void* index_rows_rt_func(bool gather, int word_bytes);

// Defined in width_ops.cu, one specialisation per translation unit.
template <int S>
const WidthOps& width_ops();

template <> const WidthOps& width_ops<1>();
template <> const WidthOps& width_ops<2>();
template <> const WidthOps& width_ops<3>();
template <> const WidthOps& width_ops<4>();
template <> const WidthOps& width_ops<5>();
template <> const WidthOps& width_ops<6>();
template <> const WidthOps& width_ops<7>();
template <> const WidthOps& width_ops<8>();
template <> const WidthOps& width_ops<9>();
template <> const WidthOps& width_ops<10>();
template <> const WidthOps& width_ops<11>();
template <> const WidthOps& width_ops<12>();
template <> const WidthOps& width_ops<13>();
template <> const WidthOps& width_ops<14>();
template <> const WidthOps& width_ops<15>();
template <> const WidthOps& width_ops<16>();

// Table for S words per struct (1..16), or nullptr.
inline const WidthOps* ops_for_words(int S) {
    switch (S) {
        case 1: return &width_ops<1>();
        case 2: return &width_ops<2>();
        case 3: return &width_ops<3>();
        case 4: return &width_ops<4>();
        case 5: return &width_ops<5>();
        case 6: return &width_ops<6>();
        case 7: return &width_ops<7>();
        case 8: return &width_ops<8>();
        case 9: return &width_ops<9>();
        case 10: return &width_ops<10>();
        case 11: return &width_ops<11>();
        case 12: return &width_ops<12>();
        case 13: return &width_ops<13>();
        case 14: return &width_ops<14>();
        case 15: return &width_ops<15>();
        case 16: return &width_ops<16>();
    }
    return nullptr;
}

}  // namespace trv
