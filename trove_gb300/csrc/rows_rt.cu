// Instantiations of the run-time-width row-form gather / scatter kernels.
#include "kernels.cuh"
#include "ops.h"

namespace trv {

namespace {
template <typename V, int G, bool GATHER>
void launch_rt(const IndexArgs& a, int m, int grid, cudaStream_t st) {
    index_rows_rt_kernel<V, G, GATHER><<<grid, 256, 0, st>>>(static_cast<const V*>(a.src), a.idx,
                                                            static_cast<V*>(a.dst), a.bound, a.n, m, a.policy);
}
}  // namespace

void launch_index_rows_rt(bool gather, int word_bytes, const IndexArgs& a, int m, int grid, cudaStream_t st) {
    if (word_bytes == 16)
        gather ? launch_rt<uint4, 2, true>(a, m, grid, st) : launch_rt<uint4, 2, false>(a, m, grid, st);
    else if (word_bytes == 8)
        gather ? launch_rt<uint2, 4, true>(a, m, grid, st) : launch_rt<uint2, 4, false>(a, m, grid, st);
    else
        gather ? launch_rt<unsigned, 4, true>(a, m, grid, st) : launch_rt<unsigned, 4, false>(a, m, grid, st);
}

const void* index_rows_rt_func(bool gather, int word_bytes) {
    if (word_bytes == 16)
        return gather ? (const void*)&index_rows_rt_kernel<uint4, 2, true> : (const void*)&index_rows_rt_kernel<uint4, 2, false>;
    if (word_bytes == 8)
        return gather ? (const void*)&index_rows_rt_kernel<uint2, 4, true> : (const void*)&index_rows_rt_kernel<uint2, 4, false>;
    return gather ? (const void*)&index_rows_rt_kernel<unsigned, 4, true>
                  : (const void*)&index_rows_rt_kernel<unsigned, 4, false>;
}

}  // namespace trv
