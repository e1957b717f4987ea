// Function qualifiers and the lane-id primitive shared by every trove header.
//
// Under nvcc the API functions are `__device__` (and `__host__ __device__`
// where they touch no warp state).  Without nvcc the headers compile as plain
// C++ for the host lane emulator used by the CPU test suite; that build must
// define TROVE_LANE_EMULATION and provide the warp intrinsics itself.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define TROVE_HD __host__ __device__ __forceinline__
#define TROVE_D __device__ __forceinline__
#define TROVE_CX __host__ __device__ constexpr
#else
#define TROVE_HD inline
#define TROVE_D inline
#define TROVE_CX constexpr
#endif

#if !defined(__CUDACC__) && !defined(TROVE_LANE_EMULATION)
#error "trove device headers need nvcc, or TROVE_LANE_EMULATION with a lane emulator"
#endif

namespace trove {
namespace detail {

// Index of the calling thread within its hardware warp (0..31).
TROVE_D unsigned lane_id() {
#if defined(__CUDA_ARCH__)
    unsigned r;
    asm("mov.u32 %0, %%laneid;" : "=r"(r));
    return r;
#elif defined(TROVE_LANE_EMULATION)
    return trove_emu_lane_id();
#else
    return 0;  // host pass of nvcc: device-only code, never executed
#endif
}

}  // namespace detail
}  // namespace trove
