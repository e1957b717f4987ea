// Host lane emulator — TEST INFRASTRUCTURE ONLY, never linked into the product.
//
// Runs warp-synchronous device code on the CPU: one std::thread per lane,
// 32 lanes per warp, and the warp intrinsics (__shfl_sync, __ballot_sync,
// __all_sync, __any_sync, __match_any_sync, __reduce_or_sync, __activemask,
// __syncwarp) built
// on per-member-mask barriers.  It lets the same harness source run against
// two header trees on a machine without a GPU:
//   * the reference's trove headers (compiled in place, with the
//     cooperative_groups / thrust shims beside this file), which yields golden
//     vectors produced by the reference's own code, and
//   * this repository's include/trove, which is then checked against them.
// Included first (-include) by every translation unit it serves.
#pragma once

#define TROVE_LANE_EMULATION 1

#include <string.h>

#include <barrier>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

// CUDA function qualifiers, for headers written for nvcc.
#define __host__
#define __device__
#define __global__
#define __forceinline__ inline

struct alignas(8) int2 {
    int x, y;
};
struct alignas(16) int4 {
    int x, y, z, w;
};
struct dim3 {
    unsigned x = 0, y = 0, z = 0;
};

namespace emu {

struct Warp {
    unsigned active = 0xFFFFFFFFu;
    alignas(16) unsigned char slot[32][64];
    std::mutex mu;
    std::map<unsigned, std::unique_ptr<std::barrier<>>> bars;

    std::barrier<>& bar(unsigned mask) {
        std::lock_guard<std::mutex> g(mu);
        auto it = bars.find(mask);
        if (it == bars.end())
            it = bars.emplace(mask, std::make_unique<std::barrier<>>(__builtin_popcount(mask))).first;
        return *it->second;
    }
};

inline thread_local int t_lane = 0;
inline thread_local Warp* t_warp = nullptr;

[[noreturn]] inline void fail(const char* what, unsigned mask, int lane) {
    std::fprintf(stderr, "lane emulator: %s (mask %08x, lane %d)\n", what, mask, lane);
    std::abort();
}

// Every member of `mask` deposits `bytes` of data; returns after all have.
// The caller reads other lanes' slots, then calls release().
inline std::barrier<>& deposit(unsigned mask, const void* data, std::size_t bytes) {
    if (!((mask >> t_lane) & 1u)) fail("calling lane not in member mask", mask, t_lane);
    if ((t_warp->active & mask) != mask) fail("member mask names an inactive lane", mask, t_lane);
    std::memcpy(t_warp->slot[t_lane], data, bytes);
    std::barrier<>& b = t_warp->bar(mask);
    b.arrive_and_wait();
    return b;
}

template <typename T>
T shfl(unsigned mask, T var, int src, int width) {
    static_assert(sizeof(T) <= 64, "shuffle payload too large");
    std::barrier<>& b = deposit(mask, &var, sizeof(T));
    const int lane = (t_lane & ~(width - 1)) | (src & (width - 1));
    if (!((mask >> lane) & 1u)) fail("shuffle source outside member mask", mask, t_lane);
    T r;
    std::memcpy(&r, t_warp->slot[lane], sizeof(T));
    b.arrive_and_wait();
    return r;
}

// Runs body(lane) on the lanes of `run_mask`, one thread per lane; __activemask
// returns run_mask throughout.
inline void run_warp(unsigned run_mask, const std::function<void(int)>& body) {
    static Warp warp;  // one emulated warp at a time
    warp.active = run_mask;
    std::thread th[32];
    for (int l = 0; l < 32; ++l) {
        if (!((run_mask >> l) & 1u)) continue;
        th[l] = std::thread([l, &body] {
            t_lane = l;
            t_warp = &warp;
            body(l);
        });
    }
    for (int l = 0; l < 32; ++l)
        if (th[l].joinable()) th[l].join();
}

}  // namespace emu

inline thread_local dim3 threadIdx;
inline thread_local dim3 blockIdx;
inline thread_local dim3 blockDim;
inline thread_local dim3 gridDim;

inline unsigned trove_emu_lane_id() { return unsigned(emu::t_lane); }
inline unsigned __activemask() { return emu::t_warp->active; }

template <typename T>
inline T __shfl_sync(unsigned mask, T var, int src, int width = 32) {
    return emu::shfl(mask, var, src, width);
}

inline unsigned __ballot_sync(unsigned mask, int pred) {
    const unsigned char p = pred ? 1 : 0;
    std::barrier<>& b = emu::deposit(mask, &p, 1);
    unsigned r = 0;
    for (int l = 0; l < 32; ++l)
        if (((mask >> l) & 1u) && emu::t_warp->slot[l][0]) r |= 1u << l;
    b.arrive_and_wait();
    return r;
}

inline unsigned __reduce_or_sync(unsigned mask, unsigned value) {
    std::barrier<>& b = emu::deposit(mask, &value, sizeof(value));
    unsigned r = 0;
    for (int l = 0; l < 32; ++l) {
        if (!((mask >> l) & 1u)) continue;
        unsigned o;
        std::memcpy(&o, emu::t_warp->slot[l], sizeof(o));
        r |= o;
    }
    b.arrive_and_wait();
    return r;
}

inline int __all_sync(unsigned mask, int pred) { return __ballot_sync(mask, pred) == mask; }
inline int __any_sync(unsigned mask, int pred) { return __ballot_sync(mask, pred) != 0; }
inline int __all(int pred) { return __all_sync(emu::t_warp->active, pred); }

template <typename T>
inline unsigned __match_any_sync(unsigned mask, T value) {
    const unsigned long long v = static_cast<unsigned long long>(value);
    std::barrier<>& b = emu::deposit(mask, &v, sizeof(v));
    unsigned r = 0;
    for (int l = 0; l < 32; ++l) {
        if (!((mask >> l) & 1u)) continue;
        unsigned long long o;
        std::memcpy(&o, emu::t_warp->slot[l], sizeof(o));
        if (o == v) r |= 1u << l;
    }
    b.arrive_and_wait();
    return r;
}

inline void __syncwarp(unsigned mask = 0xFFFFFFFFu) {
    const char z = 0;
    emu::deposit(mask, &z, 1).arrive_and_wait();
}
