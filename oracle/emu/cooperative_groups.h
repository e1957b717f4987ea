// Shim of <cooperative_groups.h> for the host lane emulator — TEST
// INFRASTRUCTURE ONLY.  Provides the few names the reference's trove/warp.h
// uses (this_thread_block, tiled_partition, thread_block_tile::shfl /
// thread_rank / num_threads) on top of lane_emu.h.
#pragma once

#ifndef TROVE_LANE_EMULATION
#error "cooperative_groups shim is for the host lane emulator only"
#endif

namespace cooperative_groups {

struct thread_block {};
inline thread_block this_thread_block() { return thread_block(); }

template <unsigned int Size, typename ParentT = void>
class thread_block_tile {
    static unsigned group_mask() {
        if (Size >= 32) return 0xFFFFFFFFu;
        return ((1u << Size) - 1u) << (trove_emu_lane_id() & ~(Size - 1));
    }

public:
    static constexpr unsigned long long num_threads() { return Size; }
    unsigned long long thread_rank() const { return trove_emu_lane_id() & (Size - 1); }
    template <typename T>
    T shfl(T var, int src) const {
        return emu::shfl(group_mask(), var, src, int(Size));
    }
};

template <unsigned int Size, typename ParentT>
thread_block_tile<Size> tiled_partition(const ParentT&) {
    return thread_block_tile<Size>();
}

}  // namespace cooperative_groups
