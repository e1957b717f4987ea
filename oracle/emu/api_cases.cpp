// Device-API test cases run on the host lane emulator — TEST INFRASTRUCTURE.
//
// One source, compiled twice by oracle/build_oracle.py:
//   * against the reference headers (-I <reference>) -> oracle/_ref/, used
//     only by tests/golden/gen_golden.py to record golden vectors, and
//   * against this repository's include/ -> oracle/_build/, checked against
//     those vectors by the CPU test suite.
// The per-lane bodies follow the reference's own test kernels:
// tests/benchmark.cu:52-128 (contiguous store / load+sum, coalesced_ptr
// gather and scatter) and tests/block.cu:13-54 (block write and copy with a
// warp_converged() check).  `D[i] = S[idx[i]]` is written as two statements
// because the reference's ref-to-ref assignment does not compile
// (trove/ptr.h:49-50).  Every entry point returns 0 on success.
#include <cstring>
#include <trove/aos.h>
#include <trove/block.h>
#include <trove/memory.h>
#include <trove/ptr.h>
#include <trove/rotate.h>
#include <trove/transpose.h>
#include <trove/utility.h>
#include <trove/warp.h>

#include <utility>

namespace {

typedef std::integer_sequence<int, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 20, 24, 33>
    widths;

void set_lane_ids(int warp, int lane) {
    threadIdx.x = unsigned(lane);
    threadIdx.y = threadIdx.z = 0;
    blockDim.x = 32;
    blockDim.y = blockDim.z = 1;
    blockIdx.x = unsigned(warp);
    blockIdx.y = blockIdx.z = 0;
    gridDim.x = 1u << 30;
    gridDim.y = gridDim.z = 1;
}

unsigned lanes_below(long long count) {
    return count >= 32 ? 0xFFFFFFFFu : (count <= 0 ? 0u : ((1u << count) - 1u));
}

template <typename T>
unsigned first_word(const T& v) {
    unsigned w;
    std::memcpy(&w, &v, sizeof(w));
    return w;
}

template <int s>
struct cases {
    typedef trove::array<int, s> T;

    template <int tile>
    static void copy_tile(const T* src, T* dst, int n) {
        for (int w = 0; w < n / 32; ++w)
            emu::run_warp(0xFFFFFFFFu, [&](int lane) {
                set_lane_ids(w, lane);
                const int i = w * 32 + lane;
                T v = trove::load_warp_contiguous<tile>(src + i);
                trove::store_warp_contiguous<tile>(v, dst + i);
            });
    }

    static int copy(int tile, const void* src, void* dst, int n) {
        const T* s_ = static_cast<const T*>(src);
        T* d_ = static_cast<T*>(dst);
        switch (tile) {
            case 32: copy_tile<32>(s_, d_, n); return 0;
            case 16: copy_tile<16>(s_, d_, n); return 0;
            case 8: copy_tile<8>(s_, d_, n); return 0;
            case 4: copy_tile<4>(s_, d_, n); return 0;
            case 2: copy_tile<2>(s_, d_, n); return 0;
        }
        return 1;
    }

    // tests/benchmark.cu:52-61: store counting_array(i * s) warp-contiguously.
    static int store_counting(void* dst, int n) {
        T* r = static_cast<T*>(dst);
        for (int w = 0; w < n / 32; ++w)
            emu::run_warp(0xFFFFFFFFu, [&](int lane) {
                set_lane_ids(w, lane);
                const int i = w * 32 + lane;
                T data = trove::counting_array<T>::impl(i * s);
                trove::store_warp_contiguous(data, r + i);
            });
        return 0;
    }

    // tests/benchmark.cu:74-80: load warp-contiguously, write the word sum.
    static int load_sum(const void* src, int* out, int n) {
        const T* p = static_cast<const T*>(src);
        for (int w = 0; w < n / 32; ++w)
            emu::run_warp(0xFFFFFFFFu, [&](int lane) {
                set_lane_ids(w, lane);
                const int i = w * 32 + lane;
                T data = trove::load_warp_contiguous(p + i);
                out[i] = trove::sum(data);
            });
        return 0;
    }

    // tests/benchmark.cu:90-99 (gather) and :101-110 (scatter); the last warp
    // is partial when n % 32 != 0, which exercises the non-converged paths.
    static int gather(const void* src, const int* idx, void* dst, int n) {
        T* s_ = const_cast<T*>(static_cast<const T*>(src));
        T* d_ = static_cast<T*>(dst);
        for (int w = 0; w * 32 < n; ++w)
            emu::run_warp(lanes_below(n - w * 32), [&](int lane) {
                set_lane_ids(w, lane);
                const int i = w * 32 + lane;
                trove::coalesced_ptr<T> S(s_);
                trove::coalesced_ptr<T> D(d_);
                T v = S[idx[i]];
                D[i] = v;
            });
        return 0;
    }

    static int scatter(const void* src, const int* idx, void* dst, int n) {
        T* s_ = const_cast<T*>(static_cast<const T*>(src));
        T* d_ = static_cast<T*>(dst);
        for (int w = 0; w * 32 < n; ++w)
            emu::run_warp(lanes_below(n - w * 32), [&](int lane) {
                set_lane_ids(w, lane);
                const int i = w * 32 + lane;
                trove::coalesced_ptr<T> S(s_);
                trove::coalesced_ptr<T> D(d_);
                T v = S[i];
                D[idx[i]] = v;
            });
        return 0;
    }

    // tests/block.cu:13-32 / :34-54 for array<int, s> with length l: write
    // counting_array(s * index), or copy, choosing the warp-contiguous form
    // when warp_converged() and the per-thread form otherwise.
    static int block(int write, const int* src, int* dst, int l) {
        for (int w = 0; w * 32 < l; ++w)
            emu::run_warp(lanes_below(l - w * 32), [&](int lane) {
                set_lane_ids(w, lane);
                const int index = w * 32 + lane;
                if (write) {
                    T d = trove::counting_array<T>::impl(s * index);
                    if (trove::warp_converged())
                        trove::store_array_warp_contiguous<s>(dst, index, d);
                    else
                        trove::store_array(dst, index, d);
                } else {
                    T d;
                    if (trove::warp_converged())
                        d = trove::load_array_warp_contiguous<s>(src, index);
                    else
                        d = trove::load_array<s>(src, index);
                    if (trove::warp_converged())
                        trove::store_array_warp_contiguous(dst, index, d);
                    else
                        trove::store_array(dst, index, d);
                }
            });
        return 0;
    }

    // Copy with a data-dependent early exit between load and store: a lane
    // whose struct's first word w satisfies w % modulus == modulus - 1 stops
    // and does not store (modulus 0: no exits).  Each warp runs in two phases
    // so that the store phase sees the exited lanes as inactive.
    // api 0: load/store_warp_contiguous; api 1: block interface.
    static int copy_exit(int api, const void* src, void* dst, long long n, unsigned modulus) {
        const T* s_ = static_cast<const T*>(src);
        T* d_ = static_cast<T*>(dst);
        T held[32];
        for (long long w = 0; w * 32 < n; ++w) {
            const unsigned live = lanes_below(n - w * 32);
            emu::run_warp(live, [&](int lane) {
                set_lane_ids(int(w), lane);
                const long long i = w * 32 + lane;
                if (api == 0)
                    held[lane] = trove::warp_converged() ? trove::load_warp_contiguous(s_ + i) : s_[i];
                else
                    held[lane] = trove::warp_converged()
                                     ? trove::load_array_warp_contiguous<s>(&s_[0].head, i)
                                     : trove::load_array<s>(&s_[0].head, i);
            });
            unsigned stay = 0;
            for (int lane = 0; lane < 32; ++lane)
                if (((live >> lane) & 1u) &&
                    !(modulus != 0 && first_word(held[lane]) % modulus == modulus - 1))
                    stay |= 1u << lane;
            if (!stay) continue;
            emu::run_warp(stay, [&](int lane) {
                set_lane_ids(int(w), lane);
                const long long i = w * 32 + lane;
                if (api == 0) {
                    if (trove::warp_converged())
                        trove::store_warp_contiguous(held[lane], d_ + i);
                    else
                        d_[i] = held[lane];
                } else {
                    if (trove::warp_converged())
                        trove::store_array_warp_contiguous(&d_[0].head, i, held[lane]);
                    else
                        trove::store_array(&d_[0].head, i, held[lane]);
                }
            });
        }
        return 0;
    }
};

// trove/memory.h on the host (the functions are __host__ __device__ and use
// no lane): kind 0 warp_load, 1 warp_load through a volatile pointer,
// 2 warp_store of in[0..S) into out, 3 uncoalesced_store of in[0..S).
template <int S>
int memory_case(int kind, int offset, int stride, const int* in, int* out) {
    typedef trove::array<int, S> A;
    if (kind == 0 || kind == 1) {
        const A a = kind == 0 ? trove::warp_load<A>(in, offset, stride)
                              : trove::warp_load<A>(static_cast<const volatile int*>(in), offset, stride);
        std::memcpy(out, &a, sizeof(A));
    } else {
        A a;
        std::memcpy(&a, in, sizeof(A));
        if (kind == 2)
            trove::warp_store(a, out, offset, stride);
        else
            trove::uncoalesced_store(a, out, stride);
    }
    return 0;
}

template <typename F, int... S>
int dispatch_width(int s, F&& f, std::integer_sequence<int, S...>) {
    int rc = 2;
    ((s == S ? (rc = f(std::integral_constant<int, S>()), 0) : 0), ...);
    return rc;
}

// --- transposes: one tile of n lanes, m elements of E per lane --------------
template <int n, int m, typename E>
void transpose_tile(int dir, int* data) {
    typedef trove::array<E, m> A;
    const unsigned live = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
    emu::run_warp(live, [&](int lane) {
        set_lane_ids(0, lane);
        E* mine = reinterpret_cast<E*>(data) + lane * m;
        A a = trove::make_array<E, m>(mine);
        trove::thread_tile<n> tile;
        if (dir == 0)
            trove::r2c_warp_transpose(a, tile);
        else
            trove::c2r_warp_transpose(a, tile);
        trove::make_carray(a, mine);
    });
}

template <int n, typename E, int... M>
int transpose_m(int dir, int m, int* data, std::integer_sequence<int, M...>) {
    int rc = 2;
    ((m == M + 2 ? (transpose_tile<n, M + 2, E>(dir, data), rc = 0) : 0), ...);
    return rc;
}

template <int n, typename E>
int transpose_n(int dir, int m, int* data) {
    if (m < 2 || m > n) return 2;
    return transpose_m<n, E>(dir, m, data, std::make_integer_sequence<int, n - 1>());
}

template <typename E>
int transpose_e(int dir, int n, int m, int* data) {
    switch (n) {
        case 2: return transpose_n<2, E>(dir, m, data);
        case 4: return transpose_n<4, E>(dir, m, data);
        case 8: return transpose_n<8, E>(dir, m, data);
        case 16: return transpose_n<16, E>(dir, m, data);
        case 32: return transpose_n<32, E>(dir, m, data);
    }
    return 2;
}

template <int... M>
int rotate_m(int m, int a, const int* in, int* out, std::integer_sequence<int, M...>) {
    int rc = 2;
    ((m == M + 1 ? (trove::make_carray(
                        trove::rotate(trove::make_array<int, M + 1>(const_cast<int*>(in)), a), out),
                    rc = 0)
                 : 0),
     ...);
    return rc;
}

}  // namespace

extern "C" {

// dir 0: r2c_warp_transpose, 1: c2r_warp_transpose; words 1/2/4 = int/int2/int4.
// data: n lanes x m elements x words ints, lane-major, transformed in place.
int emu_transpose(int dir, int n, int m, int words, int* data) {
    switch (words) {
        case 1: return transpose_e<int>(dir, n, m, data);
        case 2: return n == 32 ? transpose_e<int2>(dir, n, m, data) : 2;
        case 4: return n == 32 ? transpose_e<int4>(dir, n, m, data) : 2;
    }
    return 2;
}

int emu_rotate(int m, int a, const int* in, int* out) {
    return rotate_m(m, a, in, out, std::make_integer_sequence<int, 32>());
}

int emu_copy(int s, int tile, const void* src, void* dst, int n) {
    return dispatch_width(s, [&](auto S) { return cases<decltype(S)::value>::copy(tile, src, dst, n); }, widths());
}

int emu_store_counting(int s, void* dst, int n) {
    return dispatch_width(s, [&](auto S) { return cases<decltype(S)::value>::store_counting(dst, n); }, widths());
}

int emu_load_sum(int s, const void* src, int* out, int n) {
    return dispatch_width(s, [&](auto S) { return cases<decltype(S)::value>::load_sum(src, out, n); }, widths());
}

int emu_gather(int s, const void* src, const int* idx, void* dst, int n) {
    return dispatch_width(s, [&](auto S) { return cases<decltype(S)::value>::gather(src, idx, dst, n); }, widths());
}

int emu_scatter(int s, const void* src, const int* idx, void* dst, int n) {
    return dispatch_width(s, [&](auto S) { return cases<decltype(S)::value>::scatter(src, idx, dst, n); }, widths());
}

int emu_block(int s, int write, const int* src, int* dst, int l) {
    return dispatch_width(s, [&](auto S) { return cases<decltype(S)::value>::block(write, src, dst, l); }, widths());
}

int emu_copy_exit(int s, int api, const void* src, void* dst, long long n, unsigned modulus) {
    return dispatch_width(
        s, [&](auto S) { return cases<decltype(S)::value>::copy_exit(api, src, dst, n, modulus); }, widths());
}

int emu_memory(int s, int kind, int offset, int stride, const int* in, int* out) {
    return dispatch_width(s, [&](auto S) { return memory_case<decltype(S)::value>(kind, offset, stride, in, out); },
                          widths());
}

// warp_converged<N>() seen by each lane of `active`; out[lane] = 0/1, lanes
// outside `active` are left untouched.
int emu_warp_converged(int N, unsigned active, unsigned char* out) {
    emu::run_warp(active, [&](int lane) {
        set_lane_ids(0, lane);
        bool r = false;
        switch (N) {
            case 32: r = trove::warp_converged<32>(); break;
            case 16: r = trove::warp_converged<16>(); break;
            case 8: r = trove::warp_converged<8>(); break;
            case 4: r = trove::warp_converged<4>(); break;
            case 2: r = trove::warp_converged<2>(); break;
        }
        out[lane] = r ? 1 : 0;
    });
    return 0;
}

}  // extern "C"
