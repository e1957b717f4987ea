/*
 * CPU oracle for AoS copy / gather / scatter — TEST INFRASTRUCTURE ONLY.
 *
 * Plain C restatement of what the reference's hot path computes, used by the
 * test suite as the bit-exact reference result, by __graft_entry__.smoke(), and by
 * bench.py's CPU baseline.  Nothing in the product links or calls it.
 *
 * The reference is a device-only template library; its semantics on the hot
 * path are:
 *   - load_warp_contiguous / store_warp_contiguous (trove/aos.h:66-105) and
 *     the block interface (trove/block.h:35-65): lane i moves struct i, so a
 *     kernel that loads then stores copies dst[i] = src[i];
 *   - coalesced_ptr reads/writes (trove/ptr.h:39-45 -> trove/aos.h:258-290):
 *     dst[i] = src[idx[i]] (gather, tests/benchmark.cu:90-99) and
 *     dst[idx[i]] = src[i] (scatter, tests/benchmark.cu:101-110);
 *   - r2c_warp_transpose (trove/transpose.h:672-696): lane l, element j of a
 *     tile of n lanes receives word l*m + j of the row-form block, which sits
 *     in lane (l*m + j) % n, element (l*m + j) / n;
 *   - the reference's known-answer kernels: counting_array stores
 *     (tests/benchmark.cu:52-61, tests/block.cu:13-32) and load+sum
 *     (tests/benchmark.cu:74-80, trove/utility.h:75-78).
 * Payload is bytes; nothing is interpreted except where a test kernel says
 * so (the early-exit predicate reads the first 32-bit word).
 *
 * The seeded generators define the synthetic inputs of every workload:
 * orc_word() is a counter-based splitmix64 stream, so the CUDA library's
 * fill kernel reproduces it bit for bit at any size.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---- seeded synthetic inputs -------------------------------------------- */

static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Word k of the stream for `seed`. */
uint32_t orc_word(uint64_t seed, uint64_t k) {
    return (uint32_t)(mix64(k * 0x9E3779B97F4A7C15ull + seed * 0xD1B54A32D192ED03ull + 1) >> 32);
}

typedef struct {
    uint32_t* out;
    uint64_t begin, end, seed;
} fill_job;

static void* fill_worker(void* p) {
    fill_job* j = (fill_job*)p;
    for (uint64_t k = j->begin; k < j->end; ++k) j->out[k] = orc_word(j->seed, k);
    return NULL;
}

void orc_fill_u32(uint32_t* out, uint64_t nwords, uint64_t seed, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    fill_job jobs[256];
    for (int t = 0; t < threads; ++t) {
        jobs[t].out = out;
        jobs[t].seed = seed;
        jobs[t].begin = nwords * (uint64_t)t / (uint64_t)threads;
        jobs[t].end = nwords * (uint64_t)(t + 1) / (uint64_t)threads;
        pthread_create(&th[t], NULL, fill_worker, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
}

/* Uniform integer in [0, bound) from stream position k (bound < 2^32). */
static inline uint32_t bounded(uint64_t seed, uint64_t k, uint32_t bound) {
    return (uint32_t)(((uint64_t)orc_word(seed, k) * (uint64_t)bound) >> 32);
}

/* Fisher-Yates permutation of 0..n-1 driven by the stream. */
void orc_permutation(int32_t* idx, uint64_t n, uint64_t seed) {
    for (uint64_t i = 0; i < n; ++i) idx[i] = (int32_t)i;
    for (uint64_t i = n; i > 1; --i) {
        uint64_t j = bounded(seed, i, (uint32_t)i);
        int32_t t = idx[i - 1];
        idx[i - 1] = idx[j];
        idx[j] = t;
    }
}

/* n indices uniform in [0, range). */
void orc_uniform_indices(int32_t* idx, uint64_t n, uint32_t range, uint64_t seed) {
    for (uint64_t i = 0; i < n; ++i) idx[i] = (int32_t)bounded(seed, i, range);
}

/* Run pattern: for each aligned chunk of 32 outputs, with probability 1/2 a
 * run start + 0..31 (start uniform in [0, n-32]), else 32 independent
 * uniform indices.  Requires n >= 32. */
void orc_run_indices(int32_t* idx, uint64_t n, uint64_t seed) {
    for (uint64_t c = 0; c * 32 < n; ++c) {
        uint64_t base = c * 32;
        uint64_t len = n - base < 32 ? n - base : 32;
        if (orc_word(seed, 2 * c) & 1u) {
            uint32_t start = bounded(seed, 2 * c + 1, (uint32_t)(n - 32 + 1));
            for (uint64_t k = 0; k < len; ++k) idx[base + k] = (int32_t)(start + k);
        } else {
            for (uint64_t k = 0; k < len; ++k)
                idx[base + k] = (int32_t)bounded(seed ^ 0x5bd1e995ull, base + k, (uint32_t)n);
        }
    }
}

/* ---- the path's semantics ------------------------------------------------ */

void orc_copy(void* dst, const void* src, uint64_t n, uint32_t width) {
    const unsigned char* s = (const unsigned char*)src;
    unsigned char* d = (unsigned char*)dst;
    for (uint64_t i = 0; i < n; ++i) memcpy(d + i * width, s + i * width, width);
}

void orc_gather(void* dst, const void* src, const int32_t* idx, uint64_t n, uint32_t width) {
    const unsigned char* s = (const unsigned char*)src;
    unsigned char* d = (unsigned char*)dst;
    for (uint64_t i = 0; i < n; ++i) memcpy(d + i * width, s + (uint64_t)idx[i] * width, width);
}

void orc_scatter(void* dst, const void* src, const int32_t* idx, uint64_t n, uint32_t width) {
    const unsigned char* s = (const unsigned char*)src;
    unsigned char* d = (unsigned char*)dst;
    for (uint64_t i = 0; i < n; ++i) memcpy(d + (uint64_t)idx[i] * width, s + i * width, width);
}

/* Early-exit copy: struct i is copied unless its first 32-bit word w has
 * w % modulus == modulus - 1 (modulus 0: never); returns structs written. */
uint64_t orc_copy_exit(void* dst, const void* src, uint64_t n, uint32_t width, uint32_t modulus) {
    const unsigned char* s = (const unsigned char*)src;
    unsigned char* d = (unsigned char*)dst;
    uint64_t written = 0;
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t w0;
        memcpy(&w0, s + i * width, 4);
        if (modulus != 0 && w0 % modulus == modulus - 1) continue;
        memcpy(d + i * width, s + i * width, width);
        ++written;
    }
    return written;
}

/* Known answer of the counting-array kernels: struct i of s words holds
 * i*s, i*s+1, ..., i*s+s-1, i.e. word k == k. */
void orc_counting(int32_t* dst, uint64_t n, int s) {
    for (uint64_t k = 0; k < n * (uint64_t)s; ++k) dst[k] = (int32_t)k;
}

/* Known answer of the load+sum kernel: out[i] = sum of struct i's words
 * (wrapping 32-bit addition, left to right). */
void orc_load_sum(const int32_t* src, int32_t* out, uint64_t n, int s) {
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t acc = 0;
        for (int j = 0; j < s; ++j) acc += (uint32_t)src[i * (uint64_t)s + j];
        out[i] = (int32_t)acc;
    }
}

/* R2C semantics for a tile of n lanes and m elements: column element (l, j)
 * comes from row lane src_lane[l*m+j], row element src_elem[l*m+j]. */
void orc_r2c_source(int n, int m, int32_t* src_lane, int32_t* src_elem) {
    for (int l = 0; l < n; ++l)
        for (int j = 0; j < m; ++j) {
            int w = l * m + j;
            src_lane[w] = w % n;
            src_elem[w] = w / n;
        }
}

/* AoS -> SoA for structs of s 32-bit fields: soa[j*n + i] = aos[i*s + j]
 * (the conversion a block-interface producer/consumer kernel performs; the
 * reference's README "Block Interface"). */
void orc_aos_to_soa(uint32_t* soa, const uint32_t* aos, uint64_t n, int s) {
    for (uint64_t i = 0; i < n; ++i)
        for (int j = 0; j < s; ++j) soa[(uint64_t)j * n + i] = aos[i * (uint64_t)s + j];
}

/* ---- multithreaded forms, for the timed CPU baseline --------------------- */

typedef struct {
    int op; /* 0 copy, 1 gather, 2 scatter, 3 early-exit copy (modulus in idx slot),
               4 AoS -> SoA, 5 SoA -> AoS */
    unsigned char* dst;
    const unsigned char* src;
    const int32_t* idx;
    uint64_t begin, end, total;
    uint32_t width;
} mt_job;

/* Structs [begin, end) of an n-struct array of s words: AoS -> SoA planes
 * (plane j, word i at soa[j * n + i]) or back. */
static void layout_range(int to_soa, uint32_t* dst, const uint32_t* src, uint64_t begin, uint64_t end, uint64_t n,
                         int s) {
    for (uint64_t i = begin; i < end; ++i)
        for (int j = 0; j < s; ++j) {
            if (to_soa)
                dst[(uint64_t)j * n + i] = src[i * (uint64_t)s + j];
            else
                dst[i * (uint64_t)s + j] = src[(uint64_t)j * n + i];
        }
}

static void* mt_worker(void* p) {
    mt_job* j = (mt_job*)p;
    uint64_t cnt = j->end - j->begin;
    if (j->op == 0) {
        orc_copy(j->dst + j->begin * j->width, j->src + j->begin * j->width, cnt, j->width);
    } else if (j->op == 3) {
        orc_copy_exit(j->dst + j->begin * j->width, j->src + j->begin * j->width, cnt, j->width,
                      (uint32_t)(uintptr_t)j->idx);
    } else if (j->op == 4 || j->op == 5) {
        layout_range(j->op == 4, (uint32_t*)j->dst, (const uint32_t*)j->src, j->begin, j->end, j->total,
                     (int)(j->width / 4));
    } else if (j->op == 1) {
        orc_gather(j->dst + j->begin * j->width, j->src, j->idx + j->begin, cnt, j->width);
    } else {
        orc_scatter(j->dst, j->src + j->begin * j->width, j->idx + j->begin, cnt, j->width);
    }
    return NULL;
}

/* Static split of n structs over `threads` POSIX threads.  For op 3 the
 * early-exit modulus travels in the idx argument's value; ops 4 and 5 (the
 * AoS <-> SoA layouts of aos_oracle's orc_aos_to_soa) need width % 4 == 0. */
void orc_run_mt(int op, void* dst, const void* src, const int32_t* idx, uint64_t n, uint32_t width,
                int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    mt_job jobs[256];
    for (int t = 0; t < threads; ++t) {
        jobs[t].op = op;
        jobs[t].dst = (unsigned char*)dst;
        jobs[t].src = (const unsigned char*)src;
        jobs[t].idx = idx;
        jobs[t].width = width;
        jobs[t].total = n;
        jobs[t].begin = n * (uint64_t)t / (uint64_t)threads;
        jobs[t].end = n * (uint64_t)(t + 1) / (uint64_t)threads;
        pthread_create(&th[t], NULL, mt_worker, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
}
