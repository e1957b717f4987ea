// Autotuner: times candidate launch shapes on the GPU and caches the winner
// per (scope, op, width, length bucket).
//
//  - SCOPE_CALL entries steer the AUTO path of trv_copy / trv_gather /
//    trv_scatter (path, unroll, grid shape, bulk chunk).  trv_autotune_call
//    measures them on scratch arrays of the requested size.
//  - SCOPE_BATCH entries give the batched kernel its tile size and, for copy
//    tasks, the copy variant.  trv_autotune_batch measures them on the
//    caller's own batch: the tasks of each (op, width, bucket) group run
//    alone as a sub-batch under every candidate.
// The cache is process-wide, guarded by a mutex, and saved / loaded as a
// small JSON array (trv_autotune_save / trv_autotune_load).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "autotune.h"
#include "runtime.h"
#include "trove_gb300.h"

namespace trv {
namespace {

std::mutex g_mu;
std::map<std::tuple<int, int, int, int>, TuneChoice> g_table;

std::tuple<int, int, int, int> as_tuple(const TuneKey& k) { return std::make_tuple(k.scope, k.op, k.width, k.bucket); }

// Written between timed runs so every candidate starts from a cold L2 (the
// way a large stream of calls meets it): twice the 129 MB L2 of GB300.
struct L2Flush {
    void* buf = nullptr;
    size_t bytes = size_t(256) << 20;
    L2Flush() {
        if (cudaMalloc(&buf, bytes) != cudaSuccess) {
            cudaGetLastError();
            buf = nullptr;
        }
    }
    ~L2Flush() {
        if (buf) cudaFree(buf);
    }
    void run(cudaStream_t st, int value) const {
        if (buf) cudaMemsetAsync(buf, value, bytes, st);
    }
};

// Median milliseconds of `reps` runs of fn after one warm-up run, each run
// timed alone with CUDA events on `st` after an L2 flush.  Negative on
// failure.
template <typename F>
float time_ms(F&& fn, cudaStream_t st, const L2Flush& flush, int reps = 3) {
    if (fn() != TRV_OK) return -1.f;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return -1.f;
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return -1.f;
    }
    std::vector<float> times;
    int rc = TRV_OK;
    for (int r = 0; r < reps && rc == TRV_OK; ++r) {
        flush.run(st, r);
        cudaEventRecord(a, st);
        rc = fn();
        cudaEventRecord(b, st);
        float ms = -1.f;
        if (rc == TRV_OK && cudaEventSynchronize(b) == cudaSuccess && cudaEventElapsedTime(&ms, a, b) == cudaSuccess)
            times.push_back(ms);
        else
            rc = TRV_ERR_CUDA;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaGetLastError();
    if (rc != TRV_OK || times.empty()) return -1.f;
    std::sort(times.begin(), times.end());
    return times[times.size() / 2];
}

struct Scratch {
    void* src = nullptr;
    void* dst = nullptr;
    int* idx = nullptr;
    ~Scratch() {
        if (src) cudaFree(src);
        if (dst) cudaFree(dst);
        if (idx) cudaFree(idx);
    }
};

__global__ void uniform_index_kernel(int* idx, long long n, long long bound, unsigned long long seed) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        unsigned long long z = (unsigned long long)i * 0x9E3779B97F4A7C15ull + seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        idx[i] = (int)((z >> 32) % (unsigned long long)bound);
    }
}

__global__ void iota_index_kernel(int* idx, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) idx[i] = (int)i;
}

// Gather / scatter shapes within this fraction of the best time on random
// indices are all fast on random indices; the tie is broken on contiguous
// indices.
constexpr float kTieBand = 0.02f;

}  // namespace

int len_bucket(uint64_t n) {
    int lg = 0;
    while (n > 1) {
        n >>= 1;
        ++lg;
    }
    return lg / 2;
}

bool tune_lookup(const TuneKey& key, TuneChoice* out) {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_table.find(as_tuple(key));
    if (it == g_table.end()) return false;
    if (out) *out = it->second;
    return true;
}

void tune_store(const TuneKey& key, const TuneChoice& choice) {
    std::lock_guard<std::mutex> g(g_mu);
    g_table[as_tuple(key)] = choice;
}

}  // namespace trv

using namespace trv;

extern "C" {

static int32_t autotune_call_impl(int32_t op, uint32_t width, uint64_t n, void* stream) {
    if (op < TRV_OP_COPY || op > TRV_OP_SOA_TO_AOS || width == 0 || n == 0 || n > (uint64_t(1) << 40) / width)
        return TRV_ERR_INVALID_ARGUMENT;
    const bool exit_op = op == TRV_OP_COPY_EXIT_WARP || op == TRV_OP_COPY_EXIT_BLOCK;
    const bool layout_op = op == TRV_OP_AOS_TO_SOA || op == TRV_OP_SOA_TO_AOS;
    if ((exit_op || layout_op) && (width % 4 != 0 || width > 64)) return TRV_ERR_UNSUPPORTED;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch s;
    const L2Flush flush;
    const size_t bytes = size_t(n) * width;
    cudaError_t e = cudaMalloc(&s.src, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&s.dst, bytes);
    if (e == cudaSuccess && (op == TRV_OP_GATHER || op == TRV_OP_SCATTER)) e = cudaMalloc(&s.idx, sizeof(int) * n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? TRV_ERR_OUT_OF_MEMORY : cuda_fail(e);
    }
    if (width % 4 == 0) trv_fill_random_u32(static_cast<uint32_t*>(s.src), bytes / 4, 1, stream);
    if (s.idx) {
        uniform_index_kernel<<<device_info().sm_count * 4, 256, 0, st>>>(s.idx, (long long)n, (long long)n, 7);
        if (cudaGetLastError() != cudaSuccess) return TRV_ERR_CUDA;
    }
    std::vector<trv_launch> cands;
    if (exit_op) {
        const int path = op == TRV_OP_COPY_EXIT_WARP ? TRV_PATH_WARP : TRV_PATH_BLOCK;
        for (int u : {1, 2, 4, 8}) cands.push_back({path, u, 0, 0, 0, 0});
    } else if (layout_op) {
        for (int u : {1, 2, 4, 8}) cands.push_back({TRV_PATH_WARP, u, 0, 0, 0, 0});
    } else if (op == TRV_OP_COPY) {
        for (int chunk : {16 << 10, 24 << 10}) cands.push_back({TRV_PATH_BULK, 0, 0, 0, chunk, 0});
        for (int u : {2, 4, 8}) cands.push_back({TRV_PATH_VECTOR, u, 0, 0, 0, 0});
        if (width % 4 == 0 && width <= 64)
            for (int u : {1, 2, 4, 8}) cands.push_back({TRV_PATH_WARP, u, 0, 0, 0, 0});
    } else if (width % 4 == 0 && width <= 64) {
        for (int u : {1, 2, 4, 8})
            for (int cp : {0, 1, 3, 4, 5, 6}) {
                if ((cp == 4 || cp == 5) && op != TRV_OP_GATHER) continue;  // load hints: a scatter's random side is stores
                if (cp == 6 && op != TRV_OP_SCATTER) continue;              // destination passes
                cands.push_back({TRV_PATH_WARP, u, 0, 0, 0, cp});
            }
        for (int u : {1, 2, 4}) cands.push_back({TRV_PATH_COALESCED, u, 0, 0, 0, 0});
    } else {
        cands.push_back({TRV_PATH_VECTOR, 0, 0, 0, 0, 0});
    }
    float best = -1.f;
    trv_launch pick{};
    std::vector<float> times(cands.size(), -1.f);
    auto run_cand = [&](const trv_launch& c) -> int {
        if (exit_op) return trv_copy_exit_ex(s.dst, s.src, n, width, 625u, &c, stream);
        if (op == TRV_OP_AOS_TO_SOA) return trv_aos_to_soa_ex(s.dst, s.src, n, width, &c, stream);
        if (op == TRV_OP_SOA_TO_AOS) return trv_soa_to_aos_ex(s.dst, s.src, n, width, &c, stream);
        if (op == TRV_OP_COPY) return trv_copy_ex(s.dst, s.src, n, width, &c, stream);
        if (op == TRV_OP_GATHER) return trv_gather_ex(s.dst, s.src, n, s.idx, n, width, &c, stream);
        return trv_scatter_ex(s.dst, n, s.src, s.idx, n, width, &c, stream);
    };
    for (size_t ci = 0; ci < cands.size(); ++ci) {
        const trv_launch& c = cands[ci];
        const float ms = time_ms([&]() -> int { return run_cand(c); }, st, flush);
        times[ci] = ms;
        if (ms > 0.f && (best < 0.f || ms < best)) {
            best = ms;
            pick = c;
        }
    }
    if (best < 0.f) return TRV_ERR_CUDA;
    // Gathers and scatters are tuned on uniform random indices, where shapes
    // of the same path often tie.  The shapes within kTieBand of the best are
    // timed again on contiguous indices (idx[i] = i), which random timing
    // cannot see, and the fastest there wins: runs and consecutive stretches
    // of indices then get the shape that handles them best, at no measurable
    // cost on random ones.
    float pick_ms = best;
    if (op == TRV_OP_GATHER || op == TRV_OP_SCATTER) {
        std::vector<size_t> band;
        for (size_t ci = 0; ci < cands.size(); ++ci)
            if (times[ci] > 0.f && times[ci] <= best * (1.f + kTieBand)) band.push_back(ci);
        if (band.size() > 1) {
            iota_index_kernel<<<device_info().sm_count * 4, 256, 0, st>>>(s.idx, (long long)n);
            if (cudaGetLastError() != cudaSuccess) return TRV_ERR_CUDA;
            float best_c = -1.f;
            for (size_t ci : band) {
                const float ms = time_ms([&]() -> int { return run_cand(cands[ci]); }, st, flush);
                if (ms > 0.f && (best_c < 0.f || ms < best_c)) {
                    best_c = ms;
                    pick = cands[ci];
                    pick_ms = times[ci];
                }
            }
        }
    }
    TuneChoice ch;
    ch.path = pick.path;
    ch.unroll = pick.unroll;
    ch.grid = pick.grid_blocks;
    ch.chunk = pick.chunk_bytes;
    ch.cache_policy = pick.cache_policy;
    const double alg = double(bytes) * 2 + (op == TRV_OP_GATHER || op == TRV_OP_SCATTER ? 4.0 * double(n) : 0.0);
    ch.gbs = alg / (double(pick_ms) * 1e6);
    tune_store(TuneKey{SCOPE_CALL, op, int(width), len_bucket(n)}, ch);
    return TRV_OK;
}

int32_t trv_autotune_call(int32_t op, uint32_t width, uint64_t n, void* stream) {
    return no_throw([&] { return autotune_call_impl(op, width, n, stream); });
}

static int32_t autotune_batch_impl(const trv_task* tasks, uint64_t count, void* stream) {
    if (count > 0 && !tasks) return TRV_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const L2Flush flush;
    std::map<std::tuple<int, int, int>, std::vector<trv_task>> groups;
    for (uint64_t k = 0; k < count; ++k)
        groups[std::make_tuple(tasks[k].op, int(tasks[k].width), len_bucket(tasks[k].n))].push_back(tasks[k]);
    for (auto& kv : groups) {
        const int op = std::get<0>(kv.first);
        // (tile_bytes, blocks per SM, gather / scatter policy, copy tile path)
        std::vector<std::tuple<int, int, int, int>> cands;
        for (int tb : {32 << 10, 64 << 10, 128 << 10, 256 << 10, 1 << 20})
            for (int bps : {2, 4})
                for (int gp : {1, 4, 5, 6, 7})
                    for (int cpath : {TRV_PATH_AUTO, TRV_PATH_VECTOR}) {
                        if ((gp == 4 || gp > 5) && op != TRV_OP_GATHER) continue;  // load hints
                        if (gp != 1 && op == TRV_OP_COPY) continue;
                        if (cpath == TRV_PATH_VECTOR && op != TRV_OP_COPY) continue;
                        // the register budget is one per batch and set by its
                        // gathers and scatters; copy groups are timed at the
                        // default budget (4 blocks per SM)
                        if (bps == 2 && op == TRV_OP_COPY) continue;
                        // the 4-block build stages every row: register-row policies
                        // would repeat the staged ones there
                        if (bps == 4 && (gp == 1 || gp == 4) && op != TRV_OP_COPY) continue;
                        cands.push_back({tb, bps, gp, cpath});
                    }
        float best = -1.f;
        std::tuple<int, int, int, int> pick{0, 0, 0, 0};
        uint64_t bytes = 0;
        for (const auto& c : cands) {
            const int gp = std::get<2>(c);
            trv_batch_options o{std::get<0>(c), std::get<3>(c), 0, std::get<1>(c), op == TRV_OP_GATHER ? gp : 0,
                                op == TRV_OP_SCATTER ? gp : 0};
            trv_batch* b = nullptr;
            int rc = trv_batch_create(kv.second.data(), kv.second.size(), &o, &b);
            if (rc != TRV_OK) return rc;
            trv_batch_info(b, nullptr, &bytes);
            const float ms = time_ms([&]() -> int { return trv_batch_launch(b, stream); }, st, flush);
            trv_batch_destroy(b);
            if (ms > 0.f && (best < 0.f || ms < best)) {
                best = ms;
                pick = c;
            }
        }
        if (best < 0.f) return TRV_ERR_CUDA;
        TuneChoice ch;
        ch.tile_bytes = std::get<0>(pick);
        ch.grid = std::get<1>(pick);  // blocks per SM of the batch kernel
        ch.cache_policy = std::get<2>(pick);
        ch.path = std::get<3>(pick);  // copy groups: TRV_PATH_AUTO (TMA tiles) or TRV_PATH_VECTOR
        ch.gbs = double(bytes) / (double(best) * 1e6);
        tune_store(TuneKey{SCOPE_BATCH, op, std::get<1>(kv.first), std::get<2>(kv.first)}, ch);
    }
    return TRV_OK;
}

int32_t trv_autotune_batch(const trv_task* tasks, uint64_t count, void* stream) {
    return no_throw([&] { return autotune_batch_impl(tasks, count, stream); });
}

int32_t trv_autotune_lookup(int32_t scope, int32_t op, uint32_t width, uint64_t n, trv_launch* out,
                            int32_t* tile_bytes) {
    TuneChoice c;
    if (!tune_lookup(TuneKey{scope, op, int(width), len_bucket(n)}, &c)) return TRV_ERR_NOT_FOUND;
    if (out) *out = trv_launch{c.path, c.unroll, 0, c.grid, c.chunk, c.cache_policy};
    if (tile_bytes) *tile_bytes = c.tile_bytes;
    return TRV_OK;
}

int32_t trv_autotune_clear(void) {
    std::lock_guard<std::mutex> g(g_mu);
    g_table.clear();
    return TRV_OK;
}

static int32_t autotune_save_impl(const char* path) {
    if (!path) return TRV_ERR_INVALID_ARGUMENT;
    std::string out = "[\n";
    {
        std::lock_guard<std::mutex> g(g_mu);
        bool first = true;
        for (const auto& kv : g_table) {
            char line[400];
            const TuneChoice& c = kv.second;
            std::snprintf(line, sizeof line,
                          "%s {\"scope\": %d, \"op\": %d, \"width\": %d, \"bucket\": %d, \"path\": %d, "
                          "\"unroll\": %d, \"grid\": %d, \"chunk\": %d, \"tile_bytes\": %d, \"cache_policy\": %d, "
                          "\"gbs\": %.1f}",
                          first ? "" : ",\n", std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first),
                          std::get<3>(kv.first), c.path, c.unroll, c.grid, c.chunk, c.tile_bytes, c.cache_policy, c.gbs);
            out += line;
            first = false;
        }
    }
    out += "\n]\n";
    FILE* f = std::fopen(path, "w");
    if (!f) return TRV_ERR_INVALID_ARGUMENT;
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    std::fclose(f);
    return ok ? TRV_OK : TRV_ERR_INVALID_ARGUMENT;
}

int32_t trv_autotune_save(const char* path) {
    return no_throw([&] { return autotune_save_impl(path); });
}

// Reads the format trv_autotune_save writes: one object per entry with the
// integer fields above (gbs may be fractional).  Unknown keys are ignored;
// entries missing a key field are skipped.
static int32_t autotune_load_impl(const char* path) {
    if (!path) return TRV_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "r");
    if (!f) return TRV_ERR_NOT_FOUND;
    std::string text;
    char buf[4096];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
    std::fclose(f);
    size_t pos = 0;
    int loaded = 0;
    while ((pos = text.find('{', pos)) != std::string::npos) {
        const size_t end = text.find('}', pos);
        if (end == std::string::npos) return TRV_ERR_INVALID_ARGUMENT;
        const std::string obj = text.substr(pos, end - pos);
        auto field = [&](const char* name, double* v) -> bool {
            const std::string key = std::string("\"") + name + "\"";
            const size_t k = obj.find(key);
            if (k == std::string::npos) return false;
            const size_t colon = obj.find(':', k + key.size());
            if (colon == std::string::npos) return false;
            char* endp = nullptr;
            *v = std::strtod(obj.c_str() + colon + 1, &endp);
            return endp != obj.c_str() + colon + 1;
        };
        double scope, op, width, bucket, v;
        if (field("scope", &scope) && field("op", &op) && field("width", &width) && field("bucket", &bucket)) {
            TuneChoice c;
            if (field("path", &v)) c.path = int(v);
            if (field("unroll", &v)) c.unroll = int(v);
            if (field("grid", &v)) c.grid = int(v);
            if (field("chunk", &v)) c.chunk = int(v);
            if (field("tile_bytes", &v)) c.tile_bytes = int(v);
            if (field("cache_policy", &v)) c.cache_policy = int(v);
            if (field("gbs", &v)) c.gbs = v;
            tune_store(TuneKey{int(scope), int(op), int(width), int(bucket)}, c);
            ++loaded;
        }
        pos = end + 1;
    }
    return loaded > 0 || text.find('[') != std::string::npos ? TRV_OK : TRV_ERR_INVALID_ARGUMENT;
}

int32_t trv_autotune_load(const char* path) {
    return no_throw([&] { return autotune_load_impl(path); });
}

}  // extern "C"
