// Autotuner cache: launch choices per (scope, op, width, length bucket),
// filled by timing candidates on the GPU (autotune.cu) and persisted as JSON.
#pragma once

#include <cstdint>

namespace trv {

enum TuneScope { SCOPE_CALL = 0, SCOPE_BATCH = 1 };

struct TuneKey {
    int scope;   // TuneScope
    int op;      // TRV_OP_*
    int width;   // bytes
    int bucket;  // len_bucket(n)
};

struct TuneChoice {
    int path = 0;
    int unroll = 0;
    int grid = 0;
    int chunk = 0;
    int tile_bytes = 0;
    int cache_policy = 0;
    double gbs = 0.0;  // measured when chosen
};

// Length buckets of a factor 4: floor(log2(max(n, 1)) / 2).
int len_bucket(uint64_t n);
bool tune_lookup(const TuneKey& key, TuneChoice* out);
void tune_store(const TuneKey& key, const TuneChoice& choice);

}  // namespace trv
