// colo_host.h -- host-side structures of libcolo (datasets, results, I/O).
#pragma once
#include <stdint.h>

#include <functional>
#include <string>
#include <vector>

#include "colo.h"
#include "colo_internal.h"

namespace colo {

// Points as read from a CSV or given by the caller (raw feature ids).
struct HostPoints {
    std::vector<float> x, y;
    std::vector<int32_t> raw;
    // the id token as written, at every point whose id differs from the
    // previous point's (the feature names, colocationFinder.cpp:168-184)
    std::vector<std::pair<uint64_t, std::string>> tokens;
    bool tokens_complete = false;   // tokens hold every group start (file readers)
    float bounds[4] = {0, 0, 0, 0};
    void clear() {
        x.clear();
        y.clear();
        raw.clear();
        tokens.clear();
        tokens_complete = false;
    }
};

// Per-level trace of one job (features are global batch indices; f0 is the
// job's first feature so cand - f0 is the feature index inside the job).
struct LevelTrace {
    uint32_t k = 0;
    uint32_t f0 = 0;
    std::vector<uint32_t> cand;
    std::vector<uint64_t> ub, num, rows;
    std::vector<uint8_t> pass, prevalent;
    std::vector<float> pi;
    std::vector<uint32_t> argmin;
    std::vector<uint64_t> fquads, fcells;       // filter: full quads, cells of U_c (k >= 3)
    std::vector<float> feat;                    // cost-model features, 24 per candidate
    std::vector<float> pred;                    // LEARNED: predicted log1p(rows) per candidate
    std::vector<std::vector<uint32_t>> tables;   // row-major, kept on request
    std::vector<uint8_t> has_table;
};

// counters[]: the list in include/colo.h (colo_result_counters).
constexpr int kNumCounters = 25;
struct MineResult {
    std::vector<LevelTrace> levels;
    double times[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint64_t counters[kNumCounters] = {};
    std::vector<KernelStat> kernels;   // per-kernel CUDA-event timing (when requested)
};

struct BatchStorage;   // owned device copies for multi-job batches

colo_status read_params_file(const char* path, colo_params* p, std::string& err);
colo_status read_config_file(const char* path, std::string out[5], std::string& err);
// threads = 0: one per hardware thread, fewer for small files
colo_status parse_points_csv(const char* path, HostPoints& hp, std::string& err, unsigned threads = 0);
colo_status write_points_binary(const HostPoints& hp, const std::vector<std::string>& names, const char* path,
                                std::string& err);
colo_status read_points_binary(const char* path, HostPoints& hp, std::string& err);
// The CSV parsed on the device (colo_ingest.cu): hp as parse_points_csv fills
// it, and the coordinates' device copies in dx, dy.
colo_status parse_points_csv_device(cudaStream_t s, const char* path, HostPoints& hp, DevBuf<float>& dx,
                                    DevBuf<float>& dy, std::string& err);
colo_status write_points_csv(const HostPoints& hp, const std::vector<std::string>& names,
                             const std::vector<uint32_t>& fstart, const std::vector<uint32_t>& fcount, const char* path,
                             std::string& err);
// Positions where the raw id changes (0 first), found in parallel; *minus_one
// is set when some id is -1.
std::vector<uint64_t> group_starts(const int32_t* raw, uint64_t n, bool* minus_one);
colo_status write_patterns(const MineResult& r, const std::vector<std::string>& names,
                           const char* location, std::string& err);

}  // namespace colo

// ---------------------------------------------------------------------------
// Opaque C-ABI objects
// ---------------------------------------------------------------------------
struct colo_ctx {
    int device = 0;
    cudaStream_t s = nullptr;
    int sms = 0;
    std::string err;
    int refs = 1;          // the owner plus one per live dataset (freed at zero)
    std::vector<float> model;   // cost-model parameters for LEARNED mines (empty: none)
    int join_group = 0;         // lanes per anchor in the join (0: default; set by colo_autotune)
    int filter_unit = 0;        // candidates per warp unit in the level filter (0: default 32)
    int level_block = 0;        // threads per block of the level kernels (0: default 256)
    int level_queue = 0;        // 1: level count/fill kernels as a persistent work queue
    void* stage = nullptr;      // page-locked staging for the level loop's readbacks
    size_t stage_bytes = 0;
    cudaStream_t s2 = nullptr;  // side stream: the fill's slot scan runs there during the host's level work
    cudaEvent_t ev_counted = nullptr, ev_scanned = nullptr;
    void* ustage = nullptr;     // page-locked staging for the level loop's uploads
    size_t ustage_bytes = 0;
    size_t ustage_off = 0;      // bytes in use since the stream last drained
    uint64_t pool_peak = 0;     // most device-pool memory in use by one earlier mine (bytes)
};

struct colo_dataset {
    colo_ctx* ctx = nullptr;
    colo::HostPoints hp;
    std::vector<std::string> names;
    std::vector<uint32_t> fstart, fcount;
    colo::DevBuf<float> dx, dy;
    bool resident = false;
    bool pinned = false;                     // page-locking of the host arrays was attempted
    const float* mx = nullptr;               // device addresses of the page-locked, mapped host
    const float* my = nullptr;               //   arrays (null when locking or mapping failed)
};

struct colo_result {
    colo::MineResult r;
};

namespace colo {
struct Batch;
void candidate_features(uint32_t k, const uint32_t* mem, const uint32_t* fcount, const uint64_t* ub,
                        uint64_t prow, uint64_t fquads, uint64_t fcells, float* x);
colo_status set_err(colo_ctx* ctx, colo_status st, const std::string& msg);
void ctx_release(colo_ctx* ctx);
colo_status run_guarded(colo_ctx* ctx, const std::function<colo_status()>& fn);
uint64_t upload_dataset(colo_dataset* ds, cudaStream_t s);   // bytes copied (0 when resident)
// Points, features, job grids and the bucketed/joined device state of a batch.
// `own` keeps the concatenated device copies of multi-job batches alive.
void setup_batch(colo_ctx* ctx, colo_dataset* const* dsv, const colo_params* pv, uint32_t J, Batch& b,
                 std::vector<DevBuf<float>>& ownf, double* t_upload);
}  // namespace colo
