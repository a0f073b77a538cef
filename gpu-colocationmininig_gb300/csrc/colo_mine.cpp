// colo_mine.cpp -- the C ABI and the level loop (host orchestration).
//
// The level loop follows Begin (colocationFinder.cpp:1068-1147): degree 2
// (degree2Processing, 256-425), then per level the filter, refinement with
// participation index (generatePrevalentPatternsGeneral, 736-854), Apriori
// candidate generation (candidateColocationGeneral, 517-557) and instance
// tables for the prevalent patterns that prefix a next-level candidate
// (calcInstanceTablePatternIndexes + generateInstanceTableGeneral, 1042-1066,
// 856-909).  Instance tables stay in device memory between levels.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "colo_batch.h"
#include "colo_host.h"
#include "colo_mlp.h"

using namespace colo;

namespace colo {
namespace {

using Clock = std::chrono::steady_clock;
inline double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

template <class Fn>
colo_status guarded(colo_ctx* ctx, Fn&& fn) {
    return run_guarded(ctx, std::function<colo_status()>(fn));
}

// Feature grouping of populateData (colocationFinder.cpp:168-229): a change of
// raw id starts a new feature, named by the id token as written.  The file
// readers record the token of every group start; host arrays have none, and
// their features are named by the id's decimal form.
void group_features(colo_dataset* ds) {
    const HostPoints& hp = ds->hp;
    const uint64_t n = hp.x.size();
    ds->names.clear();
    ds->fstart.clear();
    ds->fcount.clear();
    if (hp.tokens_complete) {
        for (const auto& t : hp.tokens) {
            ds->names.push_back(t.second);
            ds->fstart.push_back((uint32_t)t.first);
        }
    } else {
        bool minus_one = false;
        for (uint64_t i : group_starts(hp.raw.data(), n, &minus_one)) {
            ds->names.push_back(std::to_string(hp.raw[i]));
            ds->fstart.push_back((uint32_t)i);
        }
    }
    ds->fcount.resize(ds->fstart.size());
    for (size_t f = 0; f < ds->fstart.size(); ++f)
        ds->fcount[f] = (f + 1 < ds->fstart.size() ? ds->fstart[f + 1] : (uint32_t)n) - ds->fstart[f];
}

// setGrid (colocationFinder.cpp:102-126).
JobGrid make_grid(const float bounds[4], float R, float thr) {
    JobGrid g{};
    g.min_x = bounds[0];
    g.min_y = bounds[1];
    float maxX = bounds[2];
    float maxYe = bounds[3] + R;
    g.w = R;
    float gsx = (maxX - g.min_x) / g.w;
    float gsy = (maxYe - g.min_y) / g.w;
    if (!(R > 0.0f) || !std::isfinite(R) || !std::isfinite(gsx) || !std::isfinite(gsy))
        throw StatusError{COLO_ERR_INPUT, "grid: distance and bounds must be finite with R > 0"};
    float cx = std::ceil(gsx), cy = std::ceil(gsy);
    if (!(cx >= 1.0f) || !(cy >= 1.0f) || cx >= 4294967296.0f || cy >= 4294967296.0f)
        throw StatusError{COLO_ERR_INPUT, "grid: the bounds line gives an empty or oversized grid"};
    g.gx = (uint32_t)cx;
    g.gy = (uint32_t)cy;
    g.total = (uint64_t)g.gx * g.gy;
    g.compat32 = (g.total + g.gx) < (1ull << 31) ? 1 : 0;
    g.R2 = R * R;
    g.R2hu = (std::nextafter(g.R2, INFINITY) - g.R2) * 0.5f;
    g.thr = thr;
    return g;
}

}  // namespace

colo_status set_err(colo_ctx* ctx, colo_status st, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return st;
}

// Datasets keep their context alive: callers may free a context before its
// datasets (garbage-collected bindings do), and a dataset frees its device
// buffers on the context's stream.
void ctx_release(colo_ctx* ctx) {
    if (--ctx->refs > 0) return;
    if (ctx->s) {
        cudaStreamSynchronize(ctx->s);
        cudaStreamDestroy(ctx->s);
    }
    if (ctx->s2) {
        cudaStreamSynchronize(ctx->s2);
        cudaStreamDestroy(ctx->s2);
    }
    if (ctx->ev_counted) cudaEventDestroy(ctx->ev_counted);
    if (ctx->ev_scanned) cudaEventDestroy(ctx->ev_scanned);
    if (ctx->stage) cudaFreeHost(ctx->stage);
    if (ctx->ustage) cudaFreeHost(ctx->ustage);
    delete ctx;
}

colo_status run_guarded(colo_ctx* ctx, const std::function<colo_status()>& fn) {
    try {
        return fn();
    } catch (const StatusError& e) {
        return set_err(ctx, e.st, e.msg);
    } catch (const CudaError& e) {
        cudaGetLastError();
        return set_err(ctx, COLO_ERR_CUDA, std::string(cudaGetErrorString(e.err)) + " in " + e.where);
    } catch (const std::bad_alloc&) {
        return set_err(ctx, COLO_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return set_err(ctx, COLO_ERR_INTERNAL, e.what());
    }
}

// Page-locks the host coordinate arrays once (uploads are then direct DMA)
// and maps them, so that kernels can also read them over the host link.
void pin_dataset(colo_dataset* ds) {
    const uint64_t n = ds->hp.x.size();
    if (ds->pinned || !n) return;
    ds->pinned = true;
    bool ok = cudaHostRegister(ds->hp.x.data(), n * 4, cudaHostRegisterMapped) == cudaSuccess;
    ok = ok && cudaHostRegister(ds->hp.y.data(), n * 4, cudaHostRegisterMapped) == cudaSuccess;
    void* px = nullptr;
    void* py = nullptr;
    ok = ok && cudaHostGetDevicePointer(&px, ds->hp.x.data(), 0) == cudaSuccess;
    ok = ok && cudaHostGetDevicePointer(&py, ds->hp.y.data(), 0) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return;
    }
    ds->mx = static_cast<const float*>(px);
    ds->my = static_cast<const float*>(py);
}

uint64_t upload_dataset(colo_dataset* ds, cudaStream_t s) {
    if (ds->resident) return 0;
    uint64_t n = ds->hp.x.size();
    pin_dataset(ds);
    // coordinates only: a point's feature follows from the feature start table
    // (points are grouped by feature), so no per-point feature array is copied
    ds->dx.alloc(n, s);
    ds->dy.alloc(n, s);
    if (n) {
        COLO_CUDA(cudaMemcpyAsync(ds->dx.get(), ds->hp.x.data(), n * 4, cudaMemcpyHostToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(ds->dy.get(), ds->hp.y.data(), n * 4, cudaMemcpyHostToDevice, s));
    }
    stream_wait(s);
    ds->resident = true;
    return 8 * n;   // bytes copied
}

namespace {

struct PatternHash {
    size_t operator()(const std::vector<uint32_t>& v) const {
        uint64_t h = 1469598103934665603ull;
        for (uint32_t x : v) h = (h ^ x) * 1099511628211ull;
        return (size_t)h;
    }
};

struct TableRef {
    uint32_t* cols = nullptr;   // column-major
    uint64_t rows = 0;
    uint64_t stride = 0;
};

struct JobState {
    uint32_t f0 = 0, nf = 0;
    float thr = 0;
    uint32_t max_size = 0;
    bool active = true;
    std::vector<uint32_t> cands;     // this level's candidates (global features)
    std::vector<uint32_t> parent;    // per candidate: index of its (k-1)-prefix among the previous level's candidates
    std::vector<TableRef> prev_tables;   // per previous-level candidate: its instance table (rows 0 if none)
    MineResult* out = nullptr;
};

// Apriori join (candidateColocationGeneral, colocationFinder.cpp:517-557):
// patterns i < j with equal (k-2)-prefix are joined; the remaining
// (k-1)-subsets must all be prevalent (generateandCheckSubsets, 669-679);
// a failing subset check ends the inner loop ("break", 541-542) and so does
// a prefix mismatch (551-552).
// Prevalent patterns of a level (all jobs) above which the next level's
// candidates are generated on the device (apriori_device); below it the host
// loop is faster than the launches and copies.
constexpr uint64_t kDeviceAprioriMin = 4096;
// Prevalent tables up to this many words (1 GiB) are filled before Apriori decides which
// of them the next level needs, so that the host's Apriori overlaps the fill.
constexpr uint64_t kEarlyFillWords = 1ull << 28;

std::vector<uint32_t> apriori_next(const std::vector<uint32_t>& prev, uint32_t km1, std::vector<uint32_t>& parent) {
    std::vector<uint32_t> out;
    parent.clear();
    size_t P = prev.size() / km1;
    if (P < 2) return out;
    std::unordered_set<std::vector<uint32_t>, PatternHash> have;
    have.reserve(P * 2);
    for (size_t i = 0; i < P; ++i) have.emplace(prev.begin() + i * km1, prev.begin() + (i + 1) * km1);
    const uint32_t k = km1 + 1;
    std::vector<uint32_t> cand(k), sub(km1);
    for (size_t i = 0; i < P; ++i) {
        const uint32_t* pi = &prev[i * km1];
        for (size_t j = i + 1; j < P; ++j) {
            const uint32_t* pj = &prev[j * km1];
            bool same = true;
            for (uint32_t t = 0; t + 1 < km1; ++t)
                if (pi[t] != pj[t]) {
                    same = false;
                    break;
                }
            if (!same || !(pi[km1 - 1] < pj[km1 - 1])) break;
            for (uint32_t t = 0; t < km1; ++t) cand[t] = pi[t];
            cand[km1] = pj[km1 - 1];
            // subsets dropping positions k-3 .. 0 (the two others are pi and pj)
            bool ok = true;
            for (int drop = (int)k - 3; drop >= 0 && ok; --drop) {
                uint32_t q = 0;
                for (uint32_t t = 0; t < k; ++t)
                    if ((int)t != drop) sub[q++] = cand[t];
                if (!have.count(sub)) ok = false;
            }
            if (!ok) break;
            out.insert(out.end(), cand.begin(), cand.end());
            parent.push_back((uint32_t)i);   // its (k-1)-prefix is prev pattern i
        }
    }
    return out;
}

// threshold_Kernel arithmetic (Codes/DeviceProcess_Kernel.h:545-573).
bool filter_pass(const uint64_t* ub, const uint32_t* mem, uint32_t k, const std::vector<uint32_t>& fcount,
                 float thr) {
    float pi0 = 1.0f;
    for (uint32_t j = 0; j < k; ++j) {
        float pr = (float)((double)ub[j] / (double)(float)fcount[mem[j]]);
        if (j == 0) pi0 = pr;
        else if (pi0 > pr) pi0 = pr;
    }
    return pi0 >= thr;
}

// Readbacks staged in page-locked memory: a device-to-host copy into pageable
// memory blocks the host until the stream reaches it, one into the context's
// pinned buffer is only queued, so one wait covers all of a phase's copies and
// finish() then moves the bytes to their destinations.  The buffer grows only
// here, after the stream has drained.
struct Readback {
    colo_ctx* ctx;
    cudaStream_t s;
    struct Item {
        void* dst;
        size_t off, bytes;
    };
    std::vector<Item> items;
    size_t off = 0;
    Readback(colo_ctx* c, cudaStream_t st, size_t need) : ctx(c), s(st) {
        need += 64 * 16;   // 16-byte alignment of each copy
        if (need > ctx->stage_bytes) {
            stream_wait(s);
            if (ctx->stage) cudaFreeHost(ctx->stage);
            ctx->stage = nullptr;
            ctx->stage_bytes = 0;
            const size_t nb = std::max<size_t>(need, (size_t)1 << 20);
            COLO_CUDA(cudaHostAlloc(&ctx->stage, nb, cudaHostAllocDefault));
            ctx->stage_bytes = nb;
        }
    }
    void copy(void* dst, const void* src, size_t bytes) {
        if (!bytes) return;
        off = (off + 15) & ~(size_t)15;
        if (off + bytes > ctx->stage_bytes) throw StatusError{COLO_ERR_INTERNAL, "readback staging too small"};
        COLO_CUDA(cudaMemcpyAsync(static_cast<char*>(ctx->stage) + off, src, bytes, cudaMemcpyDeviceToHost, s));
        items.push_back({dst, off, bytes});
        off += bytes;
    }
    void finish() {
        stream_wait(s);
        for (const Item& it : items) std::memcpy(it.dst, static_cast<char*>(ctx->stage) + it.off, it.bytes);
        items.clear();
        off = 0;
        ctx->ustage_off = 0;   // the stream has drained: every upload staged so far has landed
    }
};

// Host-to-device copies of the level loop through page-locked staging: the
// bytes are copied into ctx->ustage and the DMA is queued from there, so the
// call does not wait as a copy from pageable memory does.  The staging space is
// reused after the next Readback::finish (the stream has drained by then); it
// grows, after a drain, when a copy does not fit.
// Space for `bytes` in the upload staging; the caller writes its data there and
// queues the copy with upload_from.
unsigned char* upload_area(colo_ctx* ctx, cudaStream_t s, size_t bytes) {
    size_t off = (ctx->ustage_off + 15) & ~(size_t)15;
    if (off + bytes > ctx->ustage_bytes) {
        stream_wait(s);
        off = 0;
        if (bytes > ctx->ustage_bytes) {
            if (ctx->ustage) cudaFreeHost(ctx->ustage);
            ctx->ustage = nullptr;
            ctx->ustage_bytes = 0;
            const size_t nb = std::max<size_t>(bytes * 2, (size_t)1 << 20);
            COLO_CUDA(cudaHostAlloc(&ctx->ustage, nb, cudaHostAllocDefault));
            ctx->ustage_bytes = nb;
        }
    }
    ctx->ustage_off = off + bytes;
    return static_cast<unsigned char*>(ctx->ustage) + off;
}

void upload_from(cudaStream_t s, void* dst, const unsigned char* staged, size_t bytes) {
    if (bytes) COLO_CUDA(cudaMemcpyAsync(dst, staged, bytes, cudaMemcpyHostToDevice, s));
}

void upload(colo_ctx* ctx, cudaStream_t s, void* dst, const void* src, size_t bytes) {
    if (!bytes) return;
    unsigned char* h = upload_area(ctx, s, bytes);
    std::memcpy(h, src, bytes);
    upload_from(s, dst, h, bytes);
}

// A typed view into the level arena's one allocation.
template <class T>
struct ArenaSpan {
    T* p = nullptr;
    T* get() const { return p; }
};

// The refinement's per-level device buffers, carved from one stream-ordered
// allocation with the zero-initialised ones (bitmap, rows, chunk status, overflow)
// adjacent, so that a level costs one allocation, one clear and one free
// instead of nine, four and nine.  Parts start on 256-byte boundaries.
struct LevelArena {
    DevBuf<unsigned char> mem;
    ArenaSpan<uint32_t> bitmap;
    ArenaSpan<unsigned long long> rows;
    ArenaSpan<unsigned long long> items;    // candidate-slice entries examined (work counter)
    ArenaSpan<unsigned long long> status;   // single pass: per chunk look-back word, then the chunk ticket
    ArenaSpan<unsigned long long> tickets;  // chunk tickets of the count and fill launches (persistent queue)
    ArenaSpan<uint32_t> overflow;           // single pass: 1 when the table outgrew its capacity
    ArenaSpan<uint32_t> slots;
    ArenaSpan<CandDesc> descs;
    ArenaSpan<uint64_t> chunk_off;
    ArenaSpan<uint64_t> stats;
    // the refine's results (rows | items | overflow | stats) and inputs (descs | chunk
    // prefixes) are each one contiguous block: one copy back, one copy in
    size_t out_bytes = 0, in_bytes = 0, chunk_at = 0;
    unsigned char* out = nullptr;
    unsigned char* in = nullptr;

    void init(uint64_t nslots, uint64_t nwords, uint64_t ncand, uint64_t nchunks, uint32_t k, bool single,
              cudaStream_t s) {
        size_t off = 0;
        auto take = [&](uint64_t bytes) {
            const size_t o = off;
            off += (size_t)((bytes + 255) & ~(uint64_t)255);
            return o;
        };
        const size_t r_items = ncand * 8, r_ovf = r_items + 8, r_stats = (r_ovf + ncand * 4 + 15) & ~(size_t)15;
        out_bytes = r_stats + ncand * k * 4 * 8;
        const size_t o_out = take(out_bytes);
        const size_t o_status = single ? take((nchunks + 1) * 8) : 0;
        const size_t o_tickets = take(2 * 8);
        const size_t o_bitmap = take(std::max<uint64_t>(nwords, 1) * 4);
        const size_t zeroed = off;
        const size_t o_slots = take(std::max<uint64_t>(nslots, 1) * 4);
        chunk_at = (std::max<uint64_t>(ncand, 1) * sizeof(CandDesc) + 15) & ~(size_t)15;
        in_bytes = chunk_at + (ncand + 2) * 8;
        const size_t o_in = take(in_bytes);
        mem.alloc(off, s);
        unsigned char* b = mem.get();
        out = b + o_out;
        in = b + o_in;
        rows.p = reinterpret_cast<unsigned long long*>(out);
        items.p = reinterpret_cast<unsigned long long*>(out + r_items);
        overflow.p = reinterpret_cast<uint32_t*>(out + r_ovf);
        stats.p = reinterpret_cast<uint64_t*>(out + r_stats);
        status.p = single ? reinterpret_cast<unsigned long long*>(b + o_status) : nullptr;
        tickets.p = reinterpret_cast<unsigned long long*>(b + o_tickets);
        bitmap.p = reinterpret_cast<uint32_t*>(b + o_bitmap);
        slots.p = reinterpret_cast<uint32_t*>(b + o_slots);
        descs.p = reinterpret_cast<CandDesc*>(in);
        chunk_off.p = reinterpret_cast<uint64_t*>(in + chunk_at);
        COLO_CUDA(cudaMemsetAsync(b, 0, zeroed, s));
    }
    // descs and chunk prefixes in one upload
    void put_inputs(colo_ctx* ctx, cudaStream_t s, const std::vector<CandDesc>& hd, const std::vector<uint64_t>& ch) {
        unsigned char* h = upload_area(ctx, s, in_bytes);
        std::memcpy(h, hd.data(), hd.size() * sizeof(CandDesc));
        std::memcpy(h + chunk_at, ch.data(), std::min<size_t>(ch.size() * 8, in_bytes - chunk_at));
        upload_from(s, in, h, in_bytes);
    }
};

// Tables presized at fewer rows than this are counted and, when needed, filled
// after the next level's candidates are known instead of written while counted.
constexpr uint64_t kSinglePassMinRows = 1u << 20;

// Capacity of a presized single-pass table from the predicted log1p(rows).
uint64_t presize_rows(float pred) {
    double r = std::expm1(std::min<double>(pred, 40.0));
    if (!(r > 0)) r = 0;
    return (uint64_t)std::ceil(r * 1.5) + 32;
}

}  // namespace

// ---------------------------------------------------------------------------
// The mining driver for a batch of jobs.
// ---------------------------------------------------------------------------
void setup_batch(colo_ctx* ctx, colo_dataset* const* dsv, const colo_params* pv, uint32_t J, Batch& b,
                 std::vector<DevBuf<float>>& ownf, double* t_upload) {
    cudaStream_t s = ctx->s;
    b.s = s;
    b.sms = ctx->sms;
    b.J = J;
    if (ctx->join_group) b.join_group = ctx->join_group;
    if (ctx->filter_unit) b.filter_unit = ctx->filter_unit;
    if (ctx->level_block) b.level_block = ctx->level_block;
    b.level_queue = ctx->level_queue > 0 ? 1 : 0;
    b.test_spin = pv[0].reserved[1] > 0 ? (uint32_t)pv[0].reserved[1] : 0u;
    auto t0 = Clock::now();
    std::vector<uint32_t> job_f0(J + 1, 0);
    uint64_t N = 0;
    for (uint32_t j = 0; j < J; ++j) {
        job_f0[j + 1] = job_f0[j] + (uint32_t)dsv[j]->names.size();
        N += dsv[j]->hp.x.size();
    }
    if (N >= (1ull << 32) - 1) throw StatusError{COLO_ERR_CAPACITY, "at most 2^32-2 points per batch"};
    b.N = N;
    b.F = job_f0[J];
    if (J == 1) {
        colo_dataset* ds = dsv[0];
        if (!ds->resident) pin_dataset(ds);
        if (!ds->resident && ds->mx && ds->my) {
            // streamed: the cell-key pass reads the page-locked host arrays over
            // the host link (the only pass that reads them: it writes the packed
            // device copy every later pass uses), so no separate upload runs
            b.x = ds->mx;
            b.y = ds->my;
            b.h2d_points = 8 * N;
        } else {
            b.h2d_points = upload_dataset(ds, s);
            b.x = ds->dx.get();
            b.y = ds->dy.get();
        }
    } else {
        ownf.resize(2);
        ownf[0].alloc(N, s);
        ownf[1].alloc(N, s);
        uint64_t off = 0;
        for (uint32_t j = 0; j < J; ++j) {
            colo_dataset* ds = dsv[j];
            uint64_t n = ds->hp.x.size();
            if (!n) continue;
            COLO_CUDA(cudaMemcpyAsync(ownf[0].get() + off, ds->hp.x.data(), n * 4, cudaMemcpyHostToDevice, s));
            COLO_CUDA(cudaMemcpyAsync(ownf[1].get() + off, ds->hp.y.data(), n * 4, cudaMemcpyHostToDevice, s));
            off += n;
        }
        stream_wait(s);
        b.h2d_points = 8 * N;
        b.x = ownf[0].get();
        b.y = ownf[1].get();
    }
    if (t_upload) *t_upload = ms_since(t0);
    b.h_fstart.resize(b.F);
    b.h_fcount.resize(b.F);
    b.h_fjob.resize(b.F);
    b.jobs.resize(J);
    uint64_t key_base = 0, p0 = 0, row_base = 0;
    b.Fmax_local = 1;
    for (uint32_t j = 0; j < J; ++j) {
        colo_dataset* ds = dsv[j];
        for (uint32_t f = 0; f < ds->names.size(); ++f) {
            b.h_fstart[job_f0[j] + f] = (uint32_t)(p0 + ds->fstart[f]);
            b.h_fcount[job_f0[j] + f] = ds->fcount[f];
            b.h_fjob[job_f0[j] + f] = j;
        }
        JobGrid g = make_grid(ds->hp.bounds, pv[j].distance, pv[j].pi_threshold);
        g.key_base = key_base;
        g.row_base = row_base;
        g.f0 = job_f0[j];
        g.nf = (uint32_t)ds->names.size();
        key_base += g.total;
        row_base += g.gy;
        b.jobs[j].grid = g;
        b.jobs[j].p0 = p0;
        b.jobs[j].np = ds->hp.x.size();
        p0 += ds->hp.x.size();
        b.Fmax_local = std::max(b.Fmax_local, g.nf);
    }
    // mask words per cell: 1..8, else padded to 12, 16, 24 or 32 (the widths
    // the mask kernels are built for; up to 1024 features per job)
    b.W = (b.Fmax_local + 31) / 32;
    if (b.W > 8) b.W = b.W <= 12 ? 12 : b.W <= 16 ? 16 : b.W <= 24 ? 24 : b.W <= 32 ? 32 : b.W;
    b.key_bits = 1;
    while (b.key_bits < 64 && (1ull << b.key_bits) < key_base) b.key_bits++;
    b.rows = row_base;
    b.fstart.alloc(b.F ? b.F : 1, s);
    b.fcount.alloc(b.F ? b.F : 1, s);
    b.fjob.alloc(b.F ? b.F : 1, s);
    b.grids.alloc(J, s);
    b.flags.alloc(1, s);
    b.flags.zero(s);
    std::vector<JobGrid> hg(J);
    for (uint32_t j = 0; j < J; ++j) hg[j] = b.jobs[j].grid;
    if (b.F) {
        COLO_CUDA(cudaMemcpyAsync(b.fstart.get(), b.h_fstart.data(), b.F * 4, cudaMemcpyHostToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(b.fcount.get(), b.h_fcount.data(), b.F * 4, cudaMemcpyHostToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(b.fjob.get(), b.h_fjob.data(), b.F * 4, cudaMemcpyHostToDevice, s));
    }
    // (copies from pageable memory return once the source is staged: no wait is needed)
    COLO_CUDA(cudaMemcpyAsync(b.grids.get(), hg.data(), J * sizeof(JobGrid), cudaMemcpyHostToDevice, s));
}

// The stream-ordered pool keeps what it has mapped (its release threshold is
// "everything"), but a mine whose blocks come and go in a different order than
// the last one's may find no free block large enough and map more memory in
// the middle of a step (about a millisecond per growth on the 20M-point
// workload).  So after a mine that used more of the pool than any before it,
// the pool gets one free block of twice that peak, if the device has that
// much to spare (growing the pool by 10 GB took 4.4 ms on a GB300); later
// mines carve their blocks out of it.  The growth lands in the mine that set
// the peak (a warm-up mine, typically), not in the next one.  The pool's
// high-water mark is reset as a mine starts, so it measures that mine alone.
static cudaMemPool_t device_pool(colo_ctx* ctx) {
    cudaMemPool_t pool = nullptr;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return pool;
}

static void pool_reset_mark(colo_ctx* ctx) {
    cudaMemPool_t pool = device_pool(ctx);
    uint64_t zero = 0;
    if (pool && cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero) != cudaSuccess) cudaGetLastError();
}

static void pool_headroom(colo_ctx* ctx) {
    cudaMemPool_t pool = device_pool(ctx);
    if (!pool) return;
    uint64_t high = 0, reserved = 0;
    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &high) != cudaSuccess ||
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    if (high <= ctx->pool_peak) return;   // no new peak (one attempt per peak, whatever its outcome)
    ctx->pool_peak = high;
    size_t free_b = 0, total_b = 0;
    if (reserved >= 2 * high || cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    void* p = nullptr;
    if (2 * high <= free_b / 2 && cudaMallocAsync(&p, 2 * high, ctx->s) == cudaSuccess) {   // most stays free
        cudaFreeAsync(p, ctx->s);
        cudaStreamSynchronize(ctx->s);
    }
    cudaGetLastError();
}

static void mine_jobs(colo_ctx* ctx, colo_dataset* const* dsv, const colo_params* pv, uint32_t J,
                      MineResult** outs) {
    cudaStream_t s = ctx->s;
    const auto t_all = Clock::now();
    g_launches = 0;
    KTimer kt;
    kt.s = s;
    kt.on = (pv[0].reserved[0] & 1) != 0;
    g_ktimer = &kt;
    struct Unset {
        ~Unset() { g_ktimer = nullptr; }
    } unset;
    uint64_t cnt_items = 0, cnt_parent = 0, cnt_fillw = 0, cnt_bmw = 0, cnt_d2h = 0, cnt_refined = 0, cnt_fcm = 0;
    uint64_t cnt_single = 0, cnt_single_ovf = 0, cnt_fquads = 0, cnt_fcells = 0;
    uint64_t us_pairs_model = 0, us_level_wait = 0;
    Batch b;
    const int mode = pv[0].mode;
    const bool plain = (mode == COLO_MODE_PLAIN);
    std::vector<DevBuf<float>> ownf;
    double t_upload = 0;
    setup_batch(ctx, dsv, pv, J, b, ownf, &t_upload);
    const uint64_t N = b.N;
    std::vector<JobState> js(J);
    for (uint32_t j = 0; j < J; ++j) {
        const JobGrid& g = b.jobs[j].grid;
        js[j].f0 = g.f0;
        js[j].nf = g.nf;
        js[j].thr = pv[j].pi_threshold;
        js[j].max_size = pv[j].max_size;
        js[j].out = outs[j];
        js[j].active = g.nf >= 2 && b.jobs[j].np > 0;
    }
    auto t0 = Clock::now();

    // ---- bucketing + join ---------------------------------------------------
    if (N > 0) {
        bucket_points(b);
        build_neighborhoods(b);
    }
    double t_bucket = ms_since(t0);
    t0 = Clock::now();
    if (N > 0) join_neighbors(b);
    double t_join = ms_since(t0);   // host time: the level loop's first wait absorbs the join's tail

    double t_filter = 0, t_refine = 0, t_fill = 0, t_apriori = 0;
    uint64_t rows_written = 0;

    // ---- level loop -----------------------------------------------------------
    for (uint32_t j = 0; j < J; ++j) {
        if (!js[j].active) continue;
        for (uint32_t a = 0; a + 1 < js[j].nf; ++a)          // colocationFinder.cpp:75-82
            for (uint32_t c = a + 1; c < js[j].nf; ++c) {
                js[j].cands.push_back(js[j].f0 + a);
                js[j].cands.push_back(js[j].f0 + c);
            }
    }
    std::unique_ptr<TableBuf> tables_prev, tables_cur, single_prev;
    // level tables go to pinned host memory when forced (reserved[0] bit 3)
    // or when their device allocation fails
    bool host_tables = false;
    for (uint32_t j = 0; j < J; ++j) host_tables |= (pv[j].reserved[0] & 8) != 0;
    uint64_t cnt_host_table_bytes = 0;
    for (uint32_t k = 2;; ++k) {
        bool any = false;
        for (auto& st : js) any |= (st.active && !st.cands.empty());
        if (!any) break;
        if (k > (uint32_t)kMaxK)
            throw StatusError{COLO_ERR_CAPACITY, "patterns larger than 32 features are not supported"};
        // ---- filter ----
        t0 = Clock::now();
        std::vector<LevelTrace*> tr(J, nullptr);
        for (uint32_t j = 0; j < J; ++j) {
            if (!js[j].active || js[j].cands.empty()) continue;
            js[j].out->levels.emplace_back();
            LevelTrace& L = js[j].out->levels.back();
            L.k = k;
            L.f0 = js[j].f0;
            L.cand = js[j].cands;
            size_t C = L.cand.size() / k;
            L.ub.assign(C * k, 0);
            L.num.assign(C * k, 0);
            L.rows.assign(C, 0);
            L.pass.assign(C, 0);
            L.prevalent.assign(C, 0);
            L.pi.assign(C, -1.0f);
            L.argmin.assign(C, 0);
            L.fquads.assign(C, 0);
            L.fcells.assign(C, 0);
            L.has_table.assign(C, 0);
            tr[j] = &L;
        }
        const bool learned_mode = mode == COLO_MODE_LEARNED && !ctx->model.empty();
        bool force_single_any = false;
        for (uint32_t j = 0; j < J; ++j) force_single_any |= (pv[j].reserved[0] & 16) != 0;
        if (k == 2) {
            DevBuf<uint32_t> ub2;
            std::vector<uint64_t> job_off;
            filter_pairs(b, ub2, job_off, s);
            std::vector<uint32_t> h(job_off[J]);
            if (!h.empty()) COLO_CUDA(cudaMemcpyAsync(h.data(), ub2.get(), h.size() * 4, cudaMemcpyDeviceToHost, s));
            stream_wait(s);
            for (uint32_t j = 0; j < J; ++j) {
                if (!tr[j]) continue;
                LevelTrace& L = *tr[j];
                uint32_t nf = js[j].nf;
                for (size_t c = 0; c < L.cand.size() / 2; ++c) {
                    uint32_t l0 = L.cand[2 * c] - js[j].f0, l1 = L.cand[2 * c + 1] - js[j].f0;
                    L.ub[2 * c] = h[job_off[j] + (uint64_t)l0 * nf + l1];
                    L.ub[2 * c + 1] = h[job_off[j] + (uint64_t)l1 * nf + l0];
                    L.pass[c] = filter_pass(&L.ub[2 * c], &L.cand[2 * c], 2, b.h_fcount, js[j].thr);
                }
            }
        } else {
            std::vector<uint32_t> hc, hjob;
            std::vector<std::pair<uint32_t, size_t>> owner;
            for (uint32_t j = 0; j < J; ++j) {
                if (!tr[j]) continue;
                const LevelTrace& L = *tr[j];
                for (size_t c = 0; c < L.cand.size() / k; ++c) {
                    hc.insert(hc.end(), L.cand.begin() + c * k, L.cand.begin() + (c + 1) * k);
                    hjob.push_back(j);
                    owner.push_back({j, c});
                }
            }
            uint64_t ncand = owner.size();
            bool rec_all = false;
            for (uint32_t j = 0; j < J; ++j) rec_all |= tr[j] && (pv[j].reserved[0] & 2) != 0;
            const bool infer = learned_mode && ncand > 0;
            const bool want_x = (rec_all || infer) && ncand;
            // the level's filter buffers from one allocation: the results (bounds, cell
            // statistics, predictions: zeroed, one block read back with one copy) and the
            // inputs (candidates, parent rows, model: one block written with one copy), then
            // the cost-model inputs
            size_t off = 0;
            auto take = [&](uint64_t bytes) {
                const size_t o = off;
                off += (size_t)((bytes + 15) & ~(uint64_t)15);
                return o;
            };
            const size_t o_ub = take(ncand * k * 4), o_fs = take(ncand * 2 * 8), o_y = infer ? take(ncand * 4) : 0;
            const size_t out_bytes = off;
            const size_t o_cand = take(ncand * k * 4);
            const size_t o_prow = want_x ? take(ncand * 8) : 0, o_par = infer ? take(kMlpParams * 4) : 0;
            const size_t in_end = off;
            const size_t o_x = want_x ? take(ncand * kMlpIn * 4) : 0;
            DevBuf<unsigned char> fmem;
            fmem.alloc(off ? off : 256, s);
            unsigned char* fb = fmem.get();
            uint32_t* d_ub = reinterpret_cast<uint32_t*>(fb + o_ub);
            unsigned long long* d_fs = reinterpret_cast<unsigned long long*>(fb + o_fs);
            uint32_t* d_cand = reinterpret_cast<uint32_t*>(fb + o_cand);
            if (out_bytes) COLO_CUDA(cudaMemsetAsync(fb, 0, out_bytes, s));
            {
                unsigned char* hin = upload_area(ctx, s, in_end - o_cand);
                std::memcpy(hin, hc.data(), hc.size() * 4);
                if (want_x) {
                    uint64_t* hprow = reinterpret_cast<uint64_t*>(hin + (o_prow - o_cand));
                    for (uint64_t q = 0; q < ncand; ++q) {
                        const JobState& st = js[owner[q].first];
                        hprow[q] = st.prev_tables[st.parent[owner[q].second]].rows;
                    }
                }
                if (infer) std::memcpy(hin + (o_par - o_cand), ctx->model.data(), kMlpParams * 4);
                upload_from(s, d_cand, hin, in_end - o_cand);
            }
            filter_level(b, hc.data(), hjob.data(), ncand, k, d_ub, d_fs, d_cand);
            const auto tl0 = Clock::now();
            // cost-model features and predictions on the device, read back with the bounds
            Readback rb(ctx, s, (rec_all ? ncand * kMlpIn * 4 : 0) + out_bytes);
            std::vector<float> hX, hY;
            if (want_x) {
                const uint64_t* d_prow = reinterpret_cast<const uint64_t*>(fb + o_prow);
                float* d_x = reinterpret_cast<float*>(fb + o_x);
                mlp_features(ncand, k, d_cand, d_ub, d_fs, b.fcount.get(), d_prow, d_x, s);
                if (rec_all) {
                    hX.resize(ncand * kMlpIn);
                    rb.copy(hX.data(), d_x, hX.size() * 4);
                }
                if (infer) mlp_forward(reinterpret_cast<const float*>(fb + o_par), d_x, ncand,
                                       reinterpret_cast<float*>(fb + o_y), s);
            }
            std::vector<unsigned char> hout(out_bytes);
            rb.copy(hout.data(), fb, out_bytes);
            kt.mark("filter launches");
            rb.finish();
            kt.mark("filter wait");
            std::vector<uint32_t> hub(ncand * k);
            std::vector<uint64_t> hfs(ncand * 2);
            std::memcpy(hub.data(), hout.data() + o_ub, hub.size() * 4);
            std::memcpy(hfs.data(), hout.data() + o_fs, hfs.size() * 8);
            if (infer) {
                hY.resize(ncand);
                std::memcpy(hY.data(), hout.data() + o_y, ncand * 4);
            }
            us_level_wait += (uint64_t)(ms_since(tl0) * 1000.0);
            for (uint32_t j = 0; j < J; ++j) {
                if (!tr[j]) continue;
                const size_t C = tr[j]->cand.size() / k;
                if ((pv[j].reserved[0] & 2) != 0) tr[j]->feat.assign(C * kMlpIn, 0.f);
                if (infer) tr[j]->pred.assign(C, 0.f);
            }
            for (uint64_t q = 0; q < ncand; ++q) {
                LevelTrace& L = *tr[owner[q].first];
                size_t c = owner[q].second;
                L.fquads[c] = hfs[2 * q];
                L.fcells[c] = hfs[2 * q + 1];
                cnt_fcm += hfs[2 * q + 1] * std::min<uint32_t>(k, kMaxMembersFiltered);
                cnt_fquads += hfs[2 * q];
                cnt_fcells += hfs[2 * q + 1];
                if (!L.feat.empty()) std::memcpy(&L.feat[c * kMlpIn], &hX[q * kMlpIn], kMlpIn * sizeof(float));
                if (infer) L.pred[c] = hY[q];
            }
            for (uint64_t q = 0; q < ncand; ++q) {
                LevelTrace& L = *tr[owner[q].first];
                size_t c = owner[q].second;
                for (uint32_t t = 0; t < k; ++t) L.ub[c * k + t] = hub[q * k + t];
                L.pass[c] = filter_pass(&L.ub[c * k], &L.cand[c * k], k, b.h_fcount, js[owner[q].first].thr);
            }
        }
        // pairs: cost-model features on the host (every candidate when the caller
        // records them, reserved[0] bit 1; else the ones a LEARNED mine refines)
        // and, for LEARNED, one inference launch
        if (k == 2) {
            // pair tables are presized only when every table is written while counted (the
            // single-pass knob); otherwise pairs are counted, the needed ones filled, and no
            // prediction is spent on them
            const bool learned_pairs = learned_mode && force_single_any;
            const auto tm0 = Clock::now();
            struct AddUs {
                uint64_t& acc;
                Clock::time_point t;
                ~AddUs() { acc += (uint64_t)(ms_since(t) * 1000.0); }
            } add_us{us_pairs_model, tm0};
            std::vector<float> X;
            std::vector<std::pair<uint32_t, size_t>> who;
            for (uint32_t j = 0; j < J; ++j) {
                if (!tr[j]) continue;
                const bool all = (pv[j].reserved[0] & 2) != 0;
                if (!all && !learned_pairs) continue;
                LevelTrace& L = *tr[j];
                const size_t C = L.cand.size() / k;
                L.feat.assign(C * kMlpIn, 0.f);
                for (size_t c = 0; c < C; ++c) {
                    if (!all && !L.pass[c]) continue;
                    const uint32_t* mem = &L.cand[c * k];
                    candidate_features(k, mem, b.h_fcount.data(), &L.ub[c * k], b.h_fcount[mem[0]], 0, 0,
                                       &L.feat[c * kMlpIn]);
                    if (learned_pairs && L.pass[c]) {
                        X.insert(X.end(), &L.feat[c * kMlpIn], &L.feat[c * kMlpIn] + kMlpIn);
                        who.push_back({j, c});
                    }
                }
                if (!all) L.feat.clear();   // kept only when the caller records them
            }
            if (!who.empty()) {
                DevBuf<float> dparams, dx, dy;
                std::vector<float> y(who.size());
                dparams.alloc(kMlpParams, s);
                dx.alloc(X.size(), s);
                dy.alloc(who.size(), s);
                COLO_CUDA(cudaMemcpyAsync(dparams.get(), ctx->model.data(), kMlpParams * 4, cudaMemcpyHostToDevice, s));
                COLO_CUDA(cudaMemcpyAsync(dx.get(), X.data(), X.size() * 4, cudaMemcpyHostToDevice, s));
                mlp_forward(dparams.get(), dx.get(), who.size(), dy.get(), s);
                COLO_CUDA(cudaMemcpyAsync(y.data(), dy.get(), y.size() * 4, cudaMemcpyDeviceToHost, s));
                stream_wait(s);
                for (uint32_t j = 0; j < J; ++j)
                    if (tr[j]) tr[j]->pred.assign(tr[j]->cand.size() / k, 0.f);
                for (size_t i = 0; i < who.size(); ++i) tr[who[i].first]->pred[who[i].second] = y[i];
            }
        }
        t_filter += ms_since(t0);
        kt.mark("filter results");

        // ---- refinement: count pass + participation ----
        t0 = Clock::now();
        std::vector<CandDesc> hd;
        std::vector<std::pair<uint32_t, size_t>> owner;
        std::vector<uint64_t> slot_base, chunk_off(1, 0);
        {
            size_t most = 0;   // every candidate of the level passes at most
            for (uint32_t j = 0; j < J; ++j)
                if (tr[j]) most += tr[j]->cand.size() / k;
            hd.reserve(most);
            owner.reserve(most);
            slot_base.reserve(most);
            chunk_off.reserve(most + 1);
        }
        uint64_t nslots = 0, nwords = 0;
        for (uint32_t j = 0; j < J; ++j) {
            if (!tr[j]) continue;
            LevelTrace& L = *tr[j];
            for (size_t c = 0; c < L.cand.size() / k; ++c) {
                if (!L.pass[c]) continue;
                CandDesc d{};
                const uint32_t* mem = &L.cand[c * k];
                if (k == 2) {
                    d.parent = nullptr;
                    d.prow = b.h_fcount[mem[0]];
                    d.pstride = d.prow;
                } else {
                    const TableRef& pt = js[j].prev_tables[js[j].parent[c]];
                    if (!pt.cols && pt.rows)
                        throw StatusError{COLO_ERR_INTERNAL, "missing parent instance table"};
                    d.parent = pt.cols;
                    d.prow = pt.rows;
                    d.pstride = pt.stride;
                }
                for (uint32_t t = 0; t < k; ++t) d.m[t] = mem[t];
                d.job = j;
                d.k = k;
                uint64_t w = 0;
                for (uint32_t t = 0; t < k; ++t) w += (b.h_fcount[mem[t]] + 31) / 32;
                d.bm_base = nwords;
                nwords += w;
                slot_base.push_back(nslots);
                nslots += d.prow;
                chunk_off.push_back(chunk_off.back() + (d.prow + 31) / 32);
                hd.push_back(d);
                owner.push_back({j, c});
            }
        }
        const uint64_t ncand = hd.size();
        kt.mark("refine descriptors");
        // LEARNED: predicted rows presize one-pass tables; the queue runs largest first
        bool learned = mode == COLO_MODE_LEARNED && !ctx->model.empty() && ncand > 0;
        std::vector<uint64_t> cap, pc;
        if (learned) {
            std::vector<float> y(ncand);
            for (uint64_t q = 0; q < ncand; ++q) {
                const LevelTrace& L = *tr[owner[q].first];
                y[q] = L.pred.empty() ? 0.f : L.pred[owner[q].second];
            }
            // a row extends a parent row by one last-member instance: rows <= prow * n_last
            pc.resize(ncand);
            uint64_t words = 0;
            for (uint64_t q = 0; q < ncand; ++q) {
                const uint64_t most = hd[q].prow * (uint64_t)b.h_fcount[hd[q].m[k - 1]];
                pc[q] = std::min(presize_rows(y[q]), std::max<uint64_t>(most, 1));
                words += pc[q] * k;
            }
            // a level whose presized tables would exceed 8 GB takes the exact two-pass form
            if (words > (1ull << 31)) learned = false;
        }
        bool force_single = false;
        for (uint32_t j = 0; j < J; ++j) force_single |= (pv[j].reserved[0] & 16) != 0;
        if (learned && !force_single) {   // no table presized large enough: the order stays as it is
            bool any = false;
            for (uint64_t q = 0; q < ncand && !any; ++q) any = pc[q] >= kSinglePassMinRows;
            if (!any) {
                cap = pc;
                learned = false;   // nothing takes the single pass
            }
        }
        if (learned) {
            // the candidates whose tables are written while counted go first, largest predicted
            // first (their chunks are taken in that order); the others keep their order, which
            // keeps each job's candidates together (counting measured 14% faster that way on the
            // 512-job workload than in a global largest-first order)
            std::vector<uint64_t> perm(ncand);
            for (uint64_t q = 0; q < ncand; ++q) perm[q] = q;
            auto single_q = [&](uint64_t q) { return force_single || pc[q] >= kSinglePassMinRows; };
            const auto mid = std::stable_partition(perm.begin(), perm.end(), single_q);
            std::stable_sort(perm.begin(), mid, [&](uint64_t a, uint64_t c) { return pc[a] > pc[c]; });
            std::vector<CandDesc> hd2(ncand);
            std::vector<std::pair<uint32_t, size_t>> own2(ncand);
            std::vector<uint64_t> sb2(ncand);
            cap.resize(ncand);
            chunk_off.assign(1, 0);
            for (uint64_t i = 0; i < ncand; ++i) {
                hd2[i] = hd[perm[i]];
                own2[i] = owner[perm[i]];
                sb2[i] = slot_base[perm[i]];
                cap[i] = pc[perm[i]];
                chunk_off.push_back(chunk_off.back() + (hd2[i].prow + 31) / 32);
            }
            hd.swap(hd2);
            owner.swap(own2);
            slot_base.swap(sb2);
        }
        // the single pass writes a table while counting it; it pays for tables predicted large
        // (a fill pass would walk them again), small ones are counted and the needed ones filled
        // after the next level's candidates are known.  Candidates [0, ns) take the single pass.
        uint64_t ns = 0;
        if (learned)
            while (ns < ncand && (force_single || cap[ns] >= kSinglePassMinRows)) ++ns;
        // chunk prefixes of the two groups, each from 0: [0, ns] then [ns, ncand]
        std::vector<uint64_t> chunk_all(1, 0);
        for (uint64_t q = 0; q < ncand; ++q) {
            if (q == ns) chunk_all.push_back(0);
            chunk_all.push_back(chunk_all.back() + (hd[q].prow + 31) / 32);
        }
        if (ns == ncand) chunk_all.push_back(0);
        const uint64_t nch_single = chunk_all[ns], nch_count = chunk_all.back();
        kt.mark("refine presize");
        LevelArena ar;
        DevBuf<uint64_t> G;   // the fill's output offsets: the scan of every parent row's count
        // the side stream's scan reads the arena and writes G: the main stream waits for it
        // before either is freed, also when the level ends by an error
        struct SideScan {
            cudaStream_t s;
            cudaEvent_t ev;
            bool pending = false;
            ~SideScan() {
                if (pending) cudaStreamWaitEvent(s, ev, 0);
            }
        } side{s, ctx->ev_scanned};
        ar.init(nslots, nwords, ncand, nch_single, k, ns > 0, s);
        std::unique_ptr<TableBuf> single_cur;
        uint64_t single_words = 0;
        if (ns) {
            for (uint64_t q = 0; q < ns; ++q) single_words += cap[q] * k;
            single_cur.reset(new TableBuf());
            single_cur->alloc(single_words ? single_words : 1, s, host_tables);
            if (single_cur->on_host()) cnt_host_table_bytes += single_words * 4;
        }
        for (uint64_t q = 0, o = 0; q < ncand; ++q) {
            hd[q].slots = ar.slots.get() + slot_base[q];
            hd[q].bitmap = ar.bitmap.get();
            hd[q].rows = ar.rows.get() + q;
            if (q < ns) {
                hd[q].out = single_cur->get() + o;
                hd[q].out_cap = cap[q];
                hd[q].out_rows = cap[q];
                o += cap[q] * k;
            }
        }
        kt.mark("refine arena");
        std::vector<uint64_t> hstats(ncand * k * 4);
        Readback rb(ctx, s, ar.out_bytes + sizeof(DevFlags));
        cnt_refined += ncand;
        cnt_bmw += nwords;
        for (uint64_t q = 0; q < ncand; ++q) cnt_parent += (uint64_t)(k - 1) * hd[q].prow;
        if (ncand) {
            ar.put_inputs(ctx, s, hd, chunk_all);
            if (plain) {
                // per candidate, as the reference refines (one candidate at a time)
                DevBuf<uint64_t> one_off;
                one_off.alloc(2 * ncand, s);
                std::vector<uint64_t> hoff(2 * ncand);
                for (uint64_t q = 0; q < ncand; ++q) {
                    hoff[2 * q] = 0;
                    hoff[2 * q + 1] = chunk_off[q + 1] - chunk_off[q];
                }
                COLO_CUDA(cudaMemcpyAsync(one_off.get(), hoff.data(), 2 * ncand * 8, cudaMemcpyHostToDevice, s));
                for (uint64_t q = 0; q < ncand; ++q) {
                    LevelWork w{ar.descs.get() + q, one_off.get() + 2 * q, 1, hoff[2 * q + 1], ar.items.get()};
                    level_count(b, w, k);
                    level_pi(b, ar.descs.get() + q, 1, k, ar.stats.get() + q * k * 4);
                    COLO_CUDA(cudaMemcpyAsync(hstats.data() + q * k * 4, ar.stats.get() + q * k * 4, k * 4 * 8,
                                              cudaMemcpyDeviceToHost, s));
                    stream_wait(s);
                }
            } else {
                if (ns) {
                    LevelWork w{ar.descs.get(), ar.chunk_off.get(), ns, nch_single, ar.items.get()};
                    w.chunk_status = ar.status.get();
                    w.ticket = ar.status.get() + nch_single;
                    level_single(b, w, k, ar.overflow.get());
                }
                if (ns < ncand) {
                    LevelWork w{ar.descs.get() + ns, ar.chunk_off.get() + ns + 1, ncand - ns, nch_count, ar.items.get()};
                    w.ticket = ar.tickets.get();
                    level_count(b, w, k);
                }
                // the fill's output offsets (the scan of every row's count) on the side stream,
                // during the participation kernel, the wait and the host's Apriori; the profiled
                // pass keeps it on the main stream so that its timers see it
                if (nslots) {
                    G.alloc(nslots, s);
                    if (!kt.on) {
                        COLO_CUDA(cudaEventRecord(ctx->ev_counted, s));
                        COLO_CUDA(cudaStreamWaitEvent(ctx->s2, ctx->ev_counted, 0));
                        scan_u32_to_u64(ar.slots.get(), G.get(), nslots, ctx->s2, nullptr);
                        COLO_CUDA(cudaEventRecord(ctx->ev_scanned, ctx->s2));
                        side.pending = true;
                    } else {
                        scan_u32_to_u64(ar.slots.get(), G.get(), nslots, s, nullptr);
                    }
                }
                level_pi(b, ar.descs.get(), ncand, k, ar.stats.get());
            }
        }
        // row counts, the work counter, overflow flags and the statistics: one copy, one wait
        std::vector<uint64_t> hrows(ncand);
        std::vector<uint32_t> hovf(ncand, 0);
        unsigned long long h_items = 0;
        std::vector<unsigned char> hout(ar.out_bytes);
        if (ar.out_bytes) rb.copy(hout.data(), ar.out, ar.out_bytes);
        DevFlags hflags{};
        if (ns) rb.copy(&hflags, b.flags.get(), sizeof(hflags));
        kt.mark("refine launches");
        rb.finish();
        kt.mark("refine wait");
        if (ncand) {
            std::memcpy(hrows.data(), hout.data(), ncand * 8);
            std::memcpy(&h_items, hout.data() + ncand * 8, 8);
            std::memcpy(hovf.data(), hout.data() + ncand * 8 + 8, ncand * 4);
            if (!plain)
                std::memcpy(hstats.data(), hout.data() + (reinterpret_cast<unsigned char*>(ar.stats.get()) - ar.out),
                            hstats.size() * 8);
        }
        if (hflags.timeout)
            throw StatusError{COLO_ERR_TIMEOUT, "single-pass tables: a chunk waited too long for its predecessors"};
        // participation index (getParticipationIndex, Codes/DeviceProcess.cu:108-132)
        std::vector<uint8_t> prev_flag(ncand, 0);
        for (uint64_t q = 0; q < ncand; ++q) {
            LevelTrace& L = *tr[owner[q].first];
            size_t c = owner[q].second;
            const uint64_t* st = &hstats[q * k * 4];   // [A, last, first, full] per member
            uint64_t num[kMaxK];
            if (k == 2) {
                num[0] = st[0];
                num[1] = (st[4 + 3] - st[4 + 2]) + ((st[4 + 2] | st[1]) ? 1 : 0);
            } else {
                num[0] = st[0];
                for (uint32_t t = 1; t < k; ++t) num[t] = st[(t - 1) * 4 + 1] + st[t * 4 + 0];
            }
            float PI = 1.0f;
            uint32_t am = 0;
            for (uint32_t t = 0; t < k; ++t) {
                L.num[c * k + t] = num[t];
                float pr = (float)num[t] / (float)b.h_fcount[L.cand[c * k + t]];
                if (pr < PI) {
                    PI = pr;
                    am = t;
                }
            }
            L.pi[c] = PI;
            L.argmin[c] = am;
            L.prevalent[c] = !(PI < js[owner[q].first].thr);
            prev_flag[q] = L.prevalent[c];
        }
        // row counts (per-candidate counters of the count pass) and fill offsets
        cnt_single += ns;
        for (uint64_t q = 0; q < ns; ++q) cnt_single_ovf += hovf[q] ? 1 : 0;
        cnt_items += h_items;
        cnt_d2h += ncand * 8 + hstats.size() * 8;
        std::vector<uint64_t> gb(ncand + 1, 0);
        for (uint64_t q = 0; q < ncand; ++q) gb[q + 1] = gb[q] + hrows[q];
        for (uint64_t q = 0; q < ncand; ++q) tr[owner[q].first]->rows[owner[q].second] = gb[q + 1] - gb[q];
        t_refine += ms_since(t0);
        kt.mark("refine results");

        // ---- next candidates (Apriori), the tables they need, and the fill ----
        // A table is needed when its pattern is the prefix of a next-level candidate, so Apriori
        // decides which prevalent tables to fill.  When the tables that can be needed are small
        // (and not filled one at a time, as in the plain form), they are filled first and Apriori
        // runs on the host while the GPU fills; only the needed tables are then recorded
        // (has_table, the next level's parents, the kept tables) -- the same results either way.
        t0 = Clock::now();
        bool next_possible = false;
        for (uint32_t j = 0; j < J; ++j)
            next_possible |= tr[j] && (js[j].max_size == 0 || k + 1 <= js[j].max_size) && k + 1 <= js[j].nf &&
                             k + 1 <= (uint32_t)kMaxK;
        // A next-level candidate joins two prevalent patterns with the same first k-1 members and
        // its prefix is the first of them (candidateColocationGeneral, colocationFinder.cpp:517-557),
        // so only a prevalent pattern followed by a prevalent sibling (candidates are in
        // lexicographic order) can be needed: maybe[j][c] marks those.
        std::vector<std::vector<uint8_t>> maybe(J);
        for (uint32_t j = 0; j < J; ++j) {
            if (!tr[j]) continue;
            const LevelTrace& L = *tr[j];
            const size_t C = L.cand.size() / k;
            maybe[j].assign(C, 0);
            size_t last = SIZE_MAX;   // the previous prevalent candidate
            for (size_t c = 0; c < C; ++c) {
                if (!L.prevalent[c]) continue;
                if (last != SIZE_MAX && std::equal(L.cand.begin() + last * k, L.cand.begin() + last * k + (k - 1),
                                                   L.cand.begin() + c * k))
                    maybe[j][last] = 1;
                last = c;
            }
        }
        uint64_t maybe_words = 0;
        for (uint64_t q = 0; q < ncand; ++q)
            if (prev_flag[q] && maybe[owner[q].first][owner[q].second] && !(q < ns && !hovf[q]))
                maybe_words += (gb[q + 1] - gb[q]) * k;
        // (one job only: in a batch of many small jobs Apriori's subset test prunes most of
        // the possible tables -- on the 512-job workload the early fill took 11.3 ms per mine
        // against 2.7 ms for the needed tables after Apriori)
        const bool early_fill =
            !plain && !host_tables && next_possible && maybe_words <= kEarlyFillWords && J == 1;

        // needed[j][c]: candidate c of this level is the prefix of a next-level candidate
        std::vector<std::vector<uint8_t>> needed(J);
        auto run_apriori = [&]() {
            const auto ta = Clock::now();
            std::vector<std::vector<uint32_t>> prevs(J), prevcs(J), dnext, dpar;
            std::vector<const std::vector<uint32_t>*> gen(J, nullptr);
            uint64_t prev_total = 0;
            for (uint32_t j = 0; j < J; ++j) {
                if (!tr[j]) continue;
                LevelTrace& L = *tr[j];
                for (size_t c = 0; c < L.cand.size() / k; ++c)
                    if (L.prevalent[c]) {
                        prevs[j].insert(prevs[j].end(), L.cand.begin() + c * k, L.cand.begin() + (c + 1) * k);
                        prevcs[j].push_back((uint32_t)c);
                    }
                const bool cap_ok = (js[j].max_size == 0 || k + 1 <= js[j].max_size) && k + 1 <= js[j].nf;
                if (cap_ok) {
                    gen[j] = &prevs[j];
                    prev_total += prevcs[j].size();
                }
            }
            // many prevalent patterns: all jobs' candidates in two device passes
            bool force_dev = false;
            for (uint32_t j = 0; j < J; ++j) force_dev |= (pv[j].reserved[0] & 4) != 0;
            const bool on_device = (prev_total >= kDeviceAprioriMin || (force_dev && prev_total > 0)) &&
                                   k + 1 <= (uint32_t)kMaxK;
            if (on_device) apriori_device(s, gen, k, dnext, dpar);
            for (uint32_t j = 0; j < J; ++j) {
                if (!tr[j]) continue;
                LevelTrace& L = *tr[j];
                const std::vector<uint32_t>& prev_c = prevcs[j];
                std::vector<uint32_t> next, par;
                if (gen[j]) {
                    if (on_device) {
                        next = std::move(dnext[j]);
                        par = std::move(dpar[j]);
                    } else {
                        next = apriori_next(prevs[j], k, par);
                    }
                }
                js[j].cands = next;
                needed[j].assign(L.cand.size() / k, 0);
                for (auto& pp : par) {
                    pp = prev_c[pp];        // now an index among this level's candidates
                    needed[j][pp] = 1;
                }
                js[j].parent = std::move(par);
            }
            t_apriori += ms_since(ta);
            kt.mark("apriori");
        };
        if (!early_fill) {
            run_apriori();
            t0 = Clock::now();   // the fill's own time
        }

        // ---- fill pass for the (needed) prevalent patterns ----
        std::vector<uint64_t> fillq, keepq;   // keepq: tables the single pass already wrote whole
        uint64_t total_rows = 0;
        for (uint64_t q = 0; q < ncand; ++q) {
            if (!prev_flag[q]) continue;
            if (early_fill ? !maybe[owner[q].first][owner[q].second] : !needed[owner[q].first][owner[q].second])
                continue;
            if (q < ns && !hovf[q]) {
                keepq.push_back(q);
                continue;
            }
            fillq.push_back(q);
            total_rows += gb[q + 1] - gb[q];
        }
        for (uint64_t q = 0; q < ns; ++q)   // rows the single pass wrote (tables that fit their presize)
                if (!hovf[q]) {
                    rows_written += gb[q + 1] - gb[q];
                    cnt_fillw += (gb[q + 1] - gb[q]) * k;
                }
        tables_cur.reset(new TableBuf());
        tables_cur->alloc(total_rows * k ? total_rows * k : 1, s, host_tables);
        if (tables_cur->on_host()) cnt_host_table_bytes += total_rows * k * 4;
        // output offsets of every parent row: exclusive scan of the slots (batched: already
        // launched with the count, on the side stream; the main stream waits for it here)
        if (side.pending) {
            COLO_CUDA(cudaStreamWaitEvent(s, ctx->ev_scanned, 0));
            side.pending = false;
        }
        if (!fillq.empty() && plain) {
            G.alloc(nslots, s);
            for (uint64_t q : fillq)   // one scan per candidate, as the reference does
                scan_u32_to_u64(ar.slots.get() + slot_base[q], G.get() + slot_base[q], hd[q].prow, s, nullptr);
        }
        std::vector<CandDesc> fd;
        std::vector<uint64_t> fchunk(1, 0);
        uint64_t obase = 0;
        for (uint64_t q : fillq) {
            CandDesc d = hd[q];
            uint64_t rows = gb[q + 1] - gb[q];
            d.offs = G.get() + slot_base[q];
            d.out = tables_cur->get() + obase;
            d.out_rows = rows;
            obase += rows * k;
            fd.push_back(d);
            fchunk.push_back(fchunk.back() + (d.prow + 31) / 32);
        }
        rows_written += total_rows;
        cnt_fillw += total_rows * k;
        // the fill's descriptors and chunk prefixes: one allocation, one upload
        DevBuf<unsigned char> fin;
        CandDesc* dfd_p = nullptr;
        uint64_t* dfc_p = nullptr;
        if (!fd.empty()) {
            const size_t at = (fd.size() * sizeof(CandDesc) + 15) & ~(size_t)15;
            const size_t bytes = at + fchunk.size() * 8;
            unsigned char* h = upload_area(ctx, s, bytes);
            std::memcpy(h, fd.data(), fd.size() * sizeof(CandDesc));
            std::memcpy(h + at, fchunk.data(), fchunk.size() * 8);
            fin.alloc(bytes, s);
            dfd_p = reinterpret_cast<CandDesc*>(fin.get());
            dfc_p = reinterpret_cast<uint64_t*>(fin.get() + at);
            upload_from(s, fin.get(), h, bytes);
            if (plain) {
                DevBuf<uint64_t> one_off;
                one_off.alloc(2 * fd.size(), s);
                std::vector<uint64_t> hoff(2 * fd.size());
                for (size_t q = 0; q < fd.size(); ++q) {
                    hoff[2 * q] = 0;
                    hoff[2 * q + 1] = fchunk[q + 1] - fchunk[q];
                }
                COLO_CUDA(cudaMemcpyAsync(one_off.get(), hoff.data(), hoff.size() * 8, cudaMemcpyHostToDevice, s));
                for (size_t q = 0; q < fd.size(); ++q) {
                    LevelWork w{dfd_p + q, one_off.get() + 2 * q, 1, hoff[2 * q + 1], nullptr};
                    level_fill(b, w, k);
                    stream_wait(s);
                }
            } else {
                LevelWork w{dfd_p, dfc_p, fd.size(), fchunk.back(), nullptr};
                w.ticket = ar.tickets.get() + 1;
                level_fill(b, w, k);
            }
        }
        if (early_fill) run_apriori();   // on the host while the GPU fills
        // the needed tables among those written
        for (uint64_t q : fillq) {
            if (!needed[owner[q].first][owner[q].second]) continue;
            tr[owner[q].first]->has_table[owner[q].second] = 1;
        }
        // the tables are read back only when kept in the result (a copy on another stream); else
        // the next level's launches queue behind the fill on this stream without a wait
        bool keep_any = false;
        for (uint32_t j = 0; j < J; ++j) keep_any |= pv[j].keep_tables != 0;
        if (keep_any) stream_wait(s);
        // register the new tables (prefixes of the next level)
        for (uint32_t j = 0; j < J; ++j) {
            js[j].prev_tables.clear();
            if (tr[j]) js[j].prev_tables.assign(tr[j]->cand.size() / k, TableRef{});
        }
        std::vector<std::pair<uint64_t, TableRef>> made;
        for (size_t i = 0; i < fillq.size(); ++i)
            if (needed[owner[fillq[i]].first][owner[fillq[i]].second])
                made.push_back({fillq[i], TableRef{fd[i].out, fd[i].out_rows, fd[i].out_rows}});
        for (uint64_t q : keepq) {
            if (!needed[owner[q].first][owner[q].second]) continue;
            made.push_back({q, TableRef{hd[q].out, gb[q + 1] - gb[q], cap[q]}});
            tr[owner[q].first]->has_table[owner[q].second] = 1;
        }
        for (const auto& mt : made) {
            const uint64_t q = mt.first;
            const TableRef& t = mt.second;
            LevelTrace& L = *tr[owner[q].first];
            size_t c = owner[q].second;
            js[owner[q].first].prev_tables[c] = t;
            if (pv[owner[q].first].keep_tables) {
                uint64_t rows = t.rows;
                std::vector<uint32_t> colm(rows * k);
                if (rows)
                    COLO_CUDA(cudaMemcpy2D(colm.data(), rows * 4, t.cols, t.stride * 4, rows * 4, k,
                                           cudaMemcpyDefault));   // the tables may be in host memory
                if (L.tables.size() < L.cand.size() / k) L.tables.resize(L.cand.size() / k);
                std::vector<uint32_t>& rm = L.tables[c];
                rm.resize(rows * k);
                for (uint64_t r = 0; r < rows; ++r)
                    for (uint32_t t = 0; t < k; ++t) rm[r * k + t] = colm[(uint64_t)t * rows + r];
            }
        }
        t_fill += ms_since(t0);
        kt.mark("fill launches");
        tables_prev = std::move(tables_cur);
        single_prev = std::move(single_cur);
        for (auto& st : js)
            if (st.cands.empty()) st.active = false;
    }
    stream_wait(s);
    kt.resolve();
    for (uint32_t j = 0; j < J; ++j) {
        MineResult* r = outs[j];
        r->kernels = kt.stats;
        r->counters[5] = b.N;
        r->counters[6] = b.M;
        r->counters[7] = b.Rn;
        r->counters[8] = cnt_items;
        r->counters[9] = cnt_parent;
        r->counters[10] = cnt_fillw;
        r->counters[11] = cnt_bmw;
        r->counters[12] = b.h2d_points;
        r->counters[13] = cnt_d2h;
        r->counters[14] = b.nrl_total;
        r->counters[4] = b.join_pairs;
        r->counters[15] = cnt_refined;
        r->counters[16] = b.filter_items;
        r->counters[17] = cnt_single;
        r->counters[18] = cnt_single_ovf;
        r->counters[19] = cnt_fcm;
        r->counters[20] = cnt_fquads;
        r->counters[21] = cnt_fcells;
        r->counters[22] = us_pairs_model;
        r->counters[23] = us_level_wait;
        r->counters[24] = cnt_host_table_bytes;
        r->times[0] = ms_since(t_all);
        r->times[1] = t_upload;
        r->times[2] = t_bucket;
        r->times[3] = t_join;
        r->times[4] = t_filter;
        r->times[5] = t_refine;
        r->times[6] = t_fill;
        r->times[7] = t_apriori;
        r->counters[0] = g_launches;
        r->counters[1] = b.active_anchors;
        r->counters[2] = neighbor_entries(b);
        r->counters[3] = rows_written;
    }
}

}  // namespace colo

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* colo_status_string(colo_status s) {
    switch (s) {
        case COLO_OK: return "ok";
        case COLO_ERR_ARG: return "invalid argument";
        case COLO_ERR_IO: return "i/o error";
        case COLO_ERR_PARSE: return "parse error";
        case COLO_ERR_INPUT: return "input outside the reference's domain";
        case COLO_ERR_CUDA: return "CUDA error";
        case COLO_ERR_NOMEM: return "out of memory";
        case COLO_ERR_TIMEOUT: return "device wait timed out";
        case COLO_ERR_CAPACITY: return "capacity exceeded";
        case COLO_ERR_NO_DEVICE: return "no CUDA device";
        default: return "internal error";
    }
}

void colo_params_default(colo_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->distance = 1.0f;
    p->pi_threshold = 0.5f;
    p->mode = COLO_MODE_BATCHED;
}

colo_status colo_create(colo_ctx** out, int device) {
    if (!out) return COLO_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return COLO_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return COLO_ERR_ARG;
    std::unique_ptr<colo_ctx> c(new colo_ctx());
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) return COLO_ERR_CUDA;
    if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess) return COLO_ERR_CUDA;
    if (cudaStreamCreateWithFlags(&c->s2, cudaStreamNonBlocking) != cudaSuccess) return COLO_ERR_CUDA;
    if (cudaEventCreateWithFlags(&c->ev_counted, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_scanned, cudaEventDisableTiming) != cudaSuccess)
        return COLO_ERR_CUDA;
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    // keep freed blocks in the stream-ordered pool between calls
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    *out = c.release();
    return COLO_OK;
}

colo_status colo_destroy(colo_ctx* ctx) {
    if (!ctx) return COLO_ERR_ARG;
    ctx_release(ctx);
    return COLO_OK;
}

const char* colo_last_error(const colo_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }

colo_status colo_read_params(const char* path, colo_params* out) {
    if (!path || !out) return COLO_ERR_ARG;
    std::string err;
    return read_params_file(path, out, err);
}

colo_status colo_read_config(const char* path, char* location, char* param_file, char* dataset,
                             char* out_location, char* out_file, size_t cap) {
    if (!path || cap == 0) return COLO_ERR_ARG;
    std::string lines[5], err;
    colo_status st = read_config_file(path, lines, err);
    if (st != COLO_OK) return st;
    char* dst[5] = {location, param_file, dataset, out_location, out_file};
    for (int i = 0; i < 5; ++i) {
        if (!dst[i]) continue;
        if (lines[i].size() + 1 > cap) return COLO_ERR_CAPACITY;
        std::memcpy(dst[i], lines[i].c_str(), lines[i].size() + 1);
    }
    return COLO_OK;
}

colo_status colo_dataset_from_csv_threads(colo_ctx* ctx, const char* path, uint32_t threads, colo_dataset** out) {
    if (!ctx || !path || !out) return COLO_ERR_ARG;
    return guarded(ctx, [&]() {
        std::unique_ptr<colo_dataset> ds(new colo_dataset());
        ds->ctx = ctx;
        std::string err;
        colo_status st = parse_points_csv(path, ds->hp, err, threads);
        if (st != COLO_OK) return set_err(ctx, st, err);
        group_features(ds.get());
        ctx->refs++;
        *out = ds.release();
        return COLO_OK;
    });
}

colo_status colo_dataset_from_csv(colo_ctx* ctx, const char* path, colo_dataset** out) {
    return colo_dataset_from_csv_threads(ctx, path, 0, out);
}

colo_status colo_dataset_from_csv_device(colo_ctx* ctx, const char* path, colo_dataset** out) {
    if (!ctx || !path || !out) return COLO_ERR_ARG;
    return guarded(ctx, [&]() {
        std::unique_ptr<colo_dataset> ds(new colo_dataset());
        ds->ctx = ctx;
        std::string err;
        colo_status st = parse_points_csv_device(ctx->s, path, ds->hp, ds->dx, ds->dy, err);
        if (st != COLO_OK) return set_err(ctx, st, err);
        group_features(ds.get());
        ds->resident = true;   // the parsed coordinates are already on the device
        ctx->refs++;
        *out = ds.release();
        return COLO_OK;
    });
}

colo_status colo_dataset_from_binary(colo_ctx* ctx, const char* path, colo_dataset** out) {
    if (!ctx || !path || !out) return COLO_ERR_ARG;
    return guarded(ctx, [&]() {
        std::unique_ptr<colo_dataset> ds(new colo_dataset());
        ds->ctx = ctx;
        std::string err;
        colo_status st = read_points_binary(path, ds->hp, err);
        if (st != COLO_OK) return set_err(ctx, st, err);
        group_features(ds.get());
        ctx->refs++;
        *out = ds.release();
        return COLO_OK;
    });
}

colo_status colo_dataset_write_binary(const colo_dataset* ds, const char* path) {
    if (!ds || !path) return COLO_ERR_ARG;
    std::string err;
    colo_status st = write_points_binary(ds->hp, ds->names, path, err);
    return st != COLO_OK ? set_err(ds->ctx, st, err) : st;
}

colo_status colo_csv_to_binary(const char* csv_path, const char* bin_path, uint32_t threads, char* err,
                               size_t err_cap) {
    if (!csv_path || !bin_path) return COLO_ERR_ARG;
    std::string msg;
    colo_status st;
    try {
        colo_dataset ds;
        st = parse_points_csv(csv_path, ds.hp, msg, threads);
        if (st == COLO_OK) {
            group_features(&ds);
            st = write_points_binary(ds.hp, ds.names, bin_path, msg);
        }
    } catch (const std::bad_alloc&) {
        st = COLO_ERR_NOMEM;
        msg = "host allocation failed";
    }
    if (err && err_cap) {
        const size_t m = std::min(msg.size(), err_cap - 1);
        std::memcpy(err, msg.data(), m);
        err[m] = 0;
    }
    return st;
}

colo_status colo_dataset_from_host(colo_ctx* ctx, const float* x, const float* y, const int32_t* fid,
                                   uint64_t n, const float bounds[4], colo_dataset** out) {
    if (!ctx || !out || !bounds || (n && (!x || !y || !fid))) return COLO_ERR_ARG;
    return guarded(ctx, [&]() {
        std::unique_ptr<colo_dataset> ds(new colo_dataset());
        ds->ctx = ctx;
        ds->hp.x.assign(x, x + n);
        ds->hp.y.assign(y, y + n);
        ds->hp.raw.assign(fid, fid + n);
        for (uint64_t i = 0; i < n; ++i)
            if (fid[i] == -1) return set_err(ctx, COLO_ERR_INPUT, "feature id -1 is reserved by the reference");
        std::memcpy(ds->hp.bounds, bounds, 16);
        group_features(ds.get());
        ctx->refs++;
        *out = ds.release();
        return COLO_OK;
    });
}

colo_status colo_dataset_write_csv(const colo_dataset* ds, const char* path) {
    if (!ds || !path) return COLO_ERR_ARG;
    std::string err;
    return write_points_csv(ds->hp, ds->names, ds->fstart, ds->fcount, path, err);
}

colo_status colo_dataset_upload(colo_dataset* ds) {
    if (!ds) return COLO_ERR_ARG;
    return guarded(ds->ctx, [&]() {
        upload_dataset(ds, ds->ctx->s);
        return COLO_OK;
    });
}

colo_status colo_dataset_evict(colo_dataset* ds) {
    if (!ds) return COLO_ERR_ARG;
    ds->dx.release();
    ds->dy.release();
    ds->resident = false;
    return COLO_OK;
}

uint64_t colo_dataset_num_points(const colo_dataset* ds) { return ds ? ds->hp.x.size() : 0; }
uint32_t colo_dataset_num_features(const colo_dataset* ds) { return ds ? (uint32_t)ds->names.size() : 0; }
uint64_t colo_dataset_feature_count(const colo_dataset* ds, uint32_t f) {
    if (!ds || f >= ds->fcount.size()) return 0;
    return ds->fcount[f];
}

const char* colo_dataset_feature_name(const colo_dataset* ds, uint32_t f) {
    return (ds && f < ds->names.size()) ? ds->names[f].c_str() : nullptr;
}
void colo_dataset_free(colo_dataset* ds) {
    if (!ds) return;
    colo_ctx* ctx = ds->ctx;
    if (ctx) cudaStreamSynchronize(ctx->s);
    if (ds->pinned && !ds->hp.x.empty()) {
        cudaHostUnregister(ds->hp.x.data());
        cudaHostUnregister(ds->hp.y.data());
        cudaGetLastError();
    }
    delete ds;
    if (ctx) ctx_release(ctx);
}

colo_status colo_mine_batch(colo_ctx* ctx, colo_dataset* const* ds, const colo_params* p, uint32_t njobs,
                            colo_result** out) {
    if (!ctx || !ds || !p || !out || njobs == 0) return COLO_ERR_ARG;
    for (uint32_t j = 0; j < njobs; ++j) {
        out[j] = nullptr;
        if (!ds[j] || ds[j]->ctx != ctx) return COLO_ERR_ARG;
        if (p[j].mode != p[0].mode) return set_err(ctx, COLO_ERR_ARG, "all jobs of a batch use one mode");
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return COLO_ERR_CUDA;
    std::vector<std::unique_ptr<colo_result>> res(njobs);
    std::vector<MineResult*> mr(njobs);
    for (uint32_t j = 0; j < njobs; ++j) {
        res[j].reset(new colo_result());
        mr[j] = &res[j]->r;
    }
    colo_status st = guarded(ctx, [&]() {
        pool_reset_mark(ctx);   // from here the pool's high-water mark is this call's
        if (p[0].mode == COLO_MODE_PLAIN && njobs > 1) {
            for (uint32_t j = 0; j < njobs; ++j) mine_jobs(ctx, &ds[j], &p[j], 1, &mr[j]);
        } else {
            mine_jobs(ctx, ds, p, njobs, mr.data());
        }
        pool_headroom(ctx);   // the mine's buffers are back in the pool
        return COLO_OK;
    });
    if (st != COLO_OK) return st;
    for (uint32_t j = 0; j < njobs; ++j) out[j] = res[j].release();
    return COLO_OK;
}

colo_status colo_mine(colo_ctx* ctx, colo_dataset* ds, const colo_params* p, colo_result** out) {
    return colo_mine_batch(ctx, &ds, p, 1, out);
}

uint32_t colo_result_num_levels(const colo_result* r) { return r ? (uint32_t)r->r.levels.size() : 0; }
uint32_t colo_result_level_size(const colo_result* r, uint32_t li) {
    return (r && li < r->r.levels.size()) ? r->r.levels[li].k : 0;
}
uint64_t colo_result_level_candidates(const colo_result* r, uint32_t li) {
    return (r && li < r->r.levels.size()) ? r->r.levels[li].cand.size() / r->r.levels[li].k : 0;
}

colo_status colo_result_level(const colo_result* r, uint32_t li, uint32_t* cand, uint64_t* ub, uint8_t* pass,
                              uint64_t* rows, uint64_t* num, float* pi, uint8_t* prevalent, uint32_t* argmin) {
    if (!r || li >= r->r.levels.size()) return COLO_ERR_ARG;
    const LevelTrace& L = r->r.levels[li];
    size_t C = L.cand.size() / L.k;
    if (cand)
        for (size_t i = 0; i < L.cand.size(); ++i) cand[i] = L.cand[i] - L.f0;
    if (ub) std::memcpy(ub, L.ub.data(), L.ub.size() * 8);
    if (pass) std::memcpy(pass, L.pass.data(), C);
    if (rows) std::memcpy(rows, L.rows.data(), C * 8);
    if (num) std::memcpy(num, L.num.data(), L.num.size() * 8);
    if (pi) std::memcpy(pi, L.pi.data(), C * 4);
    if (prevalent) std::memcpy(prevalent, L.prevalent.data(), C);
    if (argmin) std::memcpy(argmin, L.argmin.data(), C * 4);
    return COLO_OK;
}

uint64_t colo_result_table(const colo_result* r, uint32_t li, uint64_t ci, uint32_t* out) {
    if (!r || li >= r->r.levels.size()) return UINT64_MAX;
    const LevelTrace& L = r->r.levels[li];
    if (ci >= L.has_table.size() || !L.has_table[ci] || ci >= L.tables.size()) return UINT64_MAX;
    const auto& t = L.tables[ci];
    if (out) std::memcpy(out, t.data(), t.size() * 4);
    return t.size() / L.k;
}

colo_status colo_result_write_patterns(const colo_result* r, const colo_dataset* ds, const char* location) {
    if (!r || !ds || !location) return COLO_ERR_ARG;
    std::string err;
    return write_patterns(r->r, ds->names, location, err);
}

colo_status colo_result_times(const colo_result* r, double* ms8) {
    if (!r || !ms8) return COLO_ERR_ARG;
    std::memcpy(ms8, r->r.times, sizeof(r->r.times));
    return COLO_OK;
}

colo_status colo_result_counters(const colo_result* r, uint64_t* c, uint32_t n) {
    if (!r || !c) return COLO_ERR_ARG;
    for (uint32_t i = 0; i < n; ++i) c[i] = i < (uint32_t)kNumCounters ? r->r.counters[i] : 0;
    return COLO_OK;
}

uint32_t colo_result_num_kernels(const colo_result* r) { return r ? (uint32_t)r->r.kernels.size() : 0; }

colo_status colo_result_kernel(const colo_result* r, uint32_t i, char* name, size_t cap, uint64_t* launches,
                               double* ms) {
    if (!r || i >= r->r.kernels.size()) return COLO_ERR_ARG;
    const KernelStat& k = r->r.kernels[i];
    if (name && cap) {
        size_t m = std::min(cap - 1, k.name.size());
        std::memcpy(name, k.name.data(), m);
        name[m] = 0;
    }
    if (launches) *launches = k.launches;
    if (ms) *ms = k.ms;
    return COLO_OK;
}

void* colo_ctx_stream(const colo_ctx* ctx) { return ctx ? (void*)ctx->s : nullptr; }

void colo_result_free(colo_result* r) { delete r; }

}  // extern "C"
