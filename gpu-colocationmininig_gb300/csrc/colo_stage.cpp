// colo_stage.cpp -- stage-level C entry points (one kernel family each), the
// counterparts of the reference's inner extern "C" API
// (Codes/DeviceProcess.h:4-36).  They run one stage on a dataset and copy
// its result to host arrays, so each kernel can be checked in isolation.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "colo_batch.h"
#include "colo_host.h"

using namespace colo;

namespace {

colo_params params_for(float R, float thr) {
    colo_params p;
    colo_params_default(&p);
    p.distance = R;
    p.pi_threshold = thr;
    return p;
}

}  // namespace

extern "C" {

colo_status colo_stage_cells(colo_ctx* ctx, colo_dataset* ds, float R, uint64_t* cell_of, uint64_t* run_cell,
                             uint32_t* run_feat, uint32_t* run_count, uint64_t* nruns) {
    if (!ctx || !ds || !nruns) return COLO_ERR_ARG;
    return run_guarded(ctx, [&]() -> colo_status {
        colo_params p = params_for(R, 0.f);
        Batch b;
        std::vector<DevBuf<float>> of;
        colo_dataset* dsv[1] = {ds};
        setup_batch(ctx, dsv, &p, 1, b, of, nullptr);
        b.keep_scell = cell_of != nullptr;
        if (b.N) bucket_points(b);
        cudaStream_t s = ctx->s;
        uint64_t cap = *nruns;
        *nruns = b.Rn;
        if (cell_of && b.N) {
            // per point: cell key of its sorted position
            std::vector<uint32_t> sid(b.N), scell(b.N);
            std::vector<uint64_t> ckey(b.M);
            COLO_CUDA(cudaMemcpyAsync(sid.data(), b.sid.get(), b.N * 4, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaMemcpyAsync(scell.data(), b.scell.get(), b.N * 4, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaMemcpyAsync(ckey.data(), b.ckey.get(), b.M * 8, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaStreamSynchronize(s));
            for (uint64_t q = 0; q < b.N; ++q) cell_of[sid[q]] = ckey[scell[q]];
        }
        if ((run_cell || run_feat || run_count) && b.Rn) {
            if (cap < b.Rn) return COLO_ERR_CAPACITY;
            std::vector<uint32_t> rf(b.Rn), rc(b.Rn), rcell(b.Rn);
            std::vector<uint64_t> ckey(b.M);
            COLO_CUDA(cudaMemcpyAsync(rf.data(), b.rfeat.get(), b.Rn * 4, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaMemcpyAsync(rc.data(), b.rcnt.get(), b.Rn * 4, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaMemcpyAsync(rcell.data(), b.rcell.get(), b.Rn * 4, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaMemcpyAsync(ckey.data(), b.ckey.get(), b.M * 8, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaStreamSynchronize(s));
            for (uint64_t r = 0; r < b.Rn; ++r) {
                if (run_cell) run_cell[r] = ckey[rcell[r]];
                if (run_feat) run_feat[r] = rf[r];
                if (run_count) run_count[r] = rc[r];
            }
        }
        return COLO_OK;
    });
}

colo_status colo_stage_neighbors(colo_ctx* ctx, colo_dataset* ds, float R, uint64_t* offs, uint32_t* nbr,
                                 uint64_t* total) {
    if (!ctx || !ds || !total) return COLO_ERR_ARG;
    return run_guarded(ctx, [&]() -> colo_status {
        colo_params p = params_for(R, 0.f);
        Batch b;
        std::vector<DevBuf<float>> of;
        colo_dataset* dsv[1] = {ds};
        setup_batch(ctx, dsv, &p, 1, b, of, nullptr);
        uint64_t cap = *total;
        if (b.N) {
            bucket_points(b);
            build_neighborhoods(b);
            join_neighbors(b);
        }
        *total = neighbor_entries(b);
        cudaStream_t s = ctx->s;
        if (offs) offs[0] = 0;
        if ((offs || nbr) && b.N) {
            // compact the per-anchor lists into a CSR
            std::vector<uint64_t> beg(b.N);
            std::vector<uint32_t> cnt(b.N), all(b.nb_cap);
            COLO_CUDA(cudaMemcpyAsync(beg.data(), b.nb_beg.get(), b.N * 8, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaMemcpyAsync(cnt.data(), b.nb_cnt.get(), b.N * 4, cudaMemcpyDeviceToHost, s));
            if (b.nb_cap)
                COLO_CUDA(cudaMemcpyAsync(all.data(), b.nb.get(), b.nb_cap * 4, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaStreamSynchronize(s));
            if (nbr && cap < neighbor_entries(b)) return COLO_ERR_CAPACITY;
            uint64_t o = 0;
            for (uint64_t a = 0; a < b.N; ++a) {
                if (nbr && cnt[a]) std::memcpy(nbr + o, all.data() + beg[a], cnt[a] * 4);
                o += cnt[a];
                if (offs) offs[a + 1] = o;
            }
        }
        COLO_CUDA(cudaStreamSynchronize(s));
        return COLO_OK;
    });
}

colo_status colo_stage_filter(colo_ctx* ctx, colo_dataset* ds, float R, float thr, const uint32_t* cand,
                              uint64_t ncand, uint32_t k, uint64_t* ub, uint8_t* pass) {
    if (!ctx || !ds || (ncand && (!cand || !ub))) return COLO_ERR_ARG;
    if (k < 2 || k > kMaxK) return COLO_ERR_ARG;
    return run_guarded(ctx, [&]() -> colo_status {
        colo_params p = params_for(R, thr);
        Batch b;
        std::vector<DevBuf<float>> of;
        colo_dataset* dsv[1] = {ds};
        setup_batch(ctx, dsv, &p, 1, b, of, nullptr);
        if (b.N) bucket_points(b);
        for (uint64_t c = 0; c < ncand * k; ++c)
            if (cand[c] >= b.F) return COLO_ERR_ARG;
        cudaStream_t s = ctx->s;
        std::vector<uint64_t> hub(ncand * k, 0);
        if (b.N && ncand) {
            if (k == 2) {
                DevBuf<uint32_t> ub2;
                std::vector<uint64_t> job_off;
                filter_pairs(b, ub2, job_off, s);
                COLO_CUDA(cudaStreamSynchronize(s));
                std::vector<uint32_t> h(job_off[1]);
                COLO_CUDA(cudaMemcpy(h.data(), ub2.get(), h.size() * 4, cudaMemcpyDeviceToHost));
                uint32_t nf = b.F;
                for (uint64_t c = 0; c < ncand; ++c) {
                    uint32_t a = cand[2 * c], bb = cand[2 * c + 1];
                    hub[2 * c] = a == bb ? 0 : h[(uint64_t)a * nf + bb];
                    hub[2 * c + 1] = a == bb ? 0 : h[(uint64_t)bb * nf + a];
                }
            } else {
                DevBuf<uint32_t> du;
                du.alloc(ncand * k, s);
                du.zero(s);
                std::vector<uint32_t> job(ncand, 0);
                filter_level(b, cand, job.data(), ncand, k, du.get(), nullptr);
                std::vector<uint32_t> h(ncand * k);
                COLO_CUDA(cudaMemcpyAsync(h.data(), du.get(), h.size() * 4, cudaMemcpyDeviceToHost, s));
                COLO_CUDA(cudaStreamSynchronize(s));
                for (uint64_t q = 0; q < ncand * k; ++q) hub[q] = h[q];
            }
        }
        std::memcpy(ub, hub.data(), hub.size() * 8);
        if (pass) {
            for (uint64_t c = 0; c < ncand; ++c) {
                float pi0 = 1.0f;
                for (uint32_t j = 0; j < k; ++j) {
                    float pr = (float)((double)hub[c * k + j] / (double)(float)b.h_fcount[cand[c * k + j]]);
                    if (j == 0) pi0 = pr;
                    else if (pi0 > pr) pi0 = pr;
                }
                pass[c] = pi0 >= thr;
            }
        }
        return COLO_OK;
    });
}

colo_status colo_stage_apriori(colo_ctx* ctx, const uint32_t* prev, uint64_t nprev, uint32_t k, uint32_t* out,
                               uint32_t* parent, uint64_t cap, uint64_t* n_out) {
    if (!ctx || !n_out || k < 2 || (nprev && !prev) || (cap && (!out || !parent))) return COLO_ERR_ARG;
    if (k > (uint32_t)kMaxK) return set_err(ctx, COLO_ERR_CAPACITY, "patterns larger than 32 features are not supported");
    return run_guarded(ctx, [&]() -> colo_status {
        std::vector<uint32_t> rows(prev, prev + nprev * (k - 1));
        std::vector<const std::vector<uint32_t>*> gen{&rows};
        std::vector<std::vector<uint32_t>> next, par;
        apriori_device(ctx->s, gen, k - 1, next, par);
        const uint64_t n = par[0].size();
        const uint64_t m = std::min<uint64_t>(n, cap);
        if (m) {
            std::memcpy(out, next[0].data(), m * k * 4);
            std::memcpy(parent, par[0].data(), m * 4);
        }
        *n_out = n;
        return COLO_OK;
    });
}

colo_status colo_stage_sqdist(colo_ctx* ctx, const float* x1, const float* y1, const float* x2, const float* y2,
                              uint64_t n, float* out) {
    return colo_stage_within(ctx, x1, y1, x2, y2, n, 0.0f, out, nullptr);
}

colo_status colo_stage_scan(colo_ctx* ctx, const void* in, uint64_t n, int wide, uint64_t* out, uint64_t* total) {
    if (!ctx || !total || (n && (!in || !out)) || (wide != 0 && wide != 1)) return COLO_ERR_ARG;
    return run_guarded(ctx, [&]() -> colo_status {
        cudaStream_t s = ctx->s;
        DevBuf<uint64_t> o, t;
        o.alloc(n ? n : 1, s);
        t.alloc(1, s);
        if (wide) {
            DevBuf<uint64_t> a;
            a.alloc(n ? n : 1, s);
            if (n) COLO_CUDA(cudaMemcpyAsync(a.get(), in, n * 8, cudaMemcpyHostToDevice, s));
            scan_u64_to_u64(a.get(), o.get(), n, s, nullptr, t.get());
        } else {
            DevBuf<uint32_t> a;
            a.alloc(n ? n : 1, s);
            if (n) COLO_CUDA(cudaMemcpyAsync(a.get(), in, n * 4, cudaMemcpyHostToDevice, s));
            scan_u32_to_u64(reinterpret_cast<const uint32_t*>(a.get()), o.get(), n, s, nullptr, t.get());
        }
        if (n) COLO_CUDA(cudaMemcpyAsync(out, o.get(), n * 8, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaMemcpyAsync(total, t.get(), 8, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaStreamSynchronize(s));
        return COLO_OK;
    });
}

colo_status colo_stage_within(colo_ctx* ctx, const float* x1, const float* y1, const float* x2, const float* y2,
                              uint64_t n, float R2, float* out, uint8_t* within) {
    if (!ctx || (n && (!x1 || !y1 || !x2 || !y2 || (!out && !within)))) return COLO_ERR_ARG;
    return run_guarded(ctx, [&]() -> colo_status {
        cudaStream_t s = ctx->s;
        DevBuf<float> a, b, c, d, o;
        DevBuf<uint8_t> w;
        if (within) w.alloc(n, s);
        a.alloc(n, s);
        b.alloc(n, s);
        c.alloc(n, s);
        d.alloc(n, s);
        o.alloc(n, s);
        if (n) {
            COLO_CUDA(cudaMemcpyAsync(a.get(), x1, n * 4, cudaMemcpyHostToDevice, s));
            COLO_CUDA(cudaMemcpyAsync(b.get(), y1, n * 4, cudaMemcpyHostToDevice, s));
            COLO_CUDA(cudaMemcpyAsync(c.get(), x2, n * 4, cudaMemcpyHostToDevice, s));
            COLO_CUDA(cudaMemcpyAsync(d.get(), y2, n * 4, cudaMemcpyHostToDevice, s));
            eval_sqdist(a.get(), b.get(), c.get(), d.get(), n, o.get(), s, R2, within ? w.get() : nullptr);
            if (out) COLO_CUDA(cudaMemcpyAsync(out, o.get(), n * 4, cudaMemcpyDeviceToHost, s));
            if (within) COLO_CUDA(cudaMemcpyAsync(within, w.get(), n, cudaMemcpyDeviceToHost, s));
        }
        COLO_CUDA(cudaStreamSynchronize(s));
        return COLO_OK;
    });
}

static constexpr int kJoinWidths = COLO_JOIN_WIDTHS;

colo_status colo_autotune(colo_ctx* ctx, colo_dataset* ds, const colo_params* p, int32_t* join_group,
                          double* ms) {
    if (!ctx || !ds || !p) return COLO_ERR_ARG;
    return run_guarded(ctx, [&]() -> colo_status {
        static const int widths[kJoinWidths] = {1, 2, 4, 8, 16, 32};
        Batch b;
        std::vector<DevBuf<float>> of;
        colo_dataset* dsv[1] = {ds};
        setup_batch(ctx, dsv, p, 1, b, of, nullptr);
        int best = 8;
        double best_ms = 1e300, t[kJoinWidths] = {0, 0, 0, 0, 0, 0};
        if (b.N) {
            bucket_points(b);
            build_neighborhoods(b);
            cudaEvent_t e0, e1;
            COLO_CUDA(cudaEventCreate(&e0));
            COLO_CUDA(cudaEventCreate(&e1));
            for (int i = 0; i < kJoinWidths; ++i) {
                b.join_group = widths[i];
                join_neighbors(b);   // warm-up
                float tot = 0.f;
                for (int rep = 0; rep < 2; ++rep) {
                    COLO_CUDA(cudaEventRecord(e0, ctx->s));
                    join_neighbors(b);
                    COLO_CUDA(cudaEventRecord(e1, ctx->s));
                    COLO_CUDA(cudaEventSynchronize(e1));
                    float v = 0.f;
                    COLO_CUDA(cudaEventElapsedTime(&v, e0, e1));
                    tot += v;
                }
                t[i] = tot / 2.0;
                if (t[i] < best_ms) {
                    best_ms = t[i];
                    best = widths[i];
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        }
        ctx->join_group = best;
        if (join_group) *join_group = best;
        if (ms) std::memcpy(ms, t, sizeof(t));
        return COLO_OK;
    });
}

}  // extern "C"

namespace {

// ---- tuning cache ----------------------------------------------------------
// One text line per tuned dataset shape:
//   colo-tune 2 n=<points> f=<features> m=<occupied cells> r=<R float bits, hex> sms=<SMs> join=<lanes>
//   funit=<candidates per filter unit> lblock=<level threads per block> lqueue=<0|1>
// Lines that do not parse are skipped; a shape tuned twice keeps its first line.
struct TuneKey {
    uint64_t n = 0, f = 0, m = 0;
    uint32_t rbits = 0;
    int sms = 0;
    bool operator==(const TuneKey& o) const {
        return n == o.n && f == o.f && m == o.m && rbits == o.rbits && sms == o.sms;
    }
};

bool cache_lookup(const char* path, const TuneKey& key, colo_tuning* t) {
    FILE* fp = std::fopen(path, "r");
    if (!fp) return false;
    char line[512];
    bool hit = false;
    while (!hit && std::fgets(line, sizeof(line), fp)) {
        unsigned long long n, f, m;
        unsigned rb;
        int sms, j, u, lb, lq, ver;
        if (std::sscanf(line, "colo-tune %d n=%llu f=%llu m=%llu r=%x sms=%d join=%d funit=%d lblock=%d lqueue=%d",
                        &ver, &n, &f, &m, &rb, &sms, &j, &u, &lb, &lq) != 10 || ver != 2)
            continue;
        TuneKey k;
        k.n = n;
        k.f = f;
        k.m = m;
        k.rbits = rb;
        k.sms = sms;
        if (!(k == key)) continue;
        t->join_group = j;
        t->filter_unit = u;
        t->level_block = lb;
        t->level_queue = lq;
        hit = true;
    }
    std::fclose(fp);
    return hit;
}

bool cache_store(const char* path, const TuneKey& key, const colo_tuning& t) {
    FILE* fp = std::fopen(path, "a");
    if (!fp) return false;
    std::fprintf(fp, "colo-tune 2 n=%llu f=%llu m=%llu r=%08x sms=%d join=%d funit=%d lblock=%d lqueue=%d\n",
                 (unsigned long long)key.n, (unsigned long long)key.f, (unsigned long long)key.m, key.rbits, key.sms,
                 t.join_group, t.filter_unit, t.level_block, t.level_queue);
    return std::fclose(fp) == 0;
}

bool valid_tuning(const colo_tuning& t) {
    const int j = t.join_group, u = t.filter_unit, lb = t.level_block;
    const bool jok = j == 0 || j == 1 || j == 2 || j == 4 || j == 8 || j == 16 || j == 32;
    const bool uok = u == 0 || u == 8 || u == 16 || u == 32;
    const bool lok = lb == 0 || lb == 64 || lb == 128 || lb == 256;
    return jok && uok && lok && (t.level_queue == 0 || t.level_queue == 1);
}

// CUDA-event milliseconds of the kernel families whose names start with one of the prefixes,
// from one profiled mine (after one unprofiled warm-up mine).
colo_status time_families(colo_ctx* ctx, colo_dataset* ds, const colo_params* p,
                          std::initializer_list<const char*> prefixes, double* ms) {
    colo_params q = *p;
    q.reserved[0] |= 1;   // time every kernel
    q.keep_tables = 0;
    colo_result* r = nullptr;
    colo_status st = colo_mine(ctx, ds, p, &r);
    colo_result_free(r);
    if (st != COLO_OK) return st;
    r = nullptr;
    st = colo_mine(ctx, ds, &q, &r);
    if (st != COLO_OK) return st;
    double t = 0;
    for (const auto& k : r->r.kernels)
        for (const char* pre : prefixes)
            if (k.name.rfind(pre, 0) == 0) t += k.ms;
    colo_result_free(r);
    *ms = t;
    return COLO_OK;
}

}  // namespace

extern "C" {

colo_status colo_autotune_all(colo_ctx* ctx, colo_dataset* ds, const colo_params* p, const char* cache_path,
                              colo_tuning* out) {
    if (!ctx || !ds || !p) return COLO_ERR_ARG;
    TuneKey key;
    key.n = ds->hp.x.size();
    key.f = ds->names.size();
    std::memcpy(&key.rbits, &p->distance, 4);
    key.sms = ctx->sms;
    // the occupied cells of the dataset at this R (one bucketing pass)
    colo_status st = run_guarded(ctx, [&]() -> colo_status {
        Batch b;
        std::vector<DevBuf<float>> of;
        colo_dataset* dsv[1] = {ds};
        setup_batch(ctx, dsv, p, 1, b, of, nullptr);
        if (b.N) bucket_points(b);
        key.m = b.M;
        return COLO_OK;
    });
    if (st != COLO_OK) return st;
    colo_tuning t{};
    if (cache_path && cache_lookup(cache_path, key, &t) && valid_tuning(t)) {
        ctx->join_group = t.join_group;
        ctx->filter_unit = t.filter_unit;
        ctx->level_block = t.level_block;
        ctx->level_queue = t.level_queue;
        t.from_cache = 1;
        if (out) *out = t;
        return COLO_OK;
    }
    // lanes per anchor in the join
    int32_t jg = 8;
    st = colo_autotune(ctx, ds, p, &jg, nullptr);
    if (st != COLO_OK) return st;
    t.join_group = jg;
    // candidates per unit of the level filter, then threads per block of the level kernels,
    // each from the time of its own kernels in a whole mine
    const int units[3] = {8, 16, 32}, blocks[3] = {64, 128, 256};
    double best = 1e300;
    t.filter_unit = 32;
    for (int u : units) {
        ctx->filter_unit = u;
        double ms = 0;
        st = time_families(ctx, ds, p, {"filter_level"}, &ms);
        if (st != COLO_OK) return st;
        if (ms < best) {
            best = ms;
            t.filter_unit = u;
        }
    }
    ctx->filter_unit = t.filter_unit;
    best = 1e300;
    t.level_block = 256;
    for (int lb : blocks) {
        ctx->level_block = lb;
        double ms = 0;
        st = time_families(ctx, ds, p, {"level_"}, &ms);
        if (st != COLO_OK) return st;
        if (ms < best) {
            best = ms;
            t.level_block = lb;
        }
    }
    ctx->level_block = t.level_block;
    best = 1e300;
    t.level_queue = 0;
    for (int lq : {0, 1}) {
        ctx->level_queue = lq;
        double ms = 0;
        st = time_families(ctx, ds, p, {"level_"}, &ms);
        if (st != COLO_OK) return st;
        if (ms < best) {
            best = ms;
            t.level_queue = lq;
        }
    }
    ctx->level_queue = t.level_queue;
    t.from_cache = 0;
    if (cache_path && !cache_store(cache_path, key, t)) {
        ctx->err = std::string("cannot write the tuning cache ") + cache_path;
        return COLO_ERR_IO;
    }
    if (out) *out = t;
    return COLO_OK;
}

colo_status colo_set_tuning(colo_ctx* ctx, const colo_tuning* t) {
    if (!ctx || !t || !valid_tuning(*t)) return COLO_ERR_ARG;
    ctx->join_group = t->join_group;
    ctx->filter_unit = t->filter_unit;
    ctx->level_block = t->level_block;
    ctx->level_queue = t->level_queue;
    return COLO_OK;
}

colo_status colo_get_tuning(const colo_ctx* ctx, colo_tuning* t) {
    if (!ctx || !t) return COLO_ERR_ARG;
    t->join_group = ctx->join_group;
    t->filter_unit = ctx->filter_unit;
    t->level_block = ctx->level_block;
    t->level_queue = ctx->level_queue;
    t->from_cache = 0;
    return COLO_OK;
}

colo_status colo_set_join_group(colo_ctx* ctx, int32_t join_group) {
    if (!ctx) return COLO_ERR_ARG;
    if (join_group != 0 && join_group != 1 && join_group != 2 && join_group != 4 && join_group != 8 &&
        join_group != 16 && join_group != 32)
        return COLO_ERR_ARG;
    ctx->join_group = join_group;
    return COLO_OK;
}

}  // extern "C"
