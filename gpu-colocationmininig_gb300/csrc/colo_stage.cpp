// colo_stage.cpp -- stage-level C entry points (one kernel family each), the
// counterparts of the reference's inner extern "C" API
// (Codes/DeviceProcess.h:4-36).  They run one stage on a dataset and copy
// its result to host arrays, so each kernel can be checked in isolation.
#include <algorithm>
#include <cstring>
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
                if (nbr) std::memcpy(nbr + o, all.data() + beg[a], cnt[a] * 4);
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

colo_status colo_set_join_group(colo_ctx* ctx, int32_t join_group) {
    if (!ctx) return COLO_ERR_ARG;
    if (join_group != 0 && join_group != 1 && join_group != 2 && join_group != 4 && join_group != 8 &&
        join_group != 16 && join_group != 32)
        return COLO_ERR_ARG;
    ctx->join_group = join_group;
    return COLO_OK;
}

}  // extern "C"
