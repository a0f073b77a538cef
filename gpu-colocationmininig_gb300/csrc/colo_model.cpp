// colo_model.cpp -- C entry points of the learned cost model: evaluation,
// gradients, GPU training, installing a trained model in a context, and the
// per-candidate features the mining loop records for training.
//
// The model predicts log1p(instance-table rows) of a candidate that passed
// the filter.  In COLO_MODE_LEARNED the prediction presizes the single-pass
// table buffers and orders the level queue; results never depend on it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "colo_host.h"
#include "colo_mlp.h"

using namespace colo;

namespace colo {

// Features of one candidate (colo_result_features documents the layout).
void candidate_features(uint32_t k, const uint32_t* mem, const uint32_t* fcount, const uint64_t* ub,
                        uint64_t prow, uint64_t fquads, uint64_t fcells, float* x) {
    auto lg = [](double v) { return std::log1p((float)v); };
    const uint32_t m = std::min<uint32_t>(k, kMaxMembersFiltered);
    for (int i = 0; i < kMlpIn; ++i) x[i] = 0.f;
    x[0] = (float)k / 8.0f;
    double minn = INFINITY, minub = INFINITY;
    for (uint32_t j = 0; j < k; ++j) minn = std::min(minn, (double)fcount[mem[j]]);
    for (uint32_t j = 0; j < m; ++j) {
        x[1 + j] = lg(fcount[mem[j]]);
        x[9 + j] = lg((double)ub[j]);
        minub = std::min(minub, (double)ub[j]);
    }
    const double nlast = fcount[mem[k - 1]];
    x[17] = lg((double)prow);
    x[18] = lg((double)fcells);
    x[19] = lg((double)fquads);
    x[20] = lg(minn);
    x[21] = lg(minub);
    x[22] = lg((double)prow) - lg(nlast);
    x[23] = k <= (uint32_t)kMaxMembersFiltered ? lg((double)ub[k - 1]) - lg(nlast) : 0.f;
}

}  // namespace colo

namespace {

colo_status check_ctx(colo_ctx* ctx) { return ctx ? COLO_OK : COLO_ERR_ARG; }

}  // namespace

extern "C" {

colo_status colo_model_forward(colo_ctx* ctx, const float* params, const float* x, uint64_t n, float* y) {
    if (check_ctx(ctx) != COLO_OK || !params || (n && (!x || !y))) return COLO_ERR_ARG;
    return run_guarded(ctx, [&]() -> colo_status {
        cudaStream_t s = ctx->s;
        DevBuf<float> dp, dx, dy;
        dp.alloc(kMlpParams, s);
        dx.alloc(n * kMlpIn, s);
        dy.alloc(n, s);
        COLO_CUDA(cudaMemcpyAsync(dp.get(), params, kMlpParams * 4, cudaMemcpyHostToDevice, s));
        if (n) {
            COLO_CUDA(cudaMemcpyAsync(dx.get(), x, n * kMlpIn * 4, cudaMemcpyHostToDevice, s));
            mlp_forward(dp.get(), dx.get(), n, dy.get(), s);
            COLO_CUDA(cudaMemcpyAsync(y, dy.get(), n * 4, cudaMemcpyDeviceToHost, s));
        }
        COLO_CUDA(cudaStreamSynchronize(s));
        return COLO_OK;
    });
}

colo_status colo_model_grad(colo_ctx* ctx, const float* params, const float* x, const float* t, uint64_t n,
                            float* grad, float* loss) {
    if (check_ctx(ctx) != COLO_OK || !params || !grad || (n && (!x || !t))) return COLO_ERR_ARG;
    return run_guarded(ctx, [&]() -> colo_status {
        cudaStream_t s = ctx->s;
        DevBuf<float> dp, dx, dt, dg, dl;
        dp.alloc(kMlpParams, s);
        dg.alloc(kMlpParams, s);
        dl.alloc(1, s);
        dg.zero(s);
        dl.zero(s);
        COLO_CUDA(cudaMemcpyAsync(dp.get(), params, kMlpParams * 4, cudaMemcpyHostToDevice, s));
        if (n) {
            dx.alloc(n * kMlpIn, s);
            dt.alloc(n, s);
            COLO_CUDA(cudaMemcpyAsync(dx.get(), x, n * kMlpIn * 4, cudaMemcpyHostToDevice, s));
            COLO_CUDA(cudaMemcpyAsync(dt.get(), t, n * 4, cudaMemcpyHostToDevice, s));
            mlp_grad(dp.get(), dx.get(), dt.get(), nullptr, n, dg.get(), dl.get(), s);
        }
        COLO_CUDA(cudaMemcpyAsync(grad, dg.get(), kMlpParams * 4, cudaMemcpyDeviceToHost, s));
        float l = 0.f;
        COLO_CUDA(cudaMemcpyAsync(&l, dl.get(), 4, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaStreamSynchronize(s));
        if (loss) *loss = l;
        return COLO_OK;
    });
}

colo_status colo_model_train(colo_ctx* ctx, float* params, const float* x, const float* t, uint64_t n,
                             uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float* epoch_loss) {
    if (check_ctx(ctx) != COLO_OK || !params || !x || !t || n == 0 || batch == 0) return COLO_ERR_ARG;
    if (n >= (1ull << 32)) return COLO_ERR_CAPACITY;
    return run_guarded(ctx, [&]() -> colo_status {
        cudaStream_t s = ctx->s;
        DevBuf<float> dp, dx, dt, dg, m1, m2, dl;
        DevBuf<uint32_t> didx;
        dp.alloc(kMlpParams, s);
        dg.alloc(kMlpParams, s);
        m1.alloc(kMlpParams, s);
        m2.alloc(kMlpParams, s);
        dl.alloc(epochs ? epochs : 1, s);
        dx.alloc(n * kMlpIn, s);
        dt.alloc(n, s);
        didx.alloc(n, s);
        dg.zero(s);
        m1.zero(s);
        m2.zero(s);
        dl.zero(s);
        COLO_CUDA(cudaMemcpyAsync(dp.get(), params, kMlpParams * 4, cudaMemcpyHostToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(dx.get(), x, n * kMlpIn * 4, cudaMemcpyHostToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(dt.get(), t, n * 4, cudaMemcpyHostToDevice, s));
        std::vector<uint32_t> perm(n);
        for (uint64_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
        std::mt19937_64 rng(seed);
        int step = 0;
        const uint64_t steps = (n + batch - 1) / batch;
        for (uint32_t e = 0; e < epochs; ++e) {
            std::shuffle(perm.begin(), perm.end(), rng);
            COLO_CUDA(cudaMemcpyAsync(didx.get(), perm.data(), n * 4, cudaMemcpyHostToDevice, s));
            for (uint64_t b0 = 0; b0 < n; b0 += batch) {
                const uint64_t nb = std::min<uint64_t>(batch, n - b0);
                mlp_grad(dp.get(), dx.get(), dt.get(), didx.get() + b0, nb, dg.get(), dl.get() + e, s);
                mlp_adam(dp.get(), dg.get(), m1.get(), m2.get(), ++step, lr, s);
            }
            // the host permutation is rewritten next epoch: wait for this one's copy
            COLO_CUDA(cudaStreamSynchronize(s));
        }
        COLO_CUDA(cudaMemcpyAsync(params, dp.get(), kMlpParams * 4, cudaMemcpyDeviceToHost, s));
        std::vector<float> hl(epochs);
        if (epochs) COLO_CUDA(cudaMemcpyAsync(hl.data(), dl.get(), epochs * 4, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaStreamSynchronize(s));
        if (epoch_loss)
            for (uint32_t e = 0; e < epochs; ++e) epoch_loss[e] = hl[e] / (float)steps;
        return COLO_OK;
    });
}

colo_status colo_ctx_set_model(colo_ctx* ctx, const float* params) {
    if (!ctx) return COLO_ERR_ARG;
    if (!params) {
        ctx->model.clear();
        return COLO_OK;
    }
    for (int i = 0; i < kMlpParams; ++i)
        if (!std::isfinite(params[i])) return set_err(ctx, COLO_ERR_ARG, "model parameters must be finite");
    ctx->model.assign(params, params + kMlpParams);
    return COLO_OK;
}

colo_status colo_result_features(const colo_result* r, uint32_t li, float* x) {
    if (!r || !x || li >= r->r.levels.size()) return COLO_ERR_ARG;
    const LevelTrace& L = r->r.levels[li];
    if (!L.feat.empty()) std::memcpy(x, L.feat.data(), L.feat.size() * sizeof(float));
    else std::memset(x, 0, L.cand.size() / (L.k ? L.k : 1) * kMlpIn * sizeof(float));
    return COLO_OK;
}

}  // extern "C"
