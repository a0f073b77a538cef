// colo_mlp.h -- the learned cost model's tensor-core kernels (colo_mlp.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace colo {

constexpr int kMlpIn = 24;       // features per candidate
constexpr int kMlpHidden = 64;
// W1[32][64] (input rows 24..31 zero) + b1[64] + W2[64][64] + b2[64] + W3[64] + b3
constexpr int kMlpParams = 32 * 64 + 64 + 64 * 64 + 64 + 64 + 1;

// Features of ncand level-k candidates (device arrays: members cand[c*k+j],
// filter bounds ub[c*k+j], quad statistics fstats[c*2..] (may be null),
// feature sizes, parent rows) into x[c*24 ..].
void mlp_features(uint64_t ncand, uint32_t k, const uint32_t* d_cand, const uint32_t* d_ub,
                  const unsigned long long* d_fstats, const uint32_t* d_fcount, const uint64_t* d_prow, float* d_x,
                  cudaStream_t s);
// y[i] = model(x[i*24 .. i*24+23]) for n rows (device pointers).
void mlp_forward(const float* d_params, const float* d_x, uint64_t n, float* d_y, cudaStream_t s);
// Adds the gradient of mean_i 0.5*(y_i - t_i)^2 over rows idx[0..n) (or 0..n
// when idx is null) to d_grad and the loss to *d_loss.
void mlp_grad(const float* d_params, const float* d_x, const float* d_t, const uint32_t* d_idx, uint64_t n,
              float* d_grad, float* d_loss, cudaStream_t s);
// One Adam step (beta 0.9 / 0.999, eps 1e-8) at step `step` (1-based); zeroes d_grad.
void mlp_adam(float* d_params, float* d_grad, float* d_m1, float* d_m2, int step, float lr, cudaStream_t s);

}  // namespace colo
