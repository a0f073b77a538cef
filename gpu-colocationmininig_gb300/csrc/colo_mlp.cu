// colo_mlp.cu -- the learned cost model: a 24 -> 64 -> 64 -> 1 ReLU MLP with
// BF16 weights and activations and FP32 accumulation, trained and evaluated
// by hand-written tensor-core kernels (mma.sync.m16n8k16 BF16 -> FP32).
//
// It predicts log1p(instance-table rows) of a candidate from cell-aggregate
// statistics and only presizes output buffers / orders work; results never
// depend on it.
//
// Rounding points (mirrored by the CPU reference in the oracle): inputs,
// weights, H1, H2, dZ2 and dZ1 are rounded to BF16 before they enter a
// product; every product accumulates in FP32; biases, losses and updates
// stay FP32.
//
// Parameter layout (FP32 master copy, kMlpParams floats):
//   W1[32][64] (rows 24..31 zero), b1[64], W2[64][64], b2[64], W3[64], b3
#include <cuda_bf16.h>

#include "colo_internal.h"
#include "colo_mlp.h"

namespace colo {
namespace {

constexpr int IN = kMlpIn, INP = 32, H = 64;
constexpr int OFF_W1 = 0, OFF_B1 = INP * H, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H, OFF_W3 = OFF_B2 + H,
              OFF_B3 = OFF_W3 + H;
constexpr int kRowsPerWarp = 16, kWarps = 8, kRowsPerBlock = kRowsPerWarp * kWarps;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared weights: BF16, both orientations for the hidden layer.
struct SmemW {
    __nv_bfloat16 w1t[H][INP];   // [out][in]  (B operand of X.W1)
    __nv_bfloat16 w2t[H][H];     // [out][in]  (B operand of H1.W2)
    __nv_bfloat16 w2[H][H];      // [in][out]  (B operand of dZ2.W2^T)
    float b1[H], b2[H], w3[H];
    float b3;
};

__device__ void load_weights(SmemW& s, const float* __restrict__ P) {
    for (int i = threadIdx.x; i < INP * H; i += blockDim.x) {
        int in = i / H, o = i % H;
        s.w1t[o][in] = __float2bfloat16_rn(P[OFF_W1 + i]);
    }
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) {
        int in = i / H, o = i % H;
        __nv_bfloat16 v = __float2bfloat16_rn(P[OFF_W2 + i]);
        s.w2t[o][in] = v;
        s.w2[in][o] = v;
    }
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        s.b1[i] = P[OFF_B1 + i];
        s.b2[i] = P[OFF_B2 + i];
        s.w3[i] = bf16r(P[OFF_W3 + i]);
    }
    if (threadIdx.x == 0) s.b3 = P[OFF_B3];
}

// B fragment of a [N][K] row-major BF16 matrix for n-tile nt, k-tile kt.
template <int K>
__device__ __forceinline__ void bfrag(const __nv_bfloat16 (*m)[K], int nt, int kt, int gid, int tig, uint32_t& b0,
                                      uint32_t& b1) {
    const __nv_bfloat16* r = m[nt * 8 + gid] + kt * 16 + tig * 2;
    b0 = *reinterpret_cast<const uint32_t*>(r);
    b1 = *reinterpret_cast<const uint32_t*>(r + 8);
}

// Forward pass of one warp's 16 rows.  Outputs pre-activations (z1, z2) in
// accumulator layout and the prediction y for rows gid and gid+8.
__device__ __forceinline__ void forward16(const SmemW& s, const float* __restrict__ X,
                                          const uint32_t* __restrict__ idx, uint64_t row0, uint64_t n, int gid,
                                          int tig, float z1[8][4], float z2[8][4], float& y_lo, float& y_hi,
                                          uint32_t xa[2][4]) {
    // X tile -> A fragments (K = 32, 2 k-tiles)
    const uint64_t r_lo = row0 + gid, r_hi = row0 + gid + 8;
    const uint64_t x_lo = r_lo < n ? (idx ? idx[r_lo] : r_lo) : 0, x_hi = r_hi < n ? (idx ? idx[r_hi] : r_hi) : 0;
    for (int kt = 0; kt < 2; ++kt) {
        float v[8];
        for (int q = 0; q < 8; ++q) {
            int col = kt * 16 + (q >= 4 ? 8 : 0) + tig * 2 + (q & 1);
            uint64_t rr = (q & 2) ? r_hi : r_lo;
            uint64_t xr = (q & 2) ? x_hi : x_lo;
            v[q] = (col < IN && rr < n) ? X[xr * IN + col] : 0.0f;
        }
        xa[kt][0] = pack_bf16(v[0], v[1]);   // row gid,   cols tig*2..
        xa[kt][1] = pack_bf16(v[2], v[3]);   // row gid+8
        xa[kt][2] = pack_bf16(v[4], v[5]);   // row gid,   cols 8+tig*2..
        xa[kt][3] = pack_bf16(v[6], v[7]);   // row gid+8
    }
    for (int nt = 0; nt < 8; ++nt) {
        float bb0 = s.b1[nt * 8 + tig * 2], bb1 = s.b1[nt * 8 + tig * 2 + 1];
        z1[nt][0] = bb0;
        z1[nt][1] = bb1;
        z1[nt][2] = bb0;
        z1[nt][3] = bb1;
        for (int kt = 0; kt < 2; ++kt) {
            uint32_t b0, b1;
            bfrag<INP>(s.w1t, nt, kt, gid, tig, b0, b1);
            mma16816(z1[nt], xa[kt], b0, b1);
        }
    }
    // H1 = relu(z1) -> A fragments (K = 64, 4 k-tiles)
    uint32_t ha[4][4];
    for (int kt = 0; kt < 4; ++kt) {
        const float* c0 = z1[2 * kt];
        const float* c1 = z1[2 * kt + 1];
        ha[kt][0] = pack_bf16(fmaxf(c0[0], 0.f), fmaxf(c0[1], 0.f));
        ha[kt][1] = pack_bf16(fmaxf(c0[2], 0.f), fmaxf(c0[3], 0.f));
        ha[kt][2] = pack_bf16(fmaxf(c1[0], 0.f), fmaxf(c1[1], 0.f));
        ha[kt][3] = pack_bf16(fmaxf(c1[2], 0.f), fmaxf(c1[3], 0.f));
    }
    for (int nt = 0; nt < 8; ++nt) {
        float bb0 = s.b2[nt * 8 + tig * 2], bb1 = s.b2[nt * 8 + tig * 2 + 1];
        z2[nt][0] = bb0;
        z2[nt][1] = bb1;
        z2[nt][2] = bb0;
        z2[nt][3] = bb1;
        for (int kt = 0; kt < 4; ++kt) {
            uint32_t b0, b1;
            bfrag<H>(s.w2t, nt, kt, gid, tig, b0, b1);
            mma16816(z2[nt], ha[kt], b0, b1);
        }
    }
    // y = bf16(relu(z2)) . w3 + b3, reduced over the 4 lanes of a row quad
    float plo = 0.f, phi = 0.f;
    for (int nt = 0; nt < 8; ++nt)
        for (int e = 0; e < 2; ++e) {
            int col = nt * 8 + tig * 2 + e;
            plo += bf16r(fmaxf(z2[nt][e], 0.f)) * s.w3[col];
            phi += bf16r(fmaxf(z2[nt][2 + e], 0.f)) * s.w3[col];
        }
    plo += __shfl_xor_sync(0xffffffffu, plo, 1);
    plo += __shfl_xor_sync(0xffffffffu, plo, 2);
    phi += __shfl_xor_sync(0xffffffffu, phi, 1);
    phi += __shfl_xor_sync(0xffffffffu, phi, 2);
    y_lo = plo + s.b3;
    y_hi = phi + s.b3;
}

__global__ void __launch_bounds__(256) k_mlp_forward(const float* __restrict__ P, const float* __restrict__ X,
                                                     uint64_t n, float* __restrict__ y) {
    __shared__ SmemW s;
    load_weights(s, P);
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, gid = lane >> 2, tig = lane & 3;
    for (uint64_t row0 = ((uint64_t)blockIdx.x * kWarps + w) * kRowsPerWarp; row0 < n;
         row0 += (uint64_t)gridDim.x * kRowsPerBlock) {
        float z1[8][4], z2[8][4], ylo, yhi;
        uint32_t xa[2][4];
        forward16(s, X, nullptr, row0, n, gid, tig, z1, z2, ylo, yhi, xa);
        if (tig == 0) {
            if (row0 + gid < n) y[row0 + gid] = ylo;
            if (row0 + gid + 8 < n) y[row0 + gid + 8] = yhi;
        }
    }
}

// Shared memory of the gradient kernel (dynamic: about 100 KB).
struct GradSmem {
    SmemW w;
    float gw1[INP * H], gw2[H * H], gb1[H], gb2[H], gw3[H], gb3, lsum;
    __nv_bfloat16 h1s[kWarps][16][H], dz2s[kWarps][16][H], dz1s[kWarps][16][H], xs[kWarps][16][INP];
};

__device__ __forceinline__ float quad_sum(float v) {   // sum over the 8 lanes sharing tig
    for (int o = 4; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Forward + backward of a mini-batch; gradients of the mean of 0.5*(y-t)^2
// over `n` rows (rows idx[r], or r when idx is null) accumulate (FP32
// atomics) into G (kMlpParams floats).
__global__ void __launch_bounds__(256) k_mlp_grad(const float* __restrict__ P, const float* __restrict__ X,
                                                  const float* __restrict__ T, const uint32_t* __restrict__ idx,
                                                  uint64_t n, float inv_n, float* __restrict__ G,
                                                  float* __restrict__ loss) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GradSmem& S = *reinterpret_cast<GradSmem*>(smem_raw);
    const SmemW& s = S.w;
    load_weights(S.w, P);
    for (int i = threadIdx.x; i < INP * H; i += blockDim.x) S.gw1[i] = 0.f;
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) S.gw2[i] = 0.f;
    for (int i = threadIdx.x; i < H; i += blockDim.x) S.gb1[i] = S.gb2[i] = S.gw3[i] = 0.f;
    if (threadIdx.x == 0) S.gb3 = S.lsum = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, gid = lane >> 2, tig = lane & 3;
    for (uint64_t row0 = ((uint64_t)blockIdx.x * kWarps + w) * kRowsPerWarp; row0 < n;
         row0 += (uint64_t)gridDim.x * kRowsPerBlock) {
        float z1[8][4], z2[8][4], ylo, yhi;
        uint32_t xa[2][4];
        forward16(s, X, idx, row0, n, gid, tig, z1, z2, ylo, yhi, xa);
        const bool vlo = row0 + gid < n, vhi = row0 + gid + 8 < n;
        const float tlo = vlo ? T[idx ? idx[row0 + gid] : row0 + gid] : 0.f;
        const float thi = vhi ? T[idx ? idx[row0 + gid + 8] : row0 + gid + 8] : 0.f;
        const float dlo = vlo ? (ylo - tlo) * inv_n : 0.f;
        const float dhi = vhi ? (yhi - thi) * inv_n : 0.f;
        {
            // loss and db3 over the 16 rows: lanes with tig == 0 hold one row pair each
            float l = tig == 0 ? ((vlo ? 0.5f * (ylo - tlo) * (ylo - tlo) : 0.f) +
                                  (vhi ? 0.5f * (yhi - thi) * (yhi - thi) : 0.f)) * inv_n
                               : 0.f;
            float g = tig == 0 ? dlo + dhi : 0.f;
            for (int o = 1; o < 32; o <<= 1) {
                l += __shfl_xor_sync(0xffffffffu, l, o);
                g += __shfl_xor_sync(0xffffffffu, g, o);
            }
            if (lane == 0) {
                atomicAdd(&S.lsum, l);
                atomicAdd(&S.gb3, g);
            }
        }
        // layer 3: dW3 = H2b^T dy; dZ2 = dy * w3 * (z2 > 0)
        float dz2[8][4];
        for (int nt = 0; nt < 8; ++nt)
            for (int e = 0; e < 2; ++e) {
                int col = nt * 8 + tig * 2 + e;
                float h_lo = bf16r(fmaxf(z2[nt][e], 0.f)), h_hi = bf16r(fmaxf(z2[nt][2 + e], 0.f));
                float g = quad_sum(h_lo * dlo + h_hi * dhi);
                if (gid == 0) atomicAdd(&S.gw3[col], g);
                dz2[nt][e] = z2[nt][e] > 0.f ? dlo * s.w3[col] : 0.f;
                dz2[nt][2 + e] = z2[nt][2 + e] > 0.f ? dhi * s.w3[col] : 0.f;
            }
        // stash H1b, dZ2b, X (BF16) for the transposed weight-gradient products
        for (int nt = 0; nt < 8; ++nt)
            for (int e = 0; e < 2; ++e) {
                int col = nt * 8 + tig * 2 + e;
                S.h1s[w][gid][col] = __float2bfloat16_rn(fmaxf(z1[nt][e], 0.f));
                S.h1s[w][gid + 8][col] = __float2bfloat16_rn(fmaxf(z1[nt][2 + e], 0.f));
                S.dz2s[w][gid][col] = __float2bfloat16_rn(dz2[nt][e]);
                S.dz2s[w][gid + 8][col] = __float2bfloat16_rn(dz2[nt][2 + e]);
            }
        for (int kt = 0; kt < 2; ++kt) {
            *reinterpret_cast<uint32_t*>(&S.xs[w][gid][kt * 16 + tig * 2]) = xa[kt][0];
            *reinterpret_cast<uint32_t*>(&S.xs[w][gid + 8][kt * 16 + tig * 2]) = xa[kt][1];
            *reinterpret_cast<uint32_t*>(&S.xs[w][gid][kt * 16 + 8 + tig * 2]) = xa[kt][2];
            *reinterpret_cast<uint32_t*>(&S.xs[w][gid + 8][kt * 16 + 8 + tig * 2]) = xa[kt][3];
        }
        // db2 = sum over rows of dZ2
        for (int nt = 0; nt < 8; ++nt)
            for (int e = 0; e < 2; ++e) {
                float g = quad_sum(dz2[nt][e] + dz2[nt][2 + e]);
                if (gid == 0) atomicAdd(&S.gb2[nt * 8 + tig * 2 + e], g);
            }
        __syncwarp();
        // dH1 = dZ2b . W2^T  (A = dZ2b from the accumulator layout)
        uint32_t da[4][4];
        for (int kt = 0; kt < 4; ++kt) {
            const float* c0 = dz2[2 * kt];
            const float* c1 = dz2[2 * kt + 1];
            da[kt][0] = pack_bf16(c0[0], c0[1]);
            da[kt][1] = pack_bf16(c0[2], c0[3]);
            da[kt][2] = pack_bf16(c1[0], c1[1]);
            da[kt][3] = pack_bf16(c1[2], c1[3]);
        }
        for (int nt = 0; nt < 8; ++nt) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            for (int kt = 0; kt < 4; ++kt) {
                uint32_t b0, b1;
                bfrag<H>(s.w2, nt, kt, gid, tig, b0, b1);
                mma16816(acc, da[kt], b0, b1);
            }
            // dZ1 = dH1 * (z1 > 0); db1; stash BF16
            for (int e = 0; e < 2; ++e) {
                int col = nt * 8 + tig * 2 + e;
                float lo = z1[nt][e] > 0.f ? acc[e] : 0.f;
                float hi = z1[nt][2 + e] > 0.f ? acc[2 + e] : 0.f;
                S.dz1s[w][gid][col] = __float2bfloat16_rn(lo);
                S.dz1s[w][gid + 8][col] = __float2bfloat16_rn(hi);
                float g = quad_sum(lo + hi);
                if (gid == 0) atomicAdd(&S.gb1[col], g);
            }
        }
        __syncwarp();
        // dW2[in][out] = sum_r H1b[r][in] * dZ2b[r][out]: M = in (4 tiles), N = out (8 tiles), K = 16 rows
        const int k0 = tig * 2;
        for (int mt = 0; mt < 4; ++mt) {
            const int m0 = mt * 16 + gid, m1 = m0 + 8;
            uint32_t a[4];
            a[0] = pack_bf16(__bfloat162float(S.h1s[w][k0][m0]), __bfloat162float(S.h1s[w][k0 + 1][m0]));
            a[1] = pack_bf16(__bfloat162float(S.h1s[w][k0][m1]), __bfloat162float(S.h1s[w][k0 + 1][m1]));
            a[2] = pack_bf16(__bfloat162float(S.h1s[w][k0 + 8][m0]), __bfloat162float(S.h1s[w][k0 + 9][m0]));
            a[3] = pack_bf16(__bfloat162float(S.h1s[w][k0 + 8][m1]), __bfloat162float(S.h1s[w][k0 + 9][m1]));
            for (int nt = 0; nt < 8; ++nt) {
                const int nn = nt * 8 + gid;
                uint32_t b0 = pack_bf16(__bfloat162float(S.dz2s[w][k0][nn]), __bfloat162float(S.dz2s[w][k0 + 1][nn]));
                uint32_t b1 = pack_bf16(__bfloat162float(S.dz2s[w][k0 + 8][nn]), __bfloat162float(S.dz2s[w][k0 + 9][nn]));
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
                mma16816(acc, a, b0, b1);
                const int col = nt * 8 + tig * 2;
                atomicAdd(&S.gw2[m0 * H + col], acc[0]);
                atomicAdd(&S.gw2[m0 * H + col + 1], acc[1]);
                atomicAdd(&S.gw2[m1 * H + col], acc[2]);
                atomicAdd(&S.gw2[m1 * H + col + 1], acc[3]);
            }
        }
        // dW1[in][out] = sum_r Xb[r][in] * dZ1b[r][out]: M = in (2 tiles), N = out (8 tiles)
        for (int mt = 0; mt < 2; ++mt) {
            const int m0 = mt * 16 + gid, m1 = m0 + 8;
            uint32_t a[4];
            a[0] = pack_bf16(__bfloat162float(S.xs[w][k0][m0]), __bfloat162float(S.xs[w][k0 + 1][m0]));
            a[1] = pack_bf16(__bfloat162float(S.xs[w][k0][m1]), __bfloat162float(S.xs[w][k0 + 1][m1]));
            a[2] = pack_bf16(__bfloat162float(S.xs[w][k0 + 8][m0]), __bfloat162float(S.xs[w][k0 + 9][m0]));
            a[3] = pack_bf16(__bfloat162float(S.xs[w][k0 + 8][m1]), __bfloat162float(S.xs[w][k0 + 9][m1]));
            for (int nt = 0; nt < 8; ++nt) {
                const int nn = nt * 8 + gid;
                uint32_t b0 = pack_bf16(__bfloat162float(S.dz1s[w][k0][nn]), __bfloat162float(S.dz1s[w][k0 + 1][nn]));
                uint32_t b1 = pack_bf16(__bfloat162float(S.dz1s[w][k0 + 8][nn]), __bfloat162float(S.dz1s[w][k0 + 9][nn]));
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
                mma16816(acc, a, b0, b1);
                const int col = nt * 8 + tig * 2;
                atomicAdd(&S.gw1[m0 * H + col], acc[0]);
                atomicAdd(&S.gw1[m0 * H + col + 1], acc[1]);
                atomicAdd(&S.gw1[m1 * H + col], acc[2]);
                atomicAdd(&S.gw1[m1 * H + col + 1], acc[3]);
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (int i = threadIdx.x; i < IN * H; i += blockDim.x) atomicAdd(&G[OFF_W1 + i], S.gw1[i]);   // rows >= 24 stay 0
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) atomicAdd(&G[OFF_W2 + i], S.gw2[i]);
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        atomicAdd(&G[OFF_B1 + i], S.gb1[i]);
        atomicAdd(&G[OFF_B2 + i], S.gb2[i]);
        atomicAdd(&G[OFF_W3 + i], S.gw3[i]);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&G[OFF_B3], S.gb3);
        atomicAdd(loss, S.lsum);
    }
}

__global__ void k_adam(float* __restrict__ P, float* __restrict__ G, float* __restrict__ m1, float* __restrict__ m2,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = G[i];
    G[i] = 0.f;
    float a = m1[i] = b1 * m1[i] + (1.f - b1) * g;
    float v = m2[i] = b2 * m2[i] + (1.f - b2) * g * g;
    P[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

__global__ void k_zero_pad_rows(float* P) {
    int i = threadIdx.x;
    for (int r = IN; r < INP; ++r)
        if (i < H) P[OFF_W1 + r * H + i] = 0.f;
}

// Cost-model features of level-k candidates (the layout colo_result_features
// documents), from the filter's bounds and quad statistics on the device.
__global__ void k_features(uint64_t ncand, uint32_t k, const uint32_t* __restrict__ cand,
                           const uint32_t* __restrict__ ub, const unsigned long long* __restrict__ fstats,
                           const uint32_t* __restrict__ fcount, const uint64_t* __restrict__ prow,
                           float* __restrict__ X) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncand) return;
    const uint32_t* mem = cand + c * k;
    const uint32_t m = k < 8 ? k : 8;
    float x[IN];
    for (int i = 0; i < IN; ++i) x[i] = 0.f;
    x[0] = (float)k / 8.0f;
    float minn = INFINITY, minub = INFINITY;
    for (uint32_t j = 0; j < k; ++j) minn = fminf(minn, (float)fcount[mem[j]]);
    for (uint32_t j = 0; j < m; ++j) {
        const float u = (float)ub[c * k + j];
        x[1 + j] = log1pf((float)fcount[mem[j]]);
        x[9 + j] = log1pf(u);
        minub = fminf(minub, u);
    }
    const float lnl = log1pf((float)fcount[mem[k - 1]]), lpr = log1pf((float)prow[c]);
    x[17] = lpr;
    x[18] = log1pf(fstats ? (float)fstats[c * 2 + 1] : 0.f);
    x[19] = log1pf(fstats ? (float)fstats[c * 2] : 0.f);
    x[20] = log1pf(minn);
    x[21] = log1pf(minub);
    x[22] = lpr - lnl;
    x[23] = k <= 8 ? log1pf((float)ub[c * k + k - 1]) - lnl : 0.f;
    for (int i = 0; i < IN; ++i) X[c * IN + i] = x[i];
}

}  // namespace

void mlp_features(uint64_t ncand, uint32_t k, const uint32_t* d_cand, const uint32_t* d_ub,
                  const unsigned long long* d_fstats, const uint32_t* d_fcount, const uint64_t* d_prow, float* d_x,
                  cudaStream_t s) {
    if (ncand == 0) return;
    KScope ks("mlp_features");
    k_features<<<(unsigned)((ncand + 127) / 128), 128, 0, s>>>(ncand, k, d_cand, d_ub, d_fstats, d_fcount, d_prow,
                                                               d_x);
    COLO_LAUNCH_CHECK();
    count_launch();
}

void mlp_forward(const float* d_params, const float* d_x, uint64_t n, float* d_y, cudaStream_t s) {
    if (n == 0) return;
    uint64_t blocks = (n + kRowsPerBlock - 1) / kRowsPerBlock;
    if (blocks > 4096) blocks = 4096;
    KScope ks("mlp_forward");
    k_mlp_forward<<<(unsigned)blocks, 256, 0, s>>>(d_params, d_x, n, d_y);
    COLO_LAUNCH_CHECK();
    count_launch();
}

void mlp_grad(const float* d_params, const float* d_x, const float* d_t, const uint32_t* d_idx, uint64_t n,
              float* d_grad, float* d_loss, cudaStream_t s) {
    if (n == 0) return;
    static thread_local int attr_dev = -1;
    int dev = 0;
    COLO_CUDA(cudaGetDevice(&dev));
    if (attr_dev != dev) {
        COLO_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GradSmem)));
        attr_dev = dev;
    }
    uint64_t blocks = (n + kRowsPerBlock - 1) / kRowsPerBlock;
    if (blocks > 1024) blocks = 1024;
    KScope ks("mlp_grad");
    k_mlp_grad<<<(unsigned)blocks, 256, sizeof(GradSmem), s>>>(d_params, d_x, d_t, d_idx, n, 1.0f / (float)n, d_grad,
                                                                d_loss);
    COLO_LAUNCH_CHECK();
    count_launch();
}

void mlp_adam(float* d_params, float* d_grad, float* d_m1, float* d_m2, int step, float lr, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    KScope ks("mlp_adam");
    k_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(d_params, d_grad, d_m1, d_m2, kMlpParams, lr, b1, b2, 1e-8f, c1, c2);
    COLO_LAUNCH_CHECK();
    k_zero_pad_rows<<<1, 64, 0, s>>>(d_params);
    COLO_LAUNCH_CHECK();
    count_launch(2);
}

}  // namespace colo
