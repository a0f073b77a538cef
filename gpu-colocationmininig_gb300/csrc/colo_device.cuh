// colo_device.cuh -- device helpers shared by the kernels of libcolo.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "colo_internal.h"

namespace colo {

// Squared distance with the reference's own expression
// (Codes/Utility_Inline.h:25-33: x1,y1 = first instance, x2,y2 = second).
// The text is kept alike on purpose: the neighbour relation must be
// bit-identical, and the device pow(float, int) it calls is CUDA's.
__device__ __forceinline__ float ref_sqdist(float x1, float y1, float x2, float y2) {
    float squareDistance = pow((x2 - x1), 2) + pow((y2 - y1), 2);
    return squareDistance;
}

// The reference's neighbour test ref_sqdist(...) <= R2, decided with two
// FP32 FMAs whenever the exact squared distance S is clearly away from the
// boundary, and with the reference expression itself otherwise.
//
// The reference value is the float nearest to S (pow is evaluated in double
// and the sum rounded to float once), so it is <= R2 exactly when S lies
// below the midpoint R2 + hu between R2 and the next float (hu = half an ulp
// of R2).  t2 = fma(dx, dx, fma(dy, dy, -R2)) approximates S - R2 with an
// error below 2^-24 (|t1| + |t2|); eps is that bound with an 8x margin plus
// the rounding of the comparisons.  Inside the band the expression itself
// decides, so the result equals ref_sqdist(...) <= R2 for every input.
__device__ __forceinline__ bool ref_within(float x1, float y1, float x2, float y2, float R2, float hu) {
    const float dx = x2 - x1, dy = y2 - y1;
    const float t1 = __fmaf_rn(dy, dy, -R2);
    const float t2 = __fmaf_rn(dx, dx, t1);
    const float eps = (fabsf(t1) + fabsf(t2) + hu) * 4.8e-7f + 1e-37f;
    if (t2 < hu - eps) return true;
    if (t2 > hu + eps) return false;
    return ref_sqdist(x1, y1, x2, y2) <= R2;
}

// Cell of a point (Codes/DeviceProcess_Kernel.h:615-625): float subtract,
// float divide, float->u32 conversion (saturating on the device).
__device__ __forceinline__ uint64_t ref_cell(const JobGrid& g, float x, float y) {
    float rx = x - g.min_x;
    float ry = y - g.min_y;
    rx /= g.w;
    ry /= g.w;
    uint32_t i = (uint32_t)rx;
    uint32_t j = (uint32_t)ry;
    uint64_t c = (uint64_t)g.gx * j + i;
    if (g.compat32) c = (uint32_t)c;
    return c;
}

// The reference's neighbour-cell rule (Codes/Utility_Inline.h:35-53 with the
// stencil loops): an in-range geometric neighbour (nx, ny) of cell column cx
// is visited unless the column-wrap tests drop it.  Out-of-range neighbours
// are never visited.
__device__ __forceinline__ bool ref_adjacent_col(uint32_t cx, uint32_t nx, uint32_t gx) {
    if (cx == 0) return nx != gx - 1;
    if (cx == gx - 1) return nx != 0;
    return true;
}

template <class T>
__device__ __forceinline__ uint64_t lower_bound_dev(const T* a, uint64_t lo, uint64_t hi, T v) {
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Number of set bits of the W-word mask m below bit b.  A cell's runs ascend
// by feature and its mask has one bit per feature present, so for local
// feature b the run index in the cell is crun + mask_rank(mask, b).
__device__ __forceinline__ uint32_t mask_rank(const uint32_t* __restrict__ m, uint32_t b) {
    const uint32_t wq = b >> 5;
    uint32_t r = 0;
    for (uint32_t w = 0; w < wq; ++w) r += __popc(m[w]);
    return r + __popc(m[wq] & ((1u << (b & 31)) - 1u));
}

// Column and row of a cell from its id within its grid (id = row * gx + col):
// a 32-bit division when the id fits, which every grid of fewer than 2^32
// cells does, else the 64-bit one.
__device__ __forceinline__ void cell_col_row(uint64_t local, uint32_t gx, uint64_t& cx, uint64_t& cy) {
    if (local < (1ull << 32)) {
        const uint32_t l = (uint32_t)local, r = l / gx;
        cy = r;
        cx = l - r * gx;
    } else {
        cy = local / gx;
        cx = local - cy * gx;
    }
}

// A point's feature is the last feature whose first point is at or before it
// (points are grouped by feature); the start table stays in L1.
__device__ __forceinline__ uint32_t feature_of(uint32_t id, uint32_t F, const uint32_t* __restrict__ fstart) {
    uint32_t lo = 0, hi = F;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (fstart[mid] <= id) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    return (1u << (threadIdx.x & 31)) - 1u;
}

// 32 x 32 bit transpose across a full warp: lane i holds row i (bit j =
// column j); afterwards lane j holds column j (bit i = row i's bit j).  Five
// block swaps of halving size: at size s, lanes without bit s take their
// partner's low s-bit groups into their high ones, lanes with bit s the
// partner's high groups into their low ones.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
    const uint32_t lane = threadIdx.x & 31;
    constexpr uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const int s = 16 >> i;
        const uint32_t m = masks[i];
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, s);
        x = (lane & (uint32_t)s) ? ((x & ~m) | ((y >> s) & m)) : ((x & m) | ((y & m) << s));
    }
    return x;
}

// Warp and block scans (one value per thread).
template <class T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive block scan of one value per thread; returns the exclusive prefix
// and writes the block total to *total.
template <class T>
__device__ __forceinline__ T block_excl_scan(T v, T* total) {
    __shared__ T warp_tot[33];   // [32] holds the block total
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    T inc = warp_incl_scan(v);
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        T w = lane < nw ? warp_tot[lane] : T(0);
        T wi = warp_incl_scan(w);
        if (lane < nw) warp_tot[lane] = wi - w;
        if (lane == nw - 1) warp_tot[32] = wi;
    }
    __syncthreads();
    T res = inc - v + warp_tot[wid];
    *total = warp_tot[32];
    __syncthreads();
    return res;
}

}  // namespace colo
