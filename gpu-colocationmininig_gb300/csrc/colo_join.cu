// colo_join.cu -- cell-pair spatial join producing the neighbour CSR
//   N+(a) = {b : feat(b) > feat(a), cell(b) adjacent to cell(a), sq(a,b) <= R^2}
// with each list ordered by (feature, neighbour cell, b): exactly the order in
// which degree2TableSlotCounter_Kernel / generalInstanceTableSlotCounter_Kernel
// visit candidates (Codes/DeviceProcess_Kernel.h:12-55, 255-316).
//
// A group of T lanes serves one anchor.  The anchor's targets are a
// contiguous suffix of its cell's neighbourhood point list (NPL), so loads are
// coalesced 4-byte streams shared by every anchor of the cell (L1/L2 reuse).
// The count pass writes |N+(a)|; the fill pass compacts hits with one warp
// ballot per step (warp-aggregated compaction, no atomics).
#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

template <int T, bool FILL>
__global__ void __launch_bounds__(256) k_join(
    uint64_t n, const uint32_t* __restrict__ sid, const uint32_t* __restrict__ scell,
    const uint32_t* __restrict__ sfeat, const float* __restrict__ sx, const float* __restrict__ sy,
    const uint64_t* __restrict__ nrl_off, const uint32_t* __restrict__ nrl_feat,
    const uint64_t* __restrict__ nrl_pos, const uint64_t* __restrict__ npl_off,
    const uint32_t* __restrict__ npl_id, const float* __restrict__ npl_x,
    const float* __restrict__ npl_y, const uint32_t* __restrict__ fjob,
    const JobGrid* __restrict__ grids, uint32_t* __restrict__ cnt,
    const uint64_t* __restrict__ nb_off, uint32_t* __restrict__ nb) {
    const int lane = threadIdx.x & 31;
    const int gl = lane % T;
    const int gbase = lane - gl;
    const uint64_t p = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / T;
    const bool valid = p < n;
    uint64_t s = 0, e = 0;
    float xa = 0.f, ya = 0.f, R2 = 0.f;
    uint32_t a = 0;
    if (valid) {
        uint32_t c = scell[p];
        uint32_t fa = sfeat[p];
        a = sid[p];
        xa = sx[p];
        ya = sy[p];
        R2 = grids[fjob[fa]].R2;
        uint64_t q0 = nrl_off[c], q1 = nrl_off[c + 1];
        // first run whose feature is above the anchor's
        uint64_t lo = q0, hi = q1;
        while (lo < hi) {
            uint64_t mid = (lo + hi) >> 1;
            if (nrl_feat[mid] <= fa) lo = mid + 1;
            else hi = mid;
        }
        e = npl_off[c + 1];
        s = lo < q1 ? nrl_pos[lo] : e;
    }
    uint32_t iters = (uint32_t)((e - s + T - 1) / T);
    uint32_t maxit = __reduce_max_sync(0xffffffffu, iters);
    const uint32_t gmask_bits = (T == 32) ? 0xffffffffu : ((1u << T) - 1u);
    uint32_t count = 0;
    uint64_t out = 0;
    if (FILL && valid) out = nb_off[a];
    for (uint32_t it = 0; it < maxit; ++it) {
        uint64_t t = s + (uint64_t)it * T + gl;
        bool ok = false;
        uint32_t bid = 0;
        if (t < e) {
            ok = ref_sqdist(xa, ya, npl_x[t], npl_y[t]) <= R2;
            if (FILL && ok) bid = npl_id[t];
        }
        uint32_t bal = __ballot_sync(0xffffffffu, ok);
        uint32_t gm = (bal >> gbase) & gmask_bits;
        if (FILL) {
            if (ok) nb[out + __popc(gm & ((1u << gl) - 1u))] = bid;
            out += __popc(gm);
        } else {
            count += __popc(gm);
        }
    }
    if (!FILL && valid && gl == 0) cnt[a] = count;
}

template <int T>
void run_join(Batch& b, bool fill, uint32_t* cnt) {
    const uint64_t n = b.N;
    KScope ks(fill ? "join_fill" : "join_count");
    uint64_t threads = n * T;
    unsigned grid = (unsigned)((threads + 255) / 256);
    if (grid == 0) grid = 1;
    if (!fill) {
        k_join<T, false><<<grid, 256, 0, b.s>>>(n, b.sid.get(), b.scell.get(), b.sfeat.get(), b.sx.get(),
                                                b.sy.get(), b.nrl_off.get(), b.nrl_feat.get(),
                                                b.nrl_pos.get(), b.npl_off.get(), b.npl_id.get(),
                                                b.npl_x.get(), b.npl_y.get(), b.fjob.get(),
                                                b.grids.get(), cnt, nullptr, nullptr);
    } else {
        k_join<T, true><<<grid, 256, 0, b.s>>>(n, b.sid.get(), b.scell.get(), b.sfeat.get(), b.sx.get(),
                                               b.sy.get(), b.nrl_off.get(), b.nrl_feat.get(),
                                               b.nrl_pos.get(), b.npl_off.get(), b.npl_id.get(),
                                               b.npl_x.get(), b.npl_y.get(), b.fjob.get(),
                                               b.grids.get(), nullptr, b.nb_off.get(), b.nb.get());
    }
    COLO_LAUNCH_CHECK();
    count_launch();
}

void dispatch_join(Batch& b, bool fill, uint32_t* cnt) {
    switch (b.join_group) {
        case 4: run_join<4>(b, fill, cnt); break;
        case 16: run_join<16>(b, fill, cnt); break;
        case 32: run_join<32>(b, fill, cnt); break;
        default: run_join<8>(b, fill, cnt); break;
    }
}

__global__ void k_sqdist(const float* __restrict__ x1, const float* __restrict__ y1,
                         const float* __restrict__ x2, const float* __restrict__ y2, uint64_t n,
                         float* __restrict__ out) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = ref_sqdist(x1[i], y1[i], x2[i], y2[i]);
}

}  // namespace

void join_neighbors(Batch& b) {
    cudaStream_t s = b.s;
    DevBuf<uint32_t> cnt;
    cnt.alloc(b.N, s);
    dispatch_join(b, false, cnt.get());
    b.nb_off.alloc(b.N + 1, s);
    uint64_t E = 0;
    scan_u32_to_u64(cnt.get(), b.nb_off.get(), b.N, s, &E);
    COLO_CUDA(cudaMemcpyAsync(b.nb_off.get() + b.N, &E, 8, cudaMemcpyHostToDevice, s));
    b.E = E;
    b.nb.alloc(E, s);
    if (E) dispatch_join(b, true, nullptr);
}

void eval_sqdist(const float* x1, const float* y1, const float* x2, const float* y2, uint64_t n,
                 float* out, cudaStream_t s) {
    if (n == 0) return;
    k_sqdist<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x1, y1, x2, y2, n, out);
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace colo
