// colo_join.cu -- cell-pair spatial join producing the neighbour lists
//   N+(a) = {b : feat(b) > feat(a), cell(b) adjacent to cell(a), sq(a,b) <= R^2}
// each ordered by (feature, neighbour cell, b): exactly the order in which
// degree2TableSlotCounter_Kernel / generalInstanceTableSlotCounter_Kernel
// visit candidates (Codes/DeviceProcess_Kernel.h:12-55, 255-316).
//
// Work is organised by run (the points of one feature in one cell): a run's
// targets are the suffix of its cell's neighbourhood run list with higher
// features, so runs without targets cost nothing and every anchor of a run
// walks the same target list (L1/L2 reuse).  A group of T lanes serves one
// anchor; target points are read straight from the cell-sorted coordinate
// arrays, and hits are compacted with one group ballot per step.
//
// Single pass: each anchor owns a region of its run's upper bound L (the
// number of target points) and writes its hits there, so no counting pass is
// needed; when the upper bounds would not fit, a count pass + scan + fill
// pass produces a compact layout instead.
#include <cmath>
#include <vector>

#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

enum { J_SINGLE = 0, J_COUNT = 1, J_FILL = 2 };

// The single pass sums the list total into kEntrySlots counters kEntryStride
// words apart (one 128-byte line each), added up when the total is read.
constexpr int kEntrySlots = 64, kEntryStride = 16;

// One anchor's neighbour list, by its group of T lanes; returns the list length.
template <int T, int MODE>
__device__ __forceinline__ uint32_t join_anchor(
    uint64_t i, const uint32_t* __restrict__ act_pos, const uint32_t* __restrict__ act_run,
    const uint32_t* __restrict__ sid, const uint32_t* __restrict__ sfeat, const float2* __restrict__ sxy,
    const uint64_t* __restrict__ run_sfx, const uint32_t* __restrict__ run_qn, const uint64_t* __restrict__ act_base,
    const uint2* __restrict__ nrl_ent, const uint32_t* __restrict__ fjob, const JobGrid* __restrict__ grids,
    uint64_t* __restrict__ nb_beg, uint32_t* __restrict__ nb_cnt, uint32_t* __restrict__ nb) {
    const int lane = threadIdx.x & 31;
    const int gl = lane % T;
    const int gbase = lane - gl;
    const uint32_t gmask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << gbase);
    const uint32_t p = act_pos[i];
    const uint32_t r = act_run[i];
    const uint32_t a = sid[p];
    const float2 pa = sxy[p];
    const float xa = pa.x, ya = pa.y;
    const JobGrid& g = grids[fjob ? fjob[sfeat[p]] : 0u];   // fjob is null for one-job batches
    const float R2 = g.R2, hu = g.R2hu;
    const uint64_t q0 = run_sfx[r], qend = q0 + run_qn[r];
    uint64_t base = 0;
    if (MODE == J_SINGLE) base = act_base[i];
    if (MODE == J_FILL) base = nb_beg[a];
    uint32_t k = 0;
    for (uint64_t q = q0; q < qend; ++q) {
        const uint2 te = nrl_ent[q];   // the target run's first sorted position and point count
        const uint32_t ts = te.x, tc = te.y;
        if constexpr (T == 1) {
            // one lane per anchor: no group vote
            for (uint32_t t = 0; t < tc; ++t) {
                const float2 pb = sxy[ts + t];
                if (ref_within(xa, ya, pb.x, pb.y, R2, hu)) {
                    if (MODE != J_COUNT) nb[base + k] = sid[ts + t];
                    ++k;
                }
            }
        } else {
            for (uint32_t b0 = 0; b0 < tc; b0 += T) {
                const uint32_t t = b0 + gl;
                bool ok = false;
                if (t < tc) {
                    const float2 pb = sxy[ts + t];
                    ok = ref_within(xa, ya, pb.x, pb.y, R2, hu);
                }
                const uint32_t bal = (__ballot_sync(gmask, ok) >> gbase) & ((T == 32) ? 0xffffffffu : ((1u << T) - 1u));
                if (MODE != J_COUNT && ok) nb[base + k + __popc(bal & ((1u << gl) - 1u))] = sid[ts + t];
                k += __popc(bal);
            }
        }
    }
    if (gl == 0) {
        nb_cnt[a] = k;
        if (MODE == J_SINGLE) nb_beg[a] = base;
    }
    return k;
}


// Six blocks per SM (40 registers): the join is latency-bound, and the sixth block
// measured 0.398 -> 0.377 ms per step on the 20M workload.
template <int T, int MODE>
__global__ void __launch_bounds__(256, 6) k_join(
    uint64_t A, const uint32_t* __restrict__ act_pos, const uint32_t* __restrict__ act_run,
    const uint32_t* __restrict__ sid, const uint32_t* __restrict__ sfeat, const float2* __restrict__ sxy,
    const uint64_t* __restrict__ run_sfx, const uint32_t* __restrict__ run_qn, const uint64_t* __restrict__ act_base,
    const uint2* __restrict__ nrl_ent, const uint32_t* __restrict__ fjob, const JobGrid* __restrict__ grids,
    uint64_t* __restrict__ nb_beg, uint32_t* __restrict__ nb_cnt, uint32_t* __restrict__ nb,
    unsigned long long* __restrict__ total) {
    const int lane = threadIdx.x & 31;
    const int gl = lane % T;
    const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / T;
    // groups past the last anchor (whole groups) count nothing but stay for the block sum
    const uint32_t k = i < A ? join_anchor<T, MODE>(i, act_pos, act_run, sid, sfeat, sxy, run_sfx, run_qn, act_base,
                                                     nrl_ent, fjob, grids, nb_beg, nb_cnt, nb)
                             : 0u;
    if (MODE == J_SINGLE) {
        // the entries of the warp's anchors (each group's count once), one atomic per warp into
        // one of kEntrySlots counters on separate lines: the list total without another pass
        // over the counts, and no block barrier (one made every warp wait for its block's
        // longest list: the 512-job batch's join ran 10.96 ms against 9.38 ms)
        unsigned long long v = gl == 0 ? k : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        if (lane == 0 && v) atomicAdd(total + (warp % kEntrySlots) * kEntryStride, v);
    }
}

template <int T>
void run_join(Batch& b, int mode, uint64_t A, const uint32_t* act_pos, const uint32_t* act_run,
              const uint64_t* act_base) {
    if (A == 0) return;
    uint64_t threads = A * T;
    unsigned grid = (unsigned)((threads + 255) / 256);
    KScope ks(mode == J_SINGLE ? "join" : mode == J_COUNT ? "join_count" : "join_fill");
#define COLO_JOIN(MD)                                                                                        \
    k_join<T, MD><<<grid, 256, 0, b.s>>>(A, act_pos, act_run, b.sid.get(), b.sfeat.get(), b.sxy.get(),       \
                                         b.run_sfx.get(), b.run_qn.get(), act_base, b.nrl_ent.get(),            \
                                         b.J > 1 ? b.fjob.get() : nullptr,                                      \
                                         b.grids.get(), b.nb_beg.get(), b.nb_cnt.get(), b.nb.get(), b.dE.get())
    if (mode == J_SINGLE) COLO_JOIN(J_SINGLE);
    else if (mode == J_COUNT) COLO_JOIN(J_COUNT);
    else COLO_JOIN(J_FILL);
#undef COLO_JOIN
    COLO_LAUNCH_CHECK();
    count_launch();
}

void dispatch_join(Batch& b, int mode, uint64_t A, const uint32_t* act_pos, const uint32_t* act_run,
                   const uint64_t* act_base) {
    switch (b.join_group) {
        case 1: run_join<1>(b, mode, A, act_pos, act_run, act_base); break;
        case 2: run_join<2>(b, mode, A, act_pos, act_run, act_base); break;
        case 4: run_join<4>(b, mode, A, act_pos, act_run, act_base); break;
        case 16: run_join<16>(b, mode, A, act_pos, act_run, act_base); break;
        case 32: run_join<32>(b, mode, A, act_pos, act_run, act_base); break;
        default: run_join<8>(b, mode, A, act_pos, act_run, act_base); break;
    }
}

__global__ void k_sqdist(const float* __restrict__ x1, const float* __restrict__ y1,
                         const float* __restrict__ x2, const float* __restrict__ y2, uint64_t n,
                         float* __restrict__ out, float R2, float hu, uint8_t* __restrict__ within) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = ref_sqdist(x1[i], y1[i], x2[i], y2[i]);
    if (within) within[i] = ref_within(x1[i], y1[i], x2[i], y2[i], R2, hu) ? 1 : 0;
}

}  // namespace

// Upper bound of the single-pass layout above which the compact two-pass
// layout is used instead (entries).
static const uint64_t kSinglePassCap = 1ull << 30;

void join_neighbors(Batch& b) {
    cudaStream_t s = b.s;
    const uint64_t Rn = b.Rn;
    // the active anchors (the points of runs with targets, by run) are listed by the
    // scan itself, into arrays sized for every point
    DevBuf<uint32_t> act_pos, act_run;
    DevBuf<uint64_t> act_base;
    act_pos.alloc(b.N ? b.N : 1, s);
    act_run.alloc(b.N ? b.N : 1, s);
    act_base.alloc(b.N ? b.N : 1, s);
    // per run: active anchors (its points, when it has targets) and the single-pass layout's
    // capacity (points x targets), both scanned in one pass; the totals A and U (= pair
    // evaluations) come back together with one wait
    DevBuf<uint64_t> totals;
    totals.alloc(2, s);
    run_scans(b.rcnt.get(), b.run_L.get(), b.rstart.get(), act_pos.get(), act_run.get(), act_base.get(), Rn, s,
              reinterpret_cast<uint32_t*>(totals.get()), totals.get() + 1);
    uint64_t ht[2] = {0, 0};
    COLO_CUDA(cudaMemcpyAsync(ht, totals.get(), 16, cudaMemcpyDeviceToHost, s));
    stream_wait(s);
    const uint32_t A = (uint32_t)ht[0];
    const uint64_t U = ht[1];
    b.active_anchors = A;
    b.join_pairs = U;
    // a point without targets keeps a zero count; its list start is never read (every
    // reader takes nb_cnt first), so only the counts are cleared
    b.nb_beg.alloc(b.N ? b.N : 1, s);
    b.nb_cnt.alloc(b.N ? b.N : 1, s);
    b.nb_cnt.zero(s);
    b.dE.alloc(kEntrySlots * kEntryStride, s);
    b.join_single = U <= kSinglePassCap;
    if (b.join_single) {
        // total entries: summed by the join's warps and read at the mine's next wait
        b.nb_cap = U;
        b.nb.alloc(U ? U : 1, s);
        b.dE.zero(s);
        dispatch_join(b, J_SINGLE, A, act_pos.get(), act_run.get(), act_base.get());
        b.E = UINT64_MAX;
    } else {
        dispatch_join(b, J_COUNT, A, act_pos.get(), act_run.get(), nullptr);
        uint64_t E = 0;
        scan_u32_to_u64(b.nb_cnt.get(), b.nb_beg.get(), b.N, s, &E);
        b.nb_cap = E;
        b.nb.alloc(E ? E : 1, s);
        dispatch_join(b, J_FILL, A, act_pos.get(), act_run.get(), nullptr);
        b.E = E;
    }
}

uint64_t neighbor_entries(Batch& b) {
    if (b.E == UINT64_MAX) {
        std::vector<unsigned long long> e(kEntrySlots * kEntryStride);
        COLO_CUDA(cudaMemcpyAsync(e.data(), b.dE.get(), e.size() * 8, cudaMemcpyDeviceToHost, b.s));
        stream_wait(b.s);
        uint64_t t = 0;
        for (int i = 0; i < kEntrySlots; ++i) t += e[(size_t)i * kEntryStride];
        b.E = t;
    }
    return b.E;
}

void eval_sqdist(const float* x1, const float* y1, const float* x2, const float* y2, uint64_t n,
                 float* out, cudaStream_t s, float R2, uint8_t* within) {
    if (n == 0) return;
    float hu = (std::nextafter(R2, INFINITY) - R2) * 0.5f;
    k_sqdist<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x1, y1, x2, y2, n, out, R2, hu, within);
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace colo
