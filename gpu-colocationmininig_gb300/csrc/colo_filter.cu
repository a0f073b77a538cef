// colo_filter.cu -- cell-aggregate upper-bound filter.
//
// Semantics (filter2_Kernel + threshold_Kernel, Codes/DeviceProcess_Kernel.h:
// 469-509 and 545-573): a quad is a 2x2 block of reference cells with lower
// corner (bx, by), 0 <= bx <= gx-2, 0 <= by <= gy-2.  It is full for
// candidate c when every member j < min(k, 8) has a point in one of its four
// cells.  U_c is the union of the cells of full quads; the bound of member j
// is the sum over U_c of that member's cell counts (members j >= 8 keep 0).
// The reference's degree-2 kernel (filter2_2_Kernel, 512-543) reads an
// uninitialised index, so pairs use the same rule.
//
// Pairs: if cell C holds feature f, C lies in U_{f,g} exactly when g occurs
// in the union of the valid quads around C, which is C's clipped 3x3 block.
// So every pair bound is one pass over the runs: for each run (C, f) and
// each feature g of the 3x3 block, add count(C, f) to bound(f side of {f,g}).
// The accumulator is an F x F matrix in shared memory.
//
// Level k >= 3: a cell is in U_c when one of its four quads is full; the
// cells tested for c are those with c's driver member (the one with the
// fewest cells) in their 3x3 block, which holds every cell of U_c.  Those
// cells are listed once per mine, per feature (driver lists), so a level
// touches only the lists of its drivers.
#include <algorithm>
#include <cstring>

#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

constexpr int kFilterThreads = 256;
constexpr int kMaxW = 32;  // mask words per cell (1024 features per job); rows of 9+ words are padded
                           // to 12, 16, 24 or 32 words when the batch is set up
constexpr uint64_t kAccMax = 16384;   // block-private level sums (64 KB of shared memory)

// One thread per run (C, f); a block owns a contiguous range of runs, so the
// job changes rarely and the F x F accumulator lives in shared memory.  cjob is
// null for a one-job batch (job 0 everywhere): the mask load then waits on one
// dependent load (the run's cell) instead of three.
__global__ void __launch_bounds__(kFilterThreads) k_filter_pairs(
    uint64_t Rn, const uint32_t* __restrict__ rcell, const uint32_t* __restrict__ cjob,
    const JobGrid* __restrict__ grids, const uint32_t* __restrict__ nbmask,
    uint32_t W, const uint32_t* __restrict__ rfeat, const uint32_t* __restrict__ rcnt,
    const uint64_t* __restrict__ job_off, uint32_t* __restrict__ ub2, uint32_t acc_dim, uint64_t runs_per_block) {
    extern __shared__ uint32_t acc[];   // acc_dim x acc_dim (acc_dim = 0: no privatisation)
    __shared__ int32_t cur_job;
    const uint64_t r0 = (uint64_t)blockIdx.x * runs_per_block;
    const uint64_t r1 = r0 + runs_per_block < Rn ? r0 + runs_per_block : Rn;
    const uint32_t accn = acc_dim * acc_dim;
    for (uint32_t i = threadIdx.x; i < accn; i += blockDim.x) acc[i] = 0;
    if (threadIdx.x == 0) cur_job = r0 < Rn ? (cjob ? (int32_t)cjob[rcell[r0]] : 0) : -1;
    __syncthreads();
    for (uint64_t base = r0; base < r1; base += blockDim.x) {
        const int32_t jb = cjob ? (int32_t)cjob[rcell[base]] : 0;
        if (jb != cur_job) {   // flush the accumulator on a job change (uniform branch)
            __syncthreads();
            uint32_t nf = grids[cur_job].nf;
            for (uint32_t i = threadIdx.x; acc_dim && i < nf * nf; i += blockDim.x) {
                uint32_t v = acc[(i / nf) * acc_dim + (i % nf)];
                if (v) atomicAdd(&ub2[job_off[cur_job] + i], v);
            }
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < accn; i += blockDim.x) acc[i] = 0;
            if (threadIdx.x == 0) cur_job = jb;
            __syncthreads();
        }
        const uint64_t r = base + threadIdx.x;
        if (r < r1) {
            const uint32_t c = rcell[r];
            const uint32_t job = cjob ? cjob[c] : 0u;
            const JobGrid g = grids[job];
            if (g.gx >= 2 && g.gy >= 2) {
                const bool priv = acc_dim && (int32_t)job == cur_job && g.nf <= acc_dim;
                const uint32_t lf = rfeat[r] - g.f0, cnt = rcnt[r];
                for (uint32_t w = 0; w < W; ++w) {
                    uint32_t bits = nbmask[(uint64_t)c * W + w];
                    while (bits) {
                        int bpos = __ffs(bits) - 1;
                        bits &= bits - 1;
                        uint32_t lg = w * 32 + bpos;
                        if (lg == lf) continue;
                        if (priv) atomicAdd(&acc[lf * acc_dim + lg], cnt);
                        else atomicAdd(&ub2[job_off[job] + (uint64_t)lf * g.nf + lg], cnt);
                    }
                }
            }
        }
    }
    __syncthreads();
    if (cur_job >= 0 && acc_dim) {
        uint32_t nf = grids[cur_job].nf;
        for (uint32_t i = threadIdx.x; i < nf * nf; i += blockDim.x) {
            uint32_t v = acc[(i / nf) * acc_dim + (i % nf)];
            if (v) atomicAdd(&ub2[job_off[cur_job] + i], v);
        }
    }
}

template <int WT>
__device__ __forceinline__ bool covers(const uint32_t* __restrict__ qm, const uint32_t (&need)[WT]) {
    bool ok = true;
#pragma unroll
    for (int w = 0; w < WT; ++w) ok &= (qm[w] & need[w]) == need[w];
    return ok;
}

template <int WT>
__device__ __forceinline__ bool covers(const uint32_t (&qm)[WT], const uint32_t (&need)[WT]) {
    bool ok = true;
#pragma unroll
    for (int w = 0; w < WT; ++w) ok &= (qm[w] & need[w]) == need[w];
    return ok;
}

// One mask row of WT words; rows start on a multiple of WT words from a
// 256-byte-aligned base, so 4-word rows load as one 16-byte vector.
template <int WT>
__device__ __forceinline__ void load_row(const uint32_t* __restrict__ p, uint32_t (&out)[WT]) {
    if constexpr (WT % 4 == 0) {
#pragma unroll
        for (int i = 0; i < WT / 4; ++i) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(p) + i);
            out[4 * i] = v.x;
            out[4 * i + 1] = v.y;
            out[4 * i + 2] = v.z;
            out[4 * i + 3] = v.w;
        }
    } else if constexpr (WT % 2 == 0) {
#pragma unroll
        for (int i = 0; i < WT / 2; ++i) {
            const uint2 v = __ldg(reinterpret_cast<const uint2*>(p) + i);
            out[2 * i] = v.x;
            out[2 * i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < WT; ++i) out[i] = __ldg(p + i);
    }
}

// ---- driver lists -----------------------------------------------------------
// The list of feature f holds the cells whose 3x3 block holds f (bit f of
// nbmask); the lists of the wanted features (the level drivers) are filled
// here, their sizes come from the quad masks' kernel.  A block owns a range of
// consecutive cells and walks it twice, 256 cells (one per thread) at a time.
// A warp's 32 cells are a bit matrix (cell x feature) per mask word;
// transposed, lane b holds feature b's column.  Pass 0 adds the columns'
// popcounts to a block histogram; one global atomic per (block, feature) then
// reserves the block's range of each list; pass 1 adds them again, the
// atomic's old value placing the warp's cells in that range, and lane b
// writes its column's cells.  Order within a list is not fixed (the level
// filter sums over it).  Batches with more than kDilHist features skip the
// histogram: one global atomic per (warp, feature).
constexpr uint32_t kDilHist = 2048;
constexpr int kDilThreads = 256;

// Bits of cell z's mask word w that are wanted: the want bitset (global
// features) taken from bit f0 + 32 w on.  The bitset holds one spare word.
__device__ __forceinline__ uint32_t dil_wanted(const uint32_t* __restrict__ want, uint32_t f0, int w, uint32_t row) {
    const uint32_t p = f0 + (uint32_t)w * 32;
    const uint32_t lo = __ldg(want + (p >> 5)), hi = __ldg(want + (p >> 5) + 1);
    return row & __funnelshift_r(lo, hi, p & 31);
}

template <int WT>
__global__ void __launch_bounds__(kDilThreads) k_dil_fill(uint64_t M, uint64_t per, const uint32_t* __restrict__ cjob,
                                                          const JobGrid* __restrict__ grids,
                                                          const uint32_t* __restrict__ nbmask, uint32_t F,
                                                          const uint64_t* __restrict__ doff,
                                                          uint32_t* __restrict__ cursor, uint32_t* __restrict__ dlist,
                                                          const uint32_t* __restrict__ want) {
    // F bases, then F counters and F touched features (F <= kDilHist; sized by the launch)
    extern __shared__ unsigned long long s_base[];
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_base + (F <= kDilHist ? F : 0));
    uint32_t* s_touch = s_cnt + (F <= kDilHist ? F : 0);
    __shared__ uint32_t s_nt;
    const bool local = F <= kDilHist;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t z0 = (uint64_t)blockIdx.x * per, z1 = z0 + per < M ? z0 + per : M;
    if (local)
        for (uint32_t i = threadIdx.x; i < F; i += blockDim.x) s_cnt[i] = 0;
    if (threadIdx.x == 0) s_nt = 0;
    __syncthreads();
    for (int pass = local ? 0 : 1; pass < 2; ++pass) {
        for (uint64_t t0 = z0; t0 < z1; t0 += kDilThreads) {
            // cell positions in 32 bits (M < 2^32) inside: the loops below are issue-bound
            const bool in = t0 + threadIdx.x < z1;
            const uint32_t z = (uint32_t)(t0 + threadIdx.x);
            const uint32_t zw = (uint32_t)(t0 + (threadIdx.x & ~31u));   // the warp's first cell
            uint32_t row[WT];
            uint32_t f0 = 0;
            if (in) {
                f0 = grids[cjob ? cjob[z] : 0u].f0;
                load_row<WT>(nbmask + (uint64_t)z * WT, row);
#pragma unroll
                for (int w = 0; w < WT; ++w)   // a nonzero word lies below F, so its bitset words exist
                    if (row[w]) row[w] = dil_wanted(want, f0, w, row[w]);
            } else {
#pragma unroll
                for (int w = 0; w < WT; ++w) row[w] = 0;
            }
            const uint32_t fl = __shfl_sync(0xffffffffu, f0, 0);
            if (!__all_sync(0xffffffffu, !in || f0 == fl)) {
                // the warp straddles a job boundary (batches of several jobs): in pass 1 every
                // lane writes its own entries, one global atomic each
#pragma unroll
                for (int w = 0; w < WT; ++w) {
                    if (pass == 1)
                        for (uint32_t bits = row[w]; bits; bits &= bits - 1) {
                            const uint32_t f = f0 + (uint32_t)w * 32 + (uint32_t)(__ffs(bits) - 1);
                            dlist[doff[f] + atomicAdd(&cursor[f], 1u)] = z;
                        }
                    row[w] = 0;
                }
            }
#pragma unroll
            for (int w = 0; w < WT; ++w) {
                if (!__any_sync(0xffffffffu, row[w])) continue;
                const uint32_t col = warp_transpose32(row[w]);
                const uint32_t n = __popc(col);
                if (!n) continue;
                const uint32_t f = fl + (uint32_t)w * 32 + lane;
                uint64_t o;
                if (local) {
                    const uint32_t old = atomicAdd(&s_cnt[f], n);
                    if (pass == 0) {
                        if (old == 0) s_touch[atomicAdd(&s_nt, 1u)] = f;
                        continue;
                    }
                    o = s_base[f] + old;
                } else {
                    o = doff[f] + atomicAdd(&cursor[f], n);
                }
                uint32_t* dst = dlist + o;
                for (uint32_t bits = col; bits; bits &= bits - 1) *dst++ = zw + (uint32_t)(__ffs(bits) - 1);
            }
        }
        if (pass == 0) {   // reserve the block's ranges; pass 1 counts again from zero
            __syncthreads();
            const uint32_t nt = s_nt;
            for (uint32_t i = threadIdx.x; i < nt; i += blockDim.x) {
                const uint32_t f = s_touch[i];
                s_base[f] = doff[f] + atomicAdd(&cursor[f], s_cnt[f]);
                s_cnt[f] = 0;
            }
            __syncthreads();
        }
    }
}

// Level k >= 3 over the driver lists.  Candidates are grouped by driver
// (group g: driver feature gfeat[g], candidates order[gstart[g] ..
// gstart[g] + gcount[g])); a unit is 32 cells of the driver's list times up
// to cu (8, 16 or 32, autotuned) of its candidates, units of one cell chunk
// adjacent (they read the same quad masks).  A warp takes a unit: lane = cell, loop over the
// candidates; a (cell Z, candidate c) pair is tested exactly as in a scan
// of every cell with the driver in its 3x3 block: Z is in U_c when one of
// its four quads covers c's members, each cell of U_c is met once, and a
// full quad is counted at its first occupied cell (qfirst).  Sums go to a
// block-private accumulator when the level's counters fit (acc_n).
template <int WT>
__global__ void __launch_bounds__(256, (WT <= 4 ? 5 : (WT <= 6 ? 4 : (WT <= 8 ? 2 : 1)))) k_filter_drv(
    uint64_t nunits, uint32_t ngroups, const uint64_t* __restrict__ uoff, const uint32_t* __restrict__ gfeat,
    const uint32_t* __restrict__ gstart, const uint32_t* __restrict__ gcount, const uint64_t* __restrict__ doff,
    const uint32_t* __restrict__ dlist, const uint32_t* __restrict__ order, const uint32_t* __restrict__ need_all,
    const uint32_t* __restrict__ lmem, uint32_t k, const uint32_t* __restrict__ qmask,
    const uint32_t* __restrict__ cmask, const uint32_t* __restrict__ crun, const uint8_t* __restrict__ qfirst,
    const uint32_t* __restrict__ rcnt, uint32_t* __restrict__ ub, unsigned long long* __restrict__ stats,
    uint32_t acc_n, uint32_t cu) {
    constexpr uint32_t W = WT;
    constexpr bool kCacheQuads = WT <= 8;
    extern __shared__ uint32_t acc[];
    const uint32_t m = k < kMaxMembersFiltered ? k : kMaxMembersFiltered;
    const uint32_t stride = m + 2;
    const int lane = threadIdx.x & 31;
    for (uint32_t i = threadIdx.x; i < acc_n; i += blockDim.x) acc[i] = 0;
    __syncthreads();
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t u = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < nunits; u += nwarps) {
        uint32_t lo = 0, hi = ngroups;   // the group of unit u: last g with uoff[g] <= u
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(uoff + mid) <= u) lo = mid;
            else hi = mid;
        }
        const uint32_t f = __ldg(gfeat + lo), G = __ldg(gcount + lo), gs = __ldg(gstart + lo);
        const uint32_t gch = (G + cu - 1) / cu;
        const uint64_t local = u - __ldg(uoff + lo);
        const uint64_t cc = local / gch;
        const uint32_t gc = (uint32_t)(local - cc * gch);
        const uint64_t l0 = __ldg(doff + f), L = __ldg(doff + f + 1) - l0;
        const uint64_t zi = cc * 32 + (uint64_t)lane;
        const bool valid = zi < L;
        const uint64_t Z = valid ? __ldg(dlist + l0 + zi) : 0u;
        const uint32_t* q4 = qmask + Z * 4 * W;
        uint32_t qr[kCacheQuads ? 4 : 1][kCacheQuads ? WT : 1];
        // the cell's own mask and first run, issued with its quads (most list cells are
        // in U_c of some candidate, and these loads would otherwise wait for the first)
        uint32_t cm[WT];
        uint32_t q0 = 0;
#pragma unroll
        for (int w = 0; w < WT; ++w) cm[w] = 0;
        if (valid) {
            if constexpr (kCacheQuads) {
#pragma unroll
                for (int q = 0; q < 4; ++q) load_row<WT>(q4 + q * W, qr[q]);
            }
            load_row<WT>(cmask + Z * W, cm);
            q0 = crun[Z];
        }
        const uint32_t t1 = gc * cu + cu < G ? gc * cu + cu : G;
        for (uint32_t t = gc * cu; t < t1; ++t) {
            const uint32_t c = __ldg(order + gs + t);
            uint32_t need[WT];
            load_row<WT>(need_all + (uint64_t)c * W, need);
            if (!valid) continue;
            uint32_t full = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                bool ok;
                if constexpr (kCacheQuads) {
                    ok = covers<WT>(qr[q], need);
                } else {
                    uint32_t qm[WT];
                    load_row<WT>(q4 + q * W, qm);
                    ok = covers<WT>(qm, need);
                }
                if (ok) full |= 1u << q;
            }
            if (!full) continue;
            uint32_t lm[4];
            load_row<4>(lmem + (uint64_t)c * 4, lm);
#pragma unroll
            for (int jj = 0; jj < kMaxMembersFiltered; ++jj) {
                if ((uint32_t)jj >= m) break;
                const uint32_t lf = (lm[jj >> 1] >> ((jj & 1) * 16)) & 0xFFFFu, wq = lf >> 5;
                uint32_t rk = 0, word = 0;
#pragma unroll
                for (int w = 0; w < WT; ++w) {
                    if ((uint32_t)w < wq) rk += __popc(cm[w]);
                    if ((uint32_t)w == wq) word = cm[w];
                }
                if (word >> (lf & 31) & 1u) {
                    const uint32_t v = rcnt[q0 + rk + __popc(word & ((1u << (lf & 31)) - 1u))];
                    if (acc_n) atomicAdd(&acc[c * stride + jj], v);
                    else atomicAdd(&ub[(uint64_t)c * k + jj], v);
                }
            }
            const uint32_t nq = __popc(full & qfirst[Z]);
            if (acc_n) {
                if (nq) atomicAdd(&acc[c * stride + m], nq);
                atomicAdd(&acc[c * stride + m + 1], 1u);
            } else if (stats) {
                if (nq) atomicAdd(&stats[(uint64_t)c * 2], (unsigned long long)nq);
                atomicAdd(&stats[(uint64_t)c * 2 + 1], 1ull);
            }
        }
    }
    if (acc_n) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < acc_n; i += blockDim.x) {
            const uint32_t v = acc[i];
            if (!v) continue;
            const uint32_t c = i / stride, r = i - c * stride;
            if (r < m) atomicAdd(&ub[(uint64_t)c * k + r], v);
            else if (stats) atomicAdd(&stats[(uint64_t)c * 2 + (r - m)], (unsigned long long)v);
        }
    }
}

}  // namespace

#define COLO_W_SWITCH(W, MACRO)                                                                   \
    switch (W) {                                                                                  \
        case 1: MACRO(1); break;                                                                  \
        case 2: MACRO(2); break;                                                                  \
        case 3: MACRO(3); break;                                                                  \
        case 4: MACRO(4); break;                                                                  \
        case 5: MACRO(5); break;                                                                  \
        case 6: MACRO(6); break;                                                                  \
        case 7: MACRO(7); break;                                                                  \
        case 8: MACRO(8); break;                                                                  \
        case 12: MACRO(12); break;                                                                \
        case 16: MACRO(16); break;                                                                \
        case 24: MACRO(24); break;                                                                \
        case 32: MACRO(32); break;                                                                \
        default: throw StatusError{COLO_ERR_INTERNAL, "mask words not padded to a supported width"}; \
    }

namespace {

// The lists of every feature in `need` (and of those already filled): the lists are filled
// again for the union when a feature is missing.
void driver_lists_fill(Batch& b, const std::vector<uint8_t>& need) {
    bool missing = false;
    for (uint32_t f = 0; f < b.F; ++f) missing |= need[f] && !b.dlist_have[f];
    if (!missing) return;
    cudaStream_t s = b.s;
    std::vector<uint32_t> want((b.F + 31) / 32 + 1, 0);   // one spare word for the kernel's funnel shift
    b.h_doff.assign(b.F + 1, 0);
    for (uint32_t f = 0; f < b.F; ++f) {
        b.dlist_have[f] |= need[f];
        if (b.dlist_have[f]) want[f >> 5] |= 1u << (f & 31);
        b.h_doff[f + 1] = b.h_doff[f] + (b.dlist_have[f] ? b.h_dcnt[f] : 0);
    }
    const uint64_t total = b.h_doff[b.F];
    b.dlist.alloc(total ? total : 1, s);
    b.doff.alloc(b.F + 1 + (want.size() + 1) / 2, s);   // offsets, then the want bitset
    uint32_t* d_want = reinterpret_cast<uint32_t*>(b.doff.get() + b.F + 1);
    COLO_CUDA(cudaMemcpyAsync(b.doff.get(), b.h_doff.data(), (b.F + 1) * 8, cudaMemcpyHostToDevice, s));
    COLO_CUDA(cudaMemcpyAsync(d_want, want.data(), want.size() * 4, cudaMemcpyHostToDevice, s));
    if (total == 0) return;
    DevBuf<uint32_t> cursor;
    cursor.alloc(b.F, s);
    cursor.zero(s);
    // one range of consecutive cells per block (a multiple of 256 cells), one wave of resident blocks;
    // shared memory for the block histogram of the batch's features (none past kDilHist)
    const size_t dsmem = b.F <= kDilHist ? (size_t)b.F * 16 : 0;
    KScope ks("driver_lists");
#define COLO_DF(WW)                                                                                              \
    do {                                                                                                         \
        int per_sm = 1;                                                                                          \
        COLO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dil_fill<WW>, kDilThreads, dsmem));   \
        uint64_t blocks = std::min<uint64_t>((b.M + kDilThreads - 1) / kDilThreads,                              \
                                             (uint64_t)b.sms * (uint64_t)std::max(per_sm, 1));                   \
        const uint64_t per = ((b.M + blocks - 1) / blocks + kDilThreads - 1) / kDilThreads * kDilThreads;        \
        blocks = (b.M + per - 1) / per;                                                                          \
        k_dil_fill<WW><<<(unsigned)blocks, kDilThreads, dsmem, s>>>(b.M, per, b.J > 1 ? b.cjob.get() : nullptr,  \
                                                               b.grids.get(), b.nbmask.get(), b.F, b.doff.get(), \
                                                               cursor.get(), b.dlist.get(), d_want);             \
    } while (0)
    COLO_W_SWITCH(b.W, COLO_DF)
#undef COLO_DF
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace

void filter_pairs(Batch& b, DevBuf<uint32_t>& ub2, std::vector<uint64_t>& job_off, cudaStream_t s) {
    job_off.assign(b.J + 1, 0);
    for (uint32_t j = 0; j < b.J; ++j)
        job_off[j + 1] = job_off[j] + (uint64_t)b.jobs[j].grid.nf * b.jobs[j].grid.nf;
    ub2.alloc(job_off[b.J] ? job_off[b.J] : 1, s);
    ub2.zero(s);
    if (b.M == 0) return;
    if (b.W > kMaxW) throw StatusError{COLO_ERR_CAPACITY, "the filter handles at most 1024 features per job"};
    DevBuf<uint64_t> d_job_off;
    d_job_off.alloc(b.J + 1, s);
    COLO_CUDA(cudaMemcpyAsync(d_job_off.get(), job_off.data(), (b.J + 1) * 8, cudaMemcpyHostToDevice, s));
    uint32_t acc_dim = b.Fmax_local;
    size_t smem = (size_t)acc_dim * acc_dim * 4;
    if (smem > 200 * 1024) {
        acc_dim = 0;
        smem = 0;
    }
    if (smem > 48 * 1024)
        COLO_CUDA(cudaFuncSetAttribute(k_filter_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // as many resident blocks per SM as the accumulator allows (at most 8)
    uint64_t per_sm = smem ? (200 * 1024) / smem : 8;
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 8) per_sm = 8;
    uint64_t blocks = (uint64_t)b.sms * per_sm;
    uint64_t per = (b.Rn + blocks - 1) / blocks;
    per = (per + kFilterThreads - 1) / kFilterThreads * kFilterThreads;
    blocks = (b.Rn + per - 1) / per;
    KScope ks("filter_pairs");
    k_filter_pairs<<<(unsigned)blocks, kFilterThreads, smem, s>>>(
        b.Rn, b.rcell.get(), b.J > 1 ? b.cjob.get() : nullptr, b.grids.get(), b.nbmask.get(), b.W, b.rfeat.get(),
        b.rcnt.get(), d_job_off.get(), ub2.get(), acc_dim, per);
    COLO_LAUNCH_CHECK();
    count_launch();
}

void filter_level(Batch& b, const uint32_t* h_cand, const uint32_t* h_job, uint64_t ncand, uint32_t k,
                  uint32_t* d_ub, unsigned long long* d_stats, const uint32_t* d_cand_in) {
    (void)d_cand_in;
    if (ncand == 0) return;
    if (b.W > kMaxW) throw StatusError{COLO_ERR_CAPACITY, "the filter handles at most 1024 features per job"};
    cudaStream_t s = b.s;
    const uint32_t m = k < kMaxMembersFiltered ? k : (uint32_t)kMaxMembersFiltered;
    // driver = member with the shortest driver list (the fewest cells with it in
    // their 3x3 block: the cells its candidates are tested on); candidates
    // grouped by driver; per candidate its need mask and local member ids
    // (16 bits each)
    std::vector<uint32_t> drv(ncand), need((size_t)ncand * b.W, 0), lmem((size_t)ncand * 4, 0);
    for (uint64_t c = 0; c < ncand; ++c) {
        const uint32_t* mem = h_cand + c * k;
        const uint32_t f0 = b.jobs[h_job[c]].grid.f0;
        uint32_t best = mem[0];
        uint64_t bn = UINT64_MAX;
        for (uint32_t j = 0; j < m; ++j) {
            const uint64_t nr = b.h_dcnt[mem[j]];
            if (nr < bn) {
                bn = nr;
                best = mem[j];
            }
            uint32_t lf = mem[j] - f0;
            need[(size_t)c * b.W + (lf >> 5)] |= 1u << (lf & 31);
            lmem[(size_t)c * 4 + (j >> 1)] |= lf << ((j & 1) * 16);
        }
        drv[c] = best;
    }
    std::vector<uint32_t> order(ncand);
    for (uint64_t c = 0; c < ncand; ++c) order[c] = (uint32_t)c;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) { return drv[a] < drv[c]; });
    std::vector<uint32_t> dcount(b.F, 0), dstart(b.F, 0);
    for (uint64_t i = 0; i < ncand; ++i) {
        const uint32_t fd = drv[order[i]];
        if (dcount[fd]++ == 0) dstart[fd] = (uint32_t)i;
    }
    uint64_t nitems = 0;   // (driver cell, candidate) pairs: the work the driver choice bounds
    for (uint32_t f = 0; f < b.F; ++f) nitems += (uint64_t)dcount[f] * (b.h_frun_off[f + 1] - b.h_frun_off[f]);
    b.filter_items += nitems;
    if (nitems == 0) return;
    {
        std::vector<uint8_t> need(b.F, 0);   // the drivers' lists (a later level's new driver refills)
        for (uint64_t c = 0; c < ncand; ++c) need[drv[c]] = 1;
        driver_lists_fill(b, need);
    }
    // groups (one per driver) and their units: 32 list cells x up to cu candidates
    const uint32_t cu = (b.filter_unit == 8 || b.filter_unit == 16) ? (uint32_t)b.filter_unit : 32u;
    std::vector<uint32_t> gfeat, gstart, gcount;
    std::vector<uint64_t> uoff(1, 0);
    for (uint32_t f = 0; f < b.F; ++f) {
        if (!dcount[f]) continue;
        const uint64_t L = b.h_doff[f + 1] - b.h_doff[f];
        gfeat.push_back(f);
        gstart.push_back(dstart[f]);
        gcount.push_back(dcount[f]);
        uoff.push_back(uoff.back() + (L + 31) / 32 * ((dcount[f] + cu - 1) / cu));
    }
    const uint32_t ngroups = (uint32_t)gfeat.size();
    const uint64_t nunits = uoff.back();
    if (nunits == 0) return;
    // one upload: need | lmem | order | gfeat | gstart | gcount | uoff (u64), mask rows and the
    // u64 part on 16-byte boundaries
    auto up4 = [](size_t v) { return (v + 3) & ~(size_t)3; };
    const size_t n_need = up4(need.size()), n_lmem = up4(lmem.size()), n_ord = up4(order.size());
    const size_t n_g = up4(ngroups);
    std::vector<uint32_t> pack(n_need + n_lmem + n_ord + 3 * n_g + 2 * uoff.size(), 0);
    size_t o = 0;
    std::copy(need.begin(), need.end(), pack.begin() + o);
    o += n_need;
    std::copy(lmem.begin(), lmem.end(), pack.begin() + o);
    o += n_lmem;
    std::copy(order.begin(), order.end(), pack.begin() + o);
    o += n_ord;
    std::copy(gfeat.begin(), gfeat.end(), pack.begin() + o);
    std::copy(gstart.begin(), gstart.end(), pack.begin() + o + n_g);
    std::copy(gcount.begin(), gcount.end(), pack.begin() + o + 2 * n_g);
    o += 3 * n_g;
    std::memcpy(pack.data() + o, uoff.data(), uoff.size() * 8);
    DevBuf<uint32_t> dpack;
    dpack.alloc(pack.size(), s);
    COLO_CUDA(cudaMemcpyAsync(dpack.get(), pack.data(), pack.size() * 4, cudaMemcpyHostToDevice, s));
    const uint32_t* d_need = dpack.get();
    const uint32_t* d_lmem = d_need + n_need;
    const uint32_t* d_order = d_lmem + n_lmem;
    const uint32_t* d_gfeat = d_order + n_ord;
    const uint32_t* d_gstart = d_gfeat + n_g;
    const uint32_t* d_gcount = d_gstart + n_g;
    const uint64_t* d_uoff = reinterpret_cast<const uint64_t*>(d_gcount + n_g);
    // block-private sums when the level's counters fit in 64 KB of shared memory
    const uint64_t acc64 = ncand * (uint64_t)(m + 2);
    const uint32_t acc_n = acc64 <= kAccMax ? (uint32_t)acc64 : 0u;
    const size_t smem = (size_t)acc_n * 4;
    // a grid-stride loop over units (one warp each): as many blocks as fit at once
    auto grid = [&](const void* fn) {
        if (smem > 48 * 1024)
            COLO_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        COLO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem));
        const uint64_t cap = (uint64_t)b.sms * (uint64_t)(per_sm > 0 ? per_sm : 1);
        const uint64_t want = (nunits + 7) / 8;
        return (unsigned)(want < cap ? want : cap);
    };
    KScope ks("filter_level");
#define COLO_FL(WW)                                                                                             \
    k_filter_drv<WW><<<grid((const void*)k_filter_drv<WW>), 256, smem, s>>>(                                    \
        nunits, ngroups, d_uoff, d_gfeat, d_gstart, d_gcount, b.doff.get(), b.dlist.get(), d_order, d_need,       \
        d_lmem, k, b.qmask.get(), b.cmask.get(), b.crun.get(), b.qfirst.get(), b.rcnt.get(), d_ub, d_stats, acc_n, cu)
    COLO_W_SWITCH(b.W, COLO_FL)
#undef COLO_FL
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace colo
