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
// Level k >= 3: quads are enumerated from the cells of a driver member (the
// one with the fewest cells); each quad is visited once (by its first driver
// cell) and each cell is counted by its first full quad in (by, bx) order.
#include <algorithm>

#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

constexpr int kFilterThreads = 256;
constexpr int kFilterWarps = kFilterThreads / 32;
constexpr int kMaxW = 8;   // mask words handled in registers (256 features per job)

// One thread per run (C, f); a block owns a contiguous range of runs, so the
// job changes rarely and the F x F accumulator lives in shared memory.
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
    if (threadIdx.x == 0) cur_job = r0 < Rn ? (int32_t)cjob[rcell[r0]] : -1;
    __syncthreads();
    for (uint64_t base = r0; base < r1; base += blockDim.x) {
        int32_t jb = (int32_t)cjob[rcell[base]];
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
            const uint32_t job = cjob[c];
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

// Level k >= 3.  Items are (driver cell, candidate) pairs taken in run
// order: a warp owns 32 consecutive (cell, feature) runs -- cell-major, so
// all warps in flight work on a narrow band of cells whose data stays in L2
// -- and expands each run whose feature drives G candidates into G items
// (warp prefix sum; candidates of one driver are adjacent lanes).
//
// Phase 1 (a lane per item): the quads containing the driver cell C (masks
// qmask[C]) that are full for the candidate and are visited from C -- a
// quad is visited only from its first cell in (ey, ex) order holding the
// driver feature, so each full quad is seen once per candidate.  Each cell
// of a visited quad is a task: a 16-bit mask, bit 4*q + e.
// Phase 2 (the warp): the tasks of the 32 items are spread over the lanes.
// A task's cell Z is counted unless an earlier quad containing Z (in
// (by, bx) order: qmask[Z][p] for p below this quad's index in Z's frame)
// is full; a counted cell adds its runs of the members (located by rank in
// Z's feature mask) to the item's shared-memory accumulator.
// Phase 3: one atomicAdd per member per item.
// stats[c*2] = full quads, stats[c*2+1] = cells in U_c.
template <int WT>
__global__ void __launch_bounds__(256) k_filter_level(
    uint64_t Rn, const uint32_t* __restrict__ rfeat, const uint32_t* __restrict__ rcell,
    const uint32_t* __restrict__ drv_count, const uint32_t* __restrict__ drv_start,
    const uint32_t* __restrict__ flocal, const uint32_t* __restrict__ order, uint32_t k,
    const uint32_t* __restrict__ cand, const uint32_t* __restrict__ need_all, const int32_t* __restrict__ nb9,
    const uint32_t* __restrict__ cmask, const uint32_t* __restrict__ qmask, const uint32_t* __restrict__ crun,
    const uint32_t* __restrict__ rcnt, uint32_t* __restrict__ ub, unsigned long long* __restrict__ stats) {
    constexpr uint32_t W = WT;
    constexpr int kM = kMaxMembersFiltered;
    __shared__ uint32_t s_need[kFilterWarps][32][WT];
    __shared__ uint32_t s_lf[kFilterWarps][32][kM];
    __shared__ uint32_t s_acc[kFilterWarps][32][kM];
    __shared__ uint32_t s_cells[kFilterWarps][32];
    const uint32_t m = k < kMaxMembersFiltered ? k : kMaxMembersFiltered;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint64_t nwarps = (uint64_t)gridDim.x * kFilterWarps;
    for (uint64_t rbase = ((uint64_t)blockIdx.x * kFilterWarps + wid) * 32; rbase < Rn; rbase += nwarps * 32) {
        // this warp's 32 runs and the candidates their features drive
        const uint64_t myr = rbase + lane;
        uint32_t G = 0, f = 0;
        if (myr < Rn) {
            f = rfeat[myr];
            G = drv_count[f];
        }
        uint32_t rin = G;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, rin, o);
            if (lane >= o) rin += t;
        }
        const uint32_t rex = rin - G;
        const uint32_t ritems = __shfl_sync(0xffffffffu, rin, 31);
        for (uint32_t i0 = 0; i0 < ritems; i0 += 32) {
            const uint32_t it = i0 + lane;
            int j = 0;   // run lane owning item it
#pragma unroll
            for (int bstep = 16; bstep > 0; bstep >>= 1) {
                uint32_t ev = __shfl_sync(0xffffffffu, rex, j + bstep);
                if (ev <= it) j += bstep;
            }
            const uint32_t rex_j = __shfl_sync(0xffffffffu, rex, j);
            const uint32_t fd = __shfl_sync(0xffffffffu, f, j);
            const bool valid = it < ritems;
            uint32_t C = 0, c = 0, tmask = 0, nquads = 0;
            if (valid) {
                C = rcell[rbase + j];
                c = order[drv_start[fd] + (it - rex_j)];
                const uint32_t lfd = flocal[fd], f0 = fd - lfd;
                uint32_t need[WT];
#pragma unroll
                for (int w = 0; w < WT; ++w) {
                    need[w] = need_all[(uint64_t)c * W + w];
                    s_need[wid][lane][w] = need[w];
                }
                const uint32_t* q4 = qmask + (uint64_t)C * 4 * W;
                // the neighbour table is loaded with the quad masks (independent loads in flight together)
                const int32_t* nbc = nb9 + (uint64_t)C * 9;
                int32_t nbv[9];
#pragma unroll
                for (int t = 0; t < 9; ++t) nbv[t] = nbc[t];
                uint32_t full = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (covers<WT>(q4 + q * W, need)) full |= 1u << q;
                if (full) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (!(full >> q & 1u)) continue;
                        const int qx = (q & 1) - 1, qy = (q >> 1) - 1;
                        bool first = true;
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ox = qx + (e & 1), oy = qy + (e >> 1);
                            if (ox == 0 && oy == 0) break;
                            const int32_t v = nbv[(oy + 1) * 3 + (ox + 1)];
                            if (first && v >= 0 && (cmask[(uint64_t)v * W + (lfd >> 5)] >> (lfd & 31) & 1u))
                                first = false;
                        }
                        if (!first) continue;
                        ++nquads;
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (nbv[(qy + (e >> 1) + 1) * 3 + (qx + (e & 1) + 1)] >= 0) tmask |= 1u << (q * 4 + e);
                    }
                }
                const uint32_t* mem = cand + (uint64_t)c * k;
#pragma unroll
                for (int jj = 0; jj < kM; ++jj) {
                    s_lf[wid][lane][jj] = (uint32_t)jj < m ? mem[jj] - f0 : 0u;
                    s_acc[wid][lane][jj] = 0;
                }
            }
            s_cells[wid][lane] = 0;
            // warp-wide task list
            const uint32_t cnt = __popc(tmask);
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const uint32_t excl = incl - cnt;
            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
            for (uint32_t t0 = 0; t0 < total; t0 += 32) {
                const uint32_t t = t0 + lane;
                int o = 0;   // owner lane: last lane whose range starts at or before t
#pragma unroll
                for (int bstep = 16; bstep > 0; bstep >>= 1) {
                    uint32_t ev = __shfl_sync(0xffffffffu, excl, o + bstep);
                    if (ev <= t) o += bstep;
                }
                const uint32_t ex_o = __shfl_sync(0xffffffffu, excl, o);
                const uint32_t tm_o = __shfl_sync(0xffffffffu, tmask, o);
                const uint32_t C_o = __shfl_sync(0xffffffffu, C, o);
                if (t >= total) continue;
                // the (t - ex_o)-th set bit of the owner's task mask
                uint32_t bits = tm_o;
                for (uint32_t i = t - ex_o; i > 0; --i) bits &= bits - 1;
                const int tb = __ffs(bits) - 1, q = tb >> 2, e = tb & 3;
                const int qx = (q & 1) - 1, qy = (q >> 1) - 1, ex = e & 1, ey = e >> 1;
                const int32_t Z = nb9[(uint64_t)C_o * 9 + (qy + ey + 1) * 3 + (qx + ex + 1)];
                uint32_t need[WT];
#pragma unroll
                for (int w = 0; w < WT; ++w) need[w] = s_need[wid][o][w];
                // this quad is quad pq of Z; earlier quads of Z are p < pq
                const int pq = (1 - ey) * 2 + (1 - ex);
                const uint32_t* z4 = qmask + (uint64_t)Z * 4 * W;
                // Z's feature mask and first run are loaded with its quad masks
                uint32_t zm[WT];
#pragma unroll
                for (int w = 0; w < WT; ++w) zm[w] = cmask[(uint64_t)Z * W + w];
                const uint32_t q0 = crun[Z];
                bool claimed = true;
#pragma unroll
                for (int p = 0; p < 3; ++p)
                    if (p < pq && covers<WT>(z4 + p * W, need)) claimed = false;
                if (!claimed) continue;
                atomicAdd(&s_cells[wid][o], 1u);
#pragma unroll
                for (int jj = 0; jj < kM; ++jj) {
                    if ((uint32_t)jj < m) {
                        const uint32_t lf = s_lf[wid][o][jj], wq = lf >> 5;
                        uint32_t rk = 0, word = 0;
#pragma unroll
                        for (int w = 0; w < WT; ++w) {
                            if ((uint32_t)w < wq) rk += __popc(zm[w]);
                            if ((uint32_t)w == wq) word = zm[w];
                        }
                        if (word >> (lf & 31) & 1u)
                            atomicAdd(&s_acc[wid][o][jj], rcnt[q0 + rk + __popc(word & ((1u << (lf & 31)) - 1u))]);
                    }
                }
            }
            __syncwarp();
            if (valid && tmask) {
#pragma unroll
                for (int jj = 0; jj < kM; ++jj)
                    if ((uint32_t)jj < m && s_acc[wid][lane][jj])
                        atomicAdd(&ub[(uint64_t)c * k + jj], s_acc[wid][lane][jj]);
                if (stats) {
                    atomicAdd(&stats[(uint64_t)c * 2], (unsigned long long)nquads);
                    atomicAdd(&stats[(uint64_t)c * 2 + 1], (unsigned long long)s_cells[wid][lane]);
                }
            }
            __syncwarp();
        }
    }
}

}  // namespace

void filter_pairs(Batch& b, DevBuf<uint32_t>& ub2, std::vector<uint64_t>& job_off, cudaStream_t s) {
    job_off.assign(b.J + 1, 0);
    for (uint32_t j = 0; j < b.J; ++j)
        job_off[j + 1] = job_off[j] + (uint64_t)b.jobs[j].grid.nf * b.jobs[j].grid.nf;
    ub2.alloc(job_off[b.J] ? job_off[b.J] : 1, s);
    ub2.zero(s);
    if (b.M == 0) return;
    if (b.W > kMaxW) throw StatusError{COLO_ERR_CAPACITY, "the filter handles at most 256 features per job"};
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
        b.Rn, b.rcell.get(), b.cjob.get(), b.grids.get(), b.nbmask.get(), b.W, b.rfeat.get(),
        b.rcnt.get(), d_job_off.get(), ub2.get(), acc_dim, per);
    COLO_LAUNCH_CHECK();
    count_launch();
}

void filter_level(Batch& b, const uint32_t* h_cand, const uint32_t* h_job, uint64_t ncand, uint32_t k,
                  uint32_t* d_ub, unsigned long long* d_stats, const uint32_t* d_cand_in) {
    if (ncand == 0) return;
    if (b.W > kMaxW) throw StatusError{COLO_ERR_CAPACITY, "the filter handles at most 256 features per job"};
    cudaStream_t s = b.s;
    const uint32_t m = k < kMaxMembersFiltered ? k : (uint32_t)kMaxMembersFiltered;
    // driver = member with the fewest cells; candidates grouped by driver
    std::vector<uint32_t> drv(ncand), need((size_t)ncand * b.W, 0);
    for (uint64_t c = 0; c < ncand; ++c) {
        const uint32_t* mem = h_cand + c * k;
        const uint32_t f0 = b.jobs[h_job[c]].grid.f0;
        uint32_t best = mem[0], bn = UINT32_MAX;
        for (uint32_t j = 0; j < m; ++j) {
            uint32_t nr = b.h_frun_off[mem[j] + 1] - b.h_frun_off[mem[j]];
            if (nr < bn) {
                bn = nr;
                best = mem[j];
            }
            uint32_t lf = mem[j] - f0;
            need[(size_t)c * b.W + (lf >> 5)] |= 1u << (lf & 31);
        }
        drv[c] = best;
    }
    // candidates grouped by driver feature: drv_count[f] of them from drv_start[f] in `order`
    std::vector<uint32_t> order(ncand);
    for (uint64_t c = 0; c < ncand; ++c) order[c] = (uint32_t)c;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) { return drv[a] < drv[c]; });
    std::vector<uint32_t> dcount(b.F, 0), dstart(b.F, 0), flocal(b.F, 0);
    for (uint64_t i = 0; i < ncand; ++i) {
        const uint32_t fd = drv[order[i]];
        if (dcount[fd]++ == 0) dstart[fd] = (uint32_t)i;
    }
    uint64_t nitems = 0;
    for (uint32_t f = 0; f < b.F; ++f) {
        flocal[f] = f - b.jobs[b.h_fjob[f]].grid.f0;
        nitems += (uint64_t)dcount[f] * (b.h_frun_off[f + 1] - b.h_frun_off[f]);
    }
    b.filter_items += nitems;
    if (nitems == 0) return;
    DevBuf<uint32_t> dcand, dneed, dcnt, dst, dfl, dord;
    if (!d_cand_in) dcand.alloc(ncand * k, s);
    const uint32_t* d_cand = d_cand_in ? d_cand_in : dcand.get();
    dneed.alloc(need.size(), s);
    dcnt.alloc(b.F, s);
    dst.alloc(b.F, s);
    dfl.alloc(b.F, s);
    dord.alloc(ncand, s);
    if (!d_cand_in) COLO_CUDA(cudaMemcpyAsync(dcand.get(), h_cand, ncand * k * 4, cudaMemcpyHostToDevice, s));
    COLO_CUDA(cudaMemcpyAsync(dneed.get(), need.data(), need.size() * 4, cudaMemcpyHostToDevice, s));
    COLO_CUDA(cudaMemcpyAsync(dcnt.get(), dcount.data(), b.F * 4, cudaMemcpyHostToDevice, s));
    COLO_CUDA(cudaMemcpyAsync(dst.get(), dstart.data(), b.F * 4, cudaMemcpyHostToDevice, s));
    COLO_CUDA(cudaMemcpyAsync(dfl.get(), flocal.data(), b.F * 4, cudaMemcpyHostToDevice, s));
    COLO_CUDA(cudaMemcpyAsync(dord.get(), order.data(), ncand * 4, cudaMemcpyHostToDevice, s));
    uint64_t blocks = (b.Rn + 255) / 256;
    uint64_t cap = (uint64_t)b.sms * 16;
    if (blocks > cap) blocks = cap;
    KScope ks("filter_level");
#define COLO_FL(WW)                                                                                          \
    k_filter_level<WW><<<(unsigned)blocks, 256, 0, s>>>(                                                     \
        b.Rn, b.rfeat.get(), b.rcell.get(), dcnt.get(), dst.get(), dfl.get(), dord.get(), k, d_cand,          \
        dneed.get(), b.nb9.get(), b.cmask.get(), b.qmask.get(), b.crun.get(), b.rcnt.get(), d_ub, d_stats)
    switch (b.W) {
        case 1: COLO_FL(1); break;
        case 2: COLO_FL(2); break;
        case 3: COLO_FL(3); break;
        case 4: COLO_FL(4); break;
        case 5: COLO_FL(5); break;
        case 6: COLO_FL(6); break;
        case 7: COLO_FL(7); break;
        default: COLO_FL(8); break;
    }
#undef COLO_FL
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace colo
