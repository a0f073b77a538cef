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
// fewest cells) in their 3x3 block, which holds every cell of U_c.
#include <algorithm>

#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

constexpr int kFilterThreads = 256;
constexpr int kFilterWarps = kFilterThreads / 32;
constexpr int kMaxW = 32;  // mask words per cell (1024 features per job); rows of 9+ words are padded
                           // to 12, 16, 24 or 32 words when the batch is set up
constexpr uint64_t kAccMax = 16384;   // block-private level sums (64 KB of shared memory)

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

// Position of the r-th set bit (r < popc(v)) of v.
__device__ __forceinline__ uint32_t select_bit(uint32_t v, uint32_t r) {
    uint32_t pos = 0;
#pragma unroll
    for (int half = 16; half > 0; half >>= 1) {
        const uint32_t lo = __popc(v & ((1u << half) - 1u));
        if (r >= lo) {
            r -= lo;
            v >>= half;
            pos += half;
        }
    }
    return pos;
}

// Last lane whose exclusive offset is <= t (the lane owning entry t).
__device__ __forceinline__ int owner_lane(uint32_t excl, uint32_t t) {
    int o = 0;
#pragma unroll
    for (int bstep = 16; bstep > 0; bstep >>= 1) {
        const uint32_t ev = __shfl_sync(0xffffffffu, excl, o + bstep);
        if (ev <= t) o += bstep;
    }
    return o;
}

__device__ __forceinline__ uint32_t warp_incl_sum(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Level k >= 3, one (cell Z, candidate c) pair per lane.
//
// A cell Z lies in U_c exactly when one of its four quads (qmask[Z]) is full
// for c.  A full quad holds a cell of every member, in particular of c's
// driver member d (the member with the fewest cells), so every cell of U_c
// has d in its 3x3 feature mask nbmask[Z].  The pairs tested are therefore
// (Z, c) for every occupied cell Z and every candidate whose driver is in
// nbmask[Z]; each pair is tested once, so each cell of U_c is counted once
// with no ownership rule.  A full quad is counted at its first occupied cell
// in (ey, ex) order (bit q of qfirst[Z]), so each is counted once.
//
// A warp takes 32 consecutive cells, expands them into (Z, driver) pairs and
// those into (Z, candidate) pairs (warp prefix sums; candidates of one driver
// in adjacent lanes, so lanes share Z's masks in L1).
// stats[c*2] = full quads, stats[c*2+1] = cells in U_c.  cjob is null for a
// one-job batch (every cell in job 0), which saves the scan a load per cell.
//
// Sums go to a block-private accumulator in shared memory when the level's
// candidates fit (acc_n = ncand * (m + 2) counters: m bounds, quads, cells),
// and are added to ub / stats once per block at the end: a level has few
// candidates and millions of hits, and global atomics on the same few
// addresses serialise in their L2 slice.
template <int WT>
__global__ void __launch_bounds__(256, (WT <= 8 ? 5 : 1)) k_filter_cells(
    uint64_t M, const uint32_t* __restrict__ cjob, const JobGrid* __restrict__ grids,
    const uint32_t* __restrict__ nbmask, const uint32_t* __restrict__ dmask,
    const uint32_t* __restrict__ drv_count, const uint32_t* __restrict__ drv_start,
    const uint32_t* __restrict__ order, const uint32_t* __restrict__ need_all, const uint32_t* __restrict__ lmem,
    uint32_t k, const uint32_t* __restrict__ qmask, const uint32_t* __restrict__ cmask,
    const uint32_t* __restrict__ crun, const uint8_t* __restrict__ qfirst, const uint32_t* __restrict__ rcnt,
    uint32_t* __restrict__ ub, unsigned long long* __restrict__ stats, uint32_t acc_n) {
    constexpr uint32_t W = WT;
    extern __shared__ uint32_t acc[];
    const uint32_t m = k < kMaxMembersFiltered ? k : kMaxMembersFiltered;
    const uint32_t stride = m + 2;
    const int lane = threadIdx.x & 31;
    for (uint32_t i = threadIdx.x; i < acc_n; i += blockDim.x) acc[i] = 0;
    __syncthreads();
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    // the next chunk's job and 3x3 mask are loaded before this chunk is
    // processed, so their latency overlaps this chunk's work
    const uint64_t zstride = nwarps * 32;
    uint64_t zbase = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32;
    uint32_t job_c = 0, nb_c[WT];
#pragma unroll
    for (int w = 0; w < WT; ++w) nb_c[w] = 0;
    if (zbase + lane < M) {
        job_c = cjob ? cjob[zbase + lane] : 0u;
        load_row<WT>(nbmask + (zbase + lane) * W, nb_c);
    }
    for (; zbase < M; zbase += zstride) {
        const uint64_t Zn = zbase + zstride + lane;
        uint32_t job_n = 0, nb_n[WT];
#pragma unroll
        for (int w = 0; w < WT; ++w) nb_n[w] = 0;
        if (Zn < M) {
            job_n = cjob ? cjob[Zn] : 0u;
            load_row<WT>(nbmask + Zn * W, nb_n);
        }
        // this lane's cell and the drivers of its 3x3 block
        const uint64_t Z = zbase + lane;
        uint32_t dz[WT], f0 = 0, nd = 0;
#pragma unroll
        for (int w = 0; w < WT; ++w) dz[w] = 0;
        if (Z < M) {
            f0 = grids[job_c].f0;
            uint32_t dm[WT];
            load_row<WT>(dmask + (uint64_t)job_c * W, dm);
#pragma unroll
            for (int w = 0; w < WT; ++w) {
                dz[w] = nb_c[w] & dm[w];
                nd += __popc(dz[w]);
            }
        }
        job_c = job_n;
#pragma unroll
        for (int w = 0; w < WT; ++w) nb_c[w] = nb_n[w];
        const uint32_t pincl = warp_incl_sum(nd, lane);
        const uint32_t pex = pincl - nd;
        const uint32_t npairs = __shfl_sync(0xffffffffu, pincl, 31);
        for (uint32_t p0 = 0; p0 < npairs; p0 += 32) {
            // (cell, driver) pair p0 + lane
            const uint32_t t = p0 + lane;
            const int o = owner_lane(pex, t);
            const uint32_t ex_o = __shfl_sync(0xffffffffu, pex, o);
            const uint32_t f0_o = __shfl_sync(0xffffffffu, f0, o);
            uint32_t r = t - ex_o, d = 0;
            bool found = false;
#pragma unroll
            for (int w = 0; w < WT; ++w) {
                const uint32_t v = __shfl_sync(0xffffffffu, dz[w], o);
                const uint32_t pc = __popc(v);
                if (!found && r < pc) {
                    d = (uint32_t)w * 32 + select_bit(v, r);
                    found = true;
                } else if (!found) {
                    r -= pc;
                }
            }
            uint32_t G = 0, start = 0;
            if (t < npairs) {
                G = drv_count[f0_o + d];
                start = drv_start[f0_o + d];
            }
            const uint64_t Zp = zbase + (uint64_t)o;
            const uint32_t iincl = warp_incl_sum(G, lane);
            const uint32_t iex = iincl - G;
            const uint32_t nitems = __shfl_sync(0xffffffffu, iincl, 31);
            for (uint32_t i0 = 0; i0 < nitems; i0 += 32) {
                // (cell, candidate) pair i0 + lane
                const uint32_t it = i0 + lane;
                const int o2 = owner_lane(iex, it);
                const uint32_t ex2 = __shfl_sync(0xffffffffu, iex, o2);
                const uint32_t st2 = __shfl_sync(0xffffffffu, start, o2);
                const uint64_t Zi = __shfl_sync(0xffffffffu, Zp, o2);
                if (it >= nitems) continue;
                const uint32_t c = order[st2 + (it - ex2)];
                uint32_t need[WT];
                load_row<WT>(need_all + (uint64_t)c * W, need);
                const uint32_t* q4 = qmask + Zi * 4 * W;
                uint32_t full = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint32_t qm[WT];
                    load_row<WT>(q4 + q * W, qm);
                    if (covers<WT>(qm, need)) full |= 1u << q;
                }
                if (!full) continue;
                uint32_t cm[WT];
                load_row<WT>(cmask + Zi * W, cm);
                const uint32_t q0 = crun[Zi];
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
                const uint32_t nq = __popc(full & qfirst[Zi]);
                if (acc_n) {
                    if (nq) atomicAdd(&acc[c * stride + m], nq);
                    atomicAdd(&acc[c * stride + m + 1], 1u);
                } else if (stats) {
                    if (nq) atomicAdd(&stats[(uint64_t)c * 2], (unsigned long long)nq);
                    atomicAdd(&stats[(uint64_t)c * 2 + 1], 1ull);
                }
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
        b.Rn, b.rcell.get(), b.cjob.get(), b.grids.get(), b.nbmask.get(), b.W, b.rfeat.get(),
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
    // driver = member with the fewest cells; candidates grouped by driver;
    // per candidate its need mask and local member ids (bytes), per job the
    // mask of its drivers
    std::vector<uint32_t> drv(ncand), need((size_t)ncand * b.W, 0), lmem((size_t)ncand * 4, 0),
        dmask((size_t)b.J * b.W, 0);
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
            lmem[(size_t)c * 4 + (j >> 1)] |= lf << ((j & 1) * 16);
        }
        drv[c] = best;
        const uint32_t ld = best - f0;
        dmask[(size_t)h_job[c] * b.W + (ld >> 5)] |= 1u << (ld & 31);
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
    // one upload: need | lmem | dmask | dcount | dstart | order, each part on a
    // 16-byte boundary (mask rows are read as vectors)
    auto up4 = [](size_t v) { return (v + 3) & ~(size_t)3; };
    const size_t n_need = up4(need.size()), n_lmem = up4(lmem.size()), n_dm = up4(dmask.size());
    std::vector<uint32_t> pack;
    pack.reserve(n_need + n_lmem + n_dm + 2 * (size_t)b.F + ncand);
    pack.insert(pack.end(), need.begin(), need.end());
    pack.resize(n_need, 0);
    pack.insert(pack.end(), lmem.begin(), lmem.end());
    pack.resize(n_need + n_lmem, 0);
    pack.insert(pack.end(), dmask.begin(), dmask.end());
    pack.resize(n_need + n_lmem + n_dm, 0);
    pack.insert(pack.end(), dcount.begin(), dcount.end());
    pack.insert(pack.end(), dstart.begin(), dstart.end());
    pack.insert(pack.end(), order.begin(), order.end());
    DevBuf<uint32_t> dpack;
    dpack.alloc(pack.size(), s);
    COLO_CUDA(cudaMemcpyAsync(dpack.get(), pack.data(), pack.size() * 4, cudaMemcpyHostToDevice, s));
    const uint32_t* d_need = dpack.get();
    const uint32_t* d_lmem = d_need + n_need;
    const uint32_t* d_dmask = d_lmem + n_lmem;
    const uint32_t* d_dcount = d_dmask + n_dm;
    const uint32_t* d_dstart = d_dcount + b.F;
    const uint32_t* d_order = d_dstart + b.F;
    // block-private sums when the level's counters fit in 64 KB of shared memory
    const uint64_t acc64 = ncand * (uint64_t)(m + 2);
    const uint32_t acc_n = acc64 <= kAccMax ? (uint32_t)acc64 : 0u;
    const size_t smem = (size_t)acc_n * 4;
    // a grid-stride loop over 32-cell chunks: as many blocks as fit at once
    auto grid = [&](const void* fn) {
        if (smem > 48 * 1024)
            COLO_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        COLO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem));
        const uint64_t cap = (uint64_t)b.sms * (uint64_t)(per_sm > 0 ? per_sm : 1);
        const uint64_t want = (b.M + 255) / 256;
        return (unsigned)(want < cap ? want : cap);
    };
    KScope ks("filter_level");
#define COLO_FL(WW)                                                                                          \
    k_filter_cells<WW><<<grid((const void*)k_filter_cells<WW>), 256, smem, s>>>(                            \
        b.M, b.J > 1 ? b.cjob.get() : nullptr, b.grids.get(), b.nbmask.get(), d_dmask, d_dcount, d_dstart, d_order,   \
        d_need, d_lmem,                                                                                              \
        k, b.qmask.get(), b.cmask.get(), b.crun.get(), b.qfirst.get(), b.rcnt.get(), d_ub, d_stats, acc_n)
    switch (b.W) {
        case 1: COLO_FL(1); break;
        case 2: COLO_FL(2); break;
        case 3: COLO_FL(3); break;
        case 4: COLO_FL(4); break;
        case 5: COLO_FL(5); break;
        case 6: COLO_FL(6); break;
        case 7: COLO_FL(7); break;
        case 8: COLO_FL(8); break;
        case 12: COLO_FL(12); break;
        case 16: COLO_FL(16); break;
        case 24: COLO_FL(24); break;
        case 32: COLO_FL(32); break;
        default: throw StatusError{COLO_ERR_INTERNAL, "mask words not padded to a supported width"};
    }
#undef COLO_FL
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace colo
