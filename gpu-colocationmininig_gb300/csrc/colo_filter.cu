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

__device__ __forceinline__ bool quad_full(const int32_t* nbz, int ox, int oy, const uint32_t* cmask,
                                          uint32_t W, const uint32_t* need) {
    // quad whose lower-left cell is at offset (ox, oy) from the 3x3 centre Z
    uint32_t m[kMaxW];
    for (uint32_t w = 0; w < W; ++w) m[w] = 0;
    for (int ey = 0; ey < 2; ++ey)
        for (int ex = 0; ex < 2; ++ex) {
            int32_t v = nbz[(oy + ey + 1) * 3 + (ox + ex + 1)];
            if (v < 0) continue;
            for (uint32_t w = 0; w < W; ++w) m[w] |= cmask[(uint64_t)v * W + w];
        }
    for (uint32_t w = 0; w < W; ++w)
        if ((m[w] & need[w]) != need[w]) return false;
    return true;
}

__global__ void k_filter_level(uint64_t nitems, uint64_t ncand, uint32_t k,
                               const uint32_t* __restrict__ cand, const uint32_t* __restrict__ driver,
                               const uint64_t* __restrict__ item_off, const uint32_t* __restrict__ frun_off,
                               const uint32_t* __restrict__ frun, const uint32_t* __restrict__ rcell,
                               const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
                               const JobGrid* __restrict__ grids, const int32_t* __restrict__ nb9,
                               const uint32_t* __restrict__ cmask, const uint32_t* __restrict__ nbmask,
                               uint32_t W, const uint32_t* __restrict__ crun, const uint32_t* __restrict__ rfeat,
                               const uint32_t* __restrict__ rcnt, uint32_t* __restrict__ ub) {
    for (uint64_t item = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; item < nitems;
         item += (uint64_t)gridDim.x * blockDim.x) {
        // candidate owning this item
        uint64_t lo = 0, hi = ncand;
        while (hi - lo > 1) {
            uint64_t mid = (lo + hi) >> 1;
            if (item_off[mid] <= item) lo = mid;
            else hi = mid;
        }
        const uint64_t c = lo;
        const uint32_t* mem = cand + c * k;
        const uint32_t fd = mem[driver[c]];
        const uint32_t run = frun[frun_off[fd] + (uint32_t)(item - item_off[c])];
        const uint32_t C = rcell[run];
        const JobGrid g = grids[cjob[C]];
        if (g.gx < 2 || g.gy < 2) continue;
        const uint32_t m = k < kMaxMembersFiltered ? k : kMaxMembersFiltered;
        uint32_t need[kMaxW];
        for (uint32_t w = 0; w < W; ++w) need[w] = 0;
        for (uint32_t j = 0; j < m; ++j) {
            uint32_t lf = mem[j] - g.f0;
            need[lf >> 5] |= 1u << (lf & 31);
        }
        // every quad containing C lies in C's 3x3 block: all members must be there
        bool present = true;
        for (uint32_t w = 0; w < W; ++w)
            if ((nbmask[(uint64_t)C * W + w] & need[w]) != need[w]) present = false;
        if (!present) continue;
        const uint32_t lfd = fd - g.f0;
        const uint64_t local = ckey[C] - g.key_base;
        const int64_t cx = (int64_t)(local % g.gx), cy = (int64_t)(local / g.gx);
        const int32_t* nbc = nb9 + (uint64_t)C * 9;
        for (int qy = -1; qy <= 0; ++qy)
            for (int qx = -1; qx <= 0; ++qx) {
                int64_t bx = cx + qx, by = cy + qy;
                if (bx < 0 || by < 0 || bx > (int64_t)g.gx - 2 || by > (int64_t)g.gy - 2) continue;
                // visit the quad from its first cell (in (ey, ex) order) holding the driver
                bool first = true;
                for (int ey = 0; ey < 2 && first; ++ey)
                    for (int ex = 0; ex < 2; ++ex) {
                        int ox = qx + ex, oy = qy + ey;
                        if (ox == 0 && oy == 0) { ey = 2; break; }
                        int32_t v = nbc[(oy + 1) * 3 + (ox + 1)];
                        if (v >= 0 && (cmask[(uint64_t)v * W + (lfd >> 5)] >> (lfd & 31) & 1u)) {
                            first = false;
                            break;
                        }
                    }
                if (!first) continue;
                if (!quad_full(nbc, qx, qy, cmask, W, need)) continue;
                // cells of the quad, each counted by its first full quad
                for (int ey = 0; ey < 2; ++ey)
                    for (int ex = 0; ex < 2; ++ex) {
                        int32_t Z = nbc[(qy + ey + 1) * 3 + (qx + ex + 1)];
                        if (Z < 0) continue;
                        const int32_t* nbz = nb9 + (uint64_t)Z * 9;
                        int64_t zx = bx + ex, zy = by + ey;
                        bool claimed = true;
                        for (int py = -1; py <= 0 && claimed; ++py)
                            for (int px = -1; px <= 0; ++px) {
                                int64_t ax = zx + px, ay = zy + py;
                                if (ay > by || (ay == by && ax >= bx)) continue;   // not earlier
                                if (ax < 0 || ay < 0 || ax > (int64_t)g.gx - 2 || ay > (int64_t)g.gy - 2)
                                    continue;
                                if (quad_full(nbz, px, py, cmask, W, need)) {
                                    claimed = false;
                                    break;
                                }
                            }
                        if (!claimed) continue;
                        uint32_t q0 = crun[Z], q1 = crun[Z + 1];
                        for (uint32_t j = 0; j < m; ++j) {
                            uint32_t pos = (uint32_t)lower_bound_dev(rfeat, (uint64_t)q0, (uint64_t)q1, mem[j]);
                            if (pos < q1 && rfeat[pos] == mem[j]) atomicAdd(&ub[c * k + j], rcnt[pos]);
                        }
                    }
            }
    }
}

}  // namespace

void filter_pairs(Batch& b, DevBuf<uint32_t>& ub2, std::vector<uint64_t>& job_off) {
    cudaStream_t s = b.s;
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
    uint64_t blocks = (uint64_t)b.sms * (smem > 100 * 1024 ? 1 : 2);
    uint64_t per = (b.Rn + blocks - 1) / blocks;
    per = (per + kFilterThreads - 1) / kFilterThreads * kFilterThreads;
    blocks = (b.Rn + per - 1) / per;
    KScope ks("filter_pairs");
    k_filter_pairs<<<(unsigned)blocks, kFilterThreads, smem, s>>>(
        b.Rn, b.rcell.get(), b.cjob.get(), b.grids.get(), b.nbmask.get(), b.W, b.rfeat.get(),
        b.rcnt.get(), d_job_off.get(), ub2.get(), acc_dim, per);
    COLO_LAUNCH_CHECK();
    count_launch();
    COLO_CUDA(cudaStreamSynchronize(s));
}

void filter_level(Batch& b, const uint32_t* d_cand, const uint32_t* d_driver, const uint64_t* d_item_off,
                  uint64_t ncand, uint64_t nitems, uint32_t k, uint32_t* d_ub) {
    if (nitems == 0) return;
    if (b.W > kMaxW) throw StatusError{COLO_ERR_CAPACITY, "the filter handles at most 256 features per job"};
    uint64_t blocks = (nitems + 255) / 256;
    uint64_t cap = (uint64_t)b.sms * 16;
    if (blocks > cap) blocks = cap;
    KScope ks("filter_level");
    k_filter_level<<<(unsigned)blocks, 256, 0, b.s>>>(
        nitems, ncand, k, d_cand, d_driver, d_item_off, b.frun_off.get(), b.frun.get(), b.rcell.get(),
        b.ckey.get(), b.cjob.get(), b.grids.get(), b.nb9.get(), b.cmask.get(), b.nbmask.get(), b.W, b.crun.get(),
        b.rfeat.get(), b.rcnt.get(), d_ub);
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace colo
