// colo_bucket.cu -- grid bucketing: a stable radix sort of points by cell key
// into a cell CSR with (cell, feature) runs, per-cell feature masks and the
// geometric 3x3 occupied-neighbour table; then the per-cell neighbourhood
// run lists that the join walks.
//
// Replaces CountCellFeatures (Codes/DeviceProcess.cu:312-369) and
// kernel_CountCellFeatures (Codes/DeviceProcess_Kernel.h:629-647): instead of
// dense totalCells x F count/start arrays, only occupied cells and runs are
// stored, so grids of 10^10 cells cost nothing.
#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

// Cell keys, packed coordinates and (vals non-null) point ids, and the digit
// histograms of every radix pass over the keys (block-private counts added to
// hist once per block), so the sort does not read the keys again to count
// them.  When the sort runs a pass its first pass generates the ids itself.

template <class KT>
__global__ void __launch_bounds__(256) k_cell_keys(
    uint64_t n, const float* __restrict__ x, const float* __restrict__ y, uint32_t F,
    const uint32_t* __restrict__ fstart, const uint32_t* __restrict__ fjob, const JobGrid* __restrict__ grids,
    KT* __restrict__ keys, uint32_t* __restrict__ vals, float2* __restrict__ xy, DevFlags* flags, RadixPlan plan,
    unsigned long long* __restrict__ hist) {
    __shared__ uint32_t h[kRadixMaxPasses * kRadixDigits];
    for (int i = threadIdx.x; i < plan.n * kRadixDigits; i += blockDim.x) h[i] = 0;
    __syncthreads();
    // each block takes one contiguous range of points (coalesced, and a
    // thread's successive points are blockDim apart, so the feature found for
    // one point usually covers the next)
    const uint64_t per = ((n + gridDim.x - 1) / gridDim.x + blockDim.x - 1) / blockDim.x * blockDim.x;
    const uint64_t i0 = (uint64_t)blockIdx.x * per, i1 = i0 + per < n ? i0 + per : n;
    uint32_t f = 0, flo = 1, fhi = 0;   // cached feature and its point range [flo, fhi)
    for (uint64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        if (!(i >= flo && i < fhi)) {
            f = feature_of((uint32_t)i, F, fstart);
            flo = fstart[f];
            fhi = f + 1 < F ? fstart[f + 1] : (uint32_t)n;
        }
        const JobGrid g = grids[fjob[f]];
        const float xi = x[i], yi = y[i];
        xy[i] = make_float2(xi, yi);
        uint64_t c = ref_cell(g, xi, yi);
        if (c >= g.total) {
            atomicAdd(&flags->out_of_grid, 1u);
            c = g.total - 1;
        }
        const KT key = (KT)(g.key_base + c);
        keys[i] = key;
        if (vals) vals[i] = (uint32_t)i;
        for (int p = 0; p < plan.n; ++p)
            atomicAdd(&h[p * kRadixDigits + ((uint32_t)(key >> plan.shift[p]) & ((1u << plan.width[p]) - 1u))], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < plan.n * kRadixDigits; i += blockDim.x) {
        const uint32_t v = h[i];
        if (v) atomicAdd(&hist[i], (unsigned long long)v);
    }
}

// Cell and run heads in the sorted order, counted and compacted in two
// passes over the keys (no flag arrays).  A 2048-point tile is eight warp
// segments of 256 points; a warp reads its segment 32 consecutive points at a
// time (coalesced) and ranks heads with ballots.  Pass 1 stores per tile the
// number of cell heads (high 32 bits) and run heads (low 32 bits); pass 2
// writes each point's cell and the head arrays at the tile's scanned base.
constexpr int kHeadThreads = 256, kHeadRounds = 8, kHeadTile = kHeadThreads * kHeadRounds;
constexpr int kHeadWarps = kHeadThreads / 32;

template <class KT>
__device__ __forceinline__ void head_flags(uint64_t p, uint64_t n, const KT* __restrict__ keys,
                                           const uint32_t* __restrict__ sfeat, bool& ch, bool& rh) {
    ch = rh = false;
    if (p >= n) return;
    ch = p == 0 || keys[p - 1] != keys[p];
    rh = ch || sfeat[p - 1] != sfeat[p];
}

// Ballots of the cell and run heads of the calling warp's segment.
template <class KT>
__device__ __forceinline__ void head_ballots(uint64_t seg, uint64_t n, const KT* __restrict__ keys,
                                             const uint32_t* __restrict__ sfeat, int lane,
                                             uint32_t (&chb)[kHeadRounds], uint32_t (&rhb)[kHeadRounds]) {
#pragma unroll
    for (int r = 0; r < kHeadRounds; ++r) {
        bool ch, rh;
        head_flags(seg + (uint64_t)r * 32 + lane, n, keys, sfeat, ch, rh);
        chb[r] = __ballot_sync(0xffffffffu, ch);
        rhb[r] = __ballot_sync(0xffffffffu, rh);
    }
}

// Sorted copies and pass 1 of the heads in one pass: per point its
// coordinates (one 8-byte gather) and feature (from the feature start table,
// points being grouped by feature; it stays in L1), and per tile the cell
// and run head counts.  A point's predecessor comes from the lane before it
// (lane 0 reads it).  An id outside the points (only after a sort that timed
// out; the host then stops the mine) reads point 0.
template <class KT>
__global__ void __launch_bounds__(kHeadThreads, 8) k_gather_heads(uint64_t n, uint32_t F, const KT* __restrict__ keys,
                                                              const uint32_t* __restrict__ sid,
                                                              const float2* __restrict__ xy,
                                                              const uint32_t* __restrict__ fstart,
                                                              float2* __restrict__ sxy, uint32_t* __restrict__ sfeat,
                                                              uint64_t* __restrict__ partial) {
    __shared__ uint64_t s_tot[kHeadWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t seg = (uint64_t)blockIdx.x * kHeadTile + (uint64_t)w * (32 * kHeadRounds);
    uint64_t v = 0;
#pragma unroll
    for (int r = 0; r < kHeadRounds; ++r) {
        const uint64_t p = seg + (uint64_t)r * 32 + lane;
        const bool in = p < n;
        KT key = 0;
        uint32_t f = 0;
        if (in) {
            uint32_t id = sid[p];
            if (id >= n) id = 0;
            sxy[p] = xy[id];
            f = feature_of(id, F, fstart);
            sfeat[p] = f;
            key = keys[p];
        }
        KT pkey = __shfl_up_sync(0xffffffffu, key, 1);
        uint32_t pf = __shfl_up_sync(0xffffffffu, f, 1);
        if (lane == 0 && in && p > 0) {
            uint32_t pid = sid[p - 1];
            if (pid >= n) pid = 0;
            pkey = keys[p - 1];
            pf = feature_of(pid, F, fstart);
        }
        const bool ch = in && (p == 0 || pkey != key);
        const bool rh = ch || (in && pf != f);
        v += ((uint64_t)__popc(__ballot_sync(0xffffffffu, ch)) << 32) + (uint64_t)__popc(__ballot_sync(0xffffffffu, rh));
    }
    if (lane == 0) s_tot[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t t = 0;
        for (int i = 0; i < kHeadWarps; ++i) t += s_tot[i];
        partial[blockIdx.x] = t;
    }
}

template <class KT>
__global__ void __launch_bounds__(kHeadThreads, 8) k_head_compact(
    uint64_t n, const KT* __restrict__ keys, const uint32_t* __restrict__ sfeat, const uint32_t* __restrict__ fjob,
    const uint64_t* __restrict__ partial, uint64_t* __restrict__ ckey, uint32_t* __restrict__ cstart,
    uint32_t* __restrict__ crun, uint32_t* __restrict__ cjob, uint32_t* __restrict__ rfeat,
    uint32_t* __restrict__ rstart, uint32_t* __restrict__ rcell, uint32_t* __restrict__ scell) {
    __shared__ uint64_t s_tot[kHeadWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t seg = (uint64_t)blockIdx.x * kHeadTile + (uint64_t)w * (32 * kHeadRounds);
    uint32_t chb[kHeadRounds], rhb[kHeadRounds];
    head_ballots(seg, n, keys, sfeat, lane, chb, rhb);
    uint64_t v = 0;
#pragma unroll
    for (int r = 0; r < kHeadRounds; ++r) v += ((uint64_t)__popc(chb[r]) << 32) + (uint64_t)__popc(rhb[r]);
    if (lane == 0) s_tot[w] = v;
    __syncthreads();
    uint64_t ex = partial[blockIdx.x];
    for (int i = 0; i < w; ++i) ex += s_tot[i];
    uint32_t cb = (uint32_t)(ex >> 32), rb = (uint32_t)ex;   // heads before this round
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kHeadRounds; ++r) {
        const uint64_t p = seg + (uint64_t)r * 32 + lane;
        const bool ch = chb[r] >> lane & 1u, rh = rhb[r] >> lane & 1u;
        const uint32_t c = cb + __popc(chb[r] & lt) + (ch ? 1u : 0u) - 1u;   // the cell of p
        const uint32_t ri = rb + __popc(rhb[r] & lt);
        if (p < n) {
            if (scell) scell[p] = c;
            if (ch) {
                ckey[c] = keys[p];
                cstart[c] = (uint32_t)p;
                crun[c] = ri;
                cjob[c] = fjob[sfeat[p]];
            }
            if (rh) {
                rfeat[ri] = sfeat[p];
                rstart[ri] = (uint32_t)p;
                rcell[ri] = c;
            }
        }
        cb += __popc(chb[r]);
        rb += __popc(rhb[r]);
    }
}

__global__ void k_run_tail(uint64_t Rn, uint64_t M, uint64_t n, const uint32_t* __restrict__ rstart,
                           uint32_t* __restrict__ rcnt, uint32_t* __restrict__ cstart,
                           uint32_t* __restrict__ crun) {
    uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < Rn) rcnt[r] = (r + 1 < Rn ? rstart[r + 1] : (uint32_t)n) - rstart[r];
    if (r == 0) {
        cstart[M] = (uint32_t)n;
        crun[M] = (uint32_t)Rn;
    }
}

// Per cell its feature mask (bit lf of word lf / 32 for each of its runs' local
// features): a thread walks the cell's runs, which ascend by feature, and writes
// every word of the row (no clearing pass, no atomics).
__global__ void k_cell_masks(uint64_t M, const uint32_t* __restrict__ crun, const uint32_t* __restrict__ rfeat,
                             const uint32_t* __restrict__ cjob, const JobGrid* __restrict__ grids, uint32_t W,
                             uint32_t* __restrict__ cmask) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M) return;
    const uint32_t f0 = grids[cjob[c]].f0;
    uint32_t r = crun[c];
    const uint32_t r1 = crun[c + 1];
    uint32_t* row = cmask + c * W;
    for (uint32_t w = 0; w < W; ++w) {
        uint32_t bits = 0;
        for (; r < r1; ++r) {
            const uint32_t lf = rfeat[r] - f0;
            if ((lf >> 5) != w) break;
            bits |= 1u << (lf & 31);
        }
        row[w] = bits;
    }
}

// rowstart[Y] = first occupied cell whose key is at or after the first key of
// grid row Y (rows of all jobs, job j's row y at Y = row_base_j + y);
// rowstart[rows] = M.
__global__ void k_row_starts(uint64_t rows, uint32_t J, uint64_t M, const uint64_t* __restrict__ ckey,
                             const JobGrid* __restrict__ grids, uint32_t* __restrict__ rowstart) {
    const uint64_t Y = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (Y > rows) return;
    if (Y == rows) {
        rowstart[Y] = (uint32_t)M;
        return;
    }
    uint32_t lo = 0, hi = J;   // last job whose first row is <= Y
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (grids[mid].row_base <= Y) lo = mid;
        else hi = mid;
    }
    const JobGrid g = grids[lo];
    const uint64_t key = g.key_base + (Y - g.row_base) * g.gx;
    rowstart[Y] = (uint32_t)lower_bound_dev(ckey, (uint64_t)0, M, key);
}

// nb9[c*9 + (dy+1)*3 + (dx+1)] = occupied index of the geometric neighbour
// (cx+dx, cy+dy) inside the job's grid, or -1.  Keys ascend along a grid row,
// so the row of the cell itself is read from the adjacent entries and each
// other row needs one lower_bound (above: after c, below: before c).
//
// qfirst[c] bit q: c is the first occupied cell of its quad q in (ey, ex)
// order (the level filter counts each full quad once, at that cell).  Quad q
// has lower-left cell (cx+qx, cy+qy), qx = (q & 1) - 1, qy = (q >> 1) - 1, and
// holds c at corner (ex, ey) = (-qx, -qy); quads outside 0 <= bx <= gx-2,
// 0 <= by <= gy-2 are never full and get no bit.
// rowstart (optional, rows + 1 entries) bounds the search of a row to the
// cells of that row.
__global__ void __launch_bounds__(128, 16) k_nb9(uint64_t M, const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
                      const JobGrid* __restrict__ grids, const uint32_t* __restrict__ rowstart,
                      int32_t* __restrict__ nb9, uint8_t* __restrict__ qfirst) {
    uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M) return;
    const JobGrid g = grids[cjob[c]];
    const uint64_t key = ckey[c];
    uint64_t ucx, ucy;
    cell_col_row(key - g.key_base, g.gx, ucx, ucy);
    const int64_t cx = (int64_t)ucx, cy = (int64_t)ucy;
    const int64_t x0 = cx > 0 ? cx - 1 : 0, x1 = cx + 1 < (int64_t)g.gx ? cx + 1 : cx;
    int32_t* out = nb9 + c * 9;
    uint32_t occ = 0;   // bit (dy+1)*3 + (dx+1): that neighbour is occupied
    for (int dy = -1; dy <= 1; ++dy) {
        int32_t v0 = -1, v1 = -1, v2 = -1;
        const int64_t ny = cy + dy;
        if (dy == 0) {
            v1 = (int32_t)c;
            if (cx > 0 && c > 0 && ckey[c - 1] == key - 1) v0 = (int32_t)(c - 1);
            if (cx + 1 < (int64_t)g.gx && c + 1 < M && ckey[c + 1] == key + 1) v2 = (int32_t)(c + 1);
        } else if (ny >= 0 && ny < (int64_t)g.gy) {
            const uint64_t k0 = g.key_base + (uint64_t)ny * g.gx + (uint64_t)x0;
            const uint64_t k1 = g.key_base + (uint64_t)ny * g.gx + (uint64_t)x1;
            // 32-bit positions (M < 2^32): the search is most of this kernel's instructions
            uint32_t lo = dy < 0 ? 0u : (uint32_t)c + 1u, hi = dy < 0 ? (uint32_t)c : (uint32_t)M;
            if (rowstart) {
                const uint64_t Y = g.row_base + (uint64_t)ny;
                lo = rowstart[Y];
                hi = rowstart[Y + 1];
            }
            while (lo < hi) {
                const uint32_t mid = lo + ((hi - lo) >> 1);
                if (ckey[mid] < k0) lo = mid + 1;
                else hi = mid;
            }
            for (uint32_t pos = lo; pos < (uint32_t)M && ckey[pos] <= k1; ++pos) {
                const int64_t dx = (int64_t)(ckey[pos] - g.key_base - (uint64_t)ny * g.gx) - cx;
                if (dx < 0) v0 = (int32_t)pos;
                else if (dx == 0) v1 = (int32_t)pos;
                else v2 = (int32_t)pos;
            }
        }
        out[(dy + 1) * 3 + 0] = v0;
        out[(dy + 1) * 3 + 1] = v1;
        out[(dy + 1) * 3 + 2] = v2;
        occ |= ((v0 >= 0 ? 1u : 0u) | (v1 >= 0 ? 2u : 0u) | (v2 >= 0 ? 4u : 0u)) << ((dy + 1) * 3);
    }
    uint32_t qf = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int qx = (q & 1) - 1, qy = (q >> 1) - 1;
        const int64_t bx = cx + qx, by = cy + qy;
        if (!(bx >= 0 && by >= 0 && bx + 2 <= (int64_t)g.gx && by + 2 <= (int64_t)g.gy)) continue;
        const int ex = -qx, ey = -qy;
        bool first = true;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            if (e >= ey * 2 + ex) break;
            const int ox = (e & 1) - ex, oy = (e >> 1) - ey;
            if (occ >> ((oy + 1) * 3 + (ox + 1)) & 1u) first = false;
        }
        if (first) qf |= 1u << q;
    }
    qfirst[c] = (uint8_t)qf;
}

// Per cell: the feature masks of the four quads (2x2 cell blocks) containing
// the cell, qmask[(c*4 + q)*W + w] with q = (qy+1)*2 + (qx+1) for the quad
// whose lower-left cell is (cx+qx, cy+qy), qx, qy in {-1, 0} -- q ascends in
// the quads' (by, bx) order.  A quad outside 0 <= bx <= gx-2,
// 0 <= by <= gy-2 gets an empty mask, so it is never full.
// nbmask[c*W + w] = union of the masks of the occupied cells of c's 3x3 block.
// One thread per cell and WT mask words (WT = W); rows are read and written
// as 16-byte vectors when W is a multiple of 4.
template <int WT>
__device__ __forceinline__ void ld_row(const uint32_t* __restrict__ p, uint32_t (&o)[WT]) {
    if constexpr (WT % 4 == 0) {
#pragma unroll
        for (int i = 0; i < WT / 4; ++i) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(p) + i);
            o[4 * i] = v.x;
            o[4 * i + 1] = v.y;
            o[4 * i + 2] = v.z;
            o[4 * i + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < WT; ++i) o[i] = __ldg(p + i);
    }
}

template <int WT>
__device__ __forceinline__ void st_row(uint32_t* __restrict__ p, const uint32_t (&v)[WT]) {
    if constexpr (WT % 4 == 0) {
#pragma unroll
        for (int i = 0; i < WT / 4; ++i)
            reinterpret_cast<uint4*>(p)[i] = make_uint4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < WT; ++i) p[i] = v[i];
    }
}

constexpr int kQuadThreads = 128;

// Features a block of cells counts in shared memory for the driver-list sizes
// (larger batches count with global atomics).
constexpr uint32_t kQuadHist = 1024;

// Per cell: the four quad masks and the 3x3 mask (nbmask), the queue of cells
// that need a neighbourhood run list, and the driver-list sizes: dcnt[f] =
// cells whose 3x3 mask holds f.  A block walks 128 cells at a time over a
// strided range and keeps one histogram for all of them (one global atomic per
// feature per block at the end); a warp's 32 cells are counted by a bit
// transpose (lane b holds feature b's column of the warp's cell x feature
// matrix and adds its popcount).
template <int WT>
__global__ void __launch_bounds__(kQuadThreads) k_quad_masks(
    uint64_t M, const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
    const JobGrid* __restrict__ grids, const int32_t* __restrict__ nb9, const uint32_t* __restrict__ cmask,
    uint32_t* __restrict__ qmask, uint32_t* __restrict__ nbmask, uint32_t* __restrict__ listq,
    uint32_t* __restrict__ nlistq, uint32_t F, uint32_t* __restrict__ dcnt) {
    __shared__ uint32_t s_hist[kQuadHist];
    __shared__ uint32_t s_cnt[kQuadThreads / 32], s_base;
    const bool local_hist = F <= kQuadHist;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (local_hist)
        for (uint32_t i = threadIdx.x; i < F; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
    for (uint64_t c0 = (uint64_t)blockIdx.x * kQuadThreads; c0 < M; c0 += (uint64_t)gridDim.x * kQuadThreads) {
        const uint64_t c = c0 + threadIdx.x;
        bool above = false;
        uint32_t all[WT];
#pragma unroll
        for (int w = 0; w < WT; ++w) all[w] = 0;
        uint32_t f0 = 0;
        if (c < M) {
            const JobGrid g = grids[cjob[c]];
            f0 = g.f0;
            uint64_t ucx, ucy;
            cell_col_row(ckey[c] - g.key_base, g.gx, ucx, ucy);
            const int64_t cx = (int64_t)ucx, cy = (int64_t)ucy;
            int32_t nb[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) nb[q] = nb9[c * 9 + q];
            uint32_t m[9][WT];
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                if (nb[q] >= 0) {
                    ld_row<WT>(cmask + (uint64_t)nb[q] * WT, m[q]);
                } else {
#pragma unroll
                    for (int w = 0; w < WT; ++w) m[q][w] = 0;
                }
#pragma unroll
                for (int w = 0; w < WT; ++w) all[w] |= m[q][w];
            }
            st_row<WT>(nbmask + c * WT, all);
            // the cell needs a neighbourhood run list when its 3x3 block holds a
            // feature above its own lowest one (m[4] is the cell's own mask; the block
            // is the union over all nine slots, a superset of the adjacent cells):
            // such cells are queued for the list kernels
            bool seen = false;
#pragma unroll
            for (int w = 0; w < WT; ++w) {
                const uint32_t own = m[4][w];
                if (seen) {
                    above |= all[w] != 0;
                } else if (own) {
                    seen = true;
                    const uint32_t low = own & (0u - own);
                    above |= (all[w] & ~((low << 1) - 1u)) != 0;
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int qx = (q & 1) - 1, qy = (q >> 1) - 1;
                const int64_t bx = cx + qx, by = cy + qy;
                const bool valid = bx >= 0 && by >= 0 && bx + 2 <= (int64_t)g.gx && by + 2 <= (int64_t)g.gy;
                uint32_t qm[WT];
#pragma unroll
                for (int w = 0; w < WT; ++w)
                    qm[w] = valid ? (m[(qy + 1) * 3 + qx + 1][w] | m[(qy + 1) * 3 + qx + 2][w] |
                                     m[(qy + 2) * 3 + qx + 1][w] | m[(qy + 2) * 3 + qx + 2][w])
                                  : 0u;
                st_row<WT>(qmask + (c * 4 + q) * WT, qm);
            }
        }
        // driver-list sizes (lanes of another job than lane 0's, at job boundaries of a
        // batch, count one bit at a time)
        {
            const uint32_t fl = __shfl_sync(0xffffffffu, f0, 0);
            if (__all_sync(0xffffffffu, c >= M || f0 == fl)) {
#pragma unroll
                for (int w = 0; w < WT; ++w) {
                    if (!__any_sync(0xffffffffu, all[w])) continue;
                    const uint32_t n = __popc(warp_transpose32(all[w]));
                    if (n) {
                        const uint32_t f = fl + (uint32_t)w * 32 + (uint32_t)lane;
                        if (local_hist) atomicAdd(&s_hist[f], n);
                        else atomicAdd(&dcnt[f], n);
                    }
                }
            } else {
#pragma unroll
                for (int w = 0; w < WT; ++w)
                    for (uint32_t bits = all[w]; bits; bits &= bits - 1)
                        atomicAdd(&dcnt[f0 + (uint32_t)w * 32 + (uint32_t)(__ffs(bits) - 1)], 1u);
            }
        }
        // one atomic per block and round for the queue
        const uint32_t has = __ballot_sync(0xffffffffu, above);
        if (lane == 0) s_cnt[wid] = (uint32_t)__popc(has);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int w = 0; w < kQuadThreads / 32; ++w) {
                const uint32_t v = s_cnt[w];
                s_cnt[w] = t;
                t += v;
            }
            s_base = t ? atomicAdd(nlistq, t) : 0u;
        }
        __syncthreads();
        if (above) listq[s_base + s_cnt[wid] + __popc(has & ((1u << lane) - 1u))] = (uint32_t)c;
        __syncthreads();   // s_cnt and s_base are rewritten by the next round
    }
    if (local_hist) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < F; i += blockDim.x)
            if (s_hist[i]) atomicAdd(&dcnt[i], s_hist[i]);
    }
}

// Runs per feature: a block-local histogram (F <= kHistMax), else global atomics.
constexpr uint32_t kHistMax = 12288;

__global__ void k_feature_runs(uint64_t Rn, uint32_t F, const uint32_t* __restrict__ rfeat, uint32_t* __restrict__ cnt) {
    extern __shared__ uint32_t h[];
    const bool local = F <= kHistMax;
    if (local)
        for (uint32_t i = threadIdx.x; i < F; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < Rn; r += (uint64_t)gridDim.x * blockDim.x) {
        if (local) atomicAdd(&h[rfeat[r]], 1u);
        else atomicAdd(&cnt[rfeat[r]], 1u);
    }
    __syncthreads();
    if (local)
        for (uint32_t i = threadIdx.x; i < F; i += blockDim.x)
            if (h[i]) atomicAdd(&cnt[i], h[i]);
}

// ---------------------------------------------------------------------------
// Neighbourhood run lists.  For cell c the adjacent cells A(c) (the
// reference's stencil, ascending cell ids) contribute their runs; NRL(c)
// orders them by (feature, cell), which is the order the reference's kernels
// visit candidates of one feature.  For each run of c the list suffix with
// higher features holds exactly the join targets of the run's points.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int adjacent_cells(uint64_t c, const uint64_t* ckey, const uint32_t* cjob,
                                              const JobGrid* grids, const int32_t* nb9,
                                              int32_t* out) {
    const JobGrid g = grids[cjob[c]];
    uint64_t ucx, ucy;
    cell_col_row(ckey[c] - g.key_base, g.gx, ucx, ucy);
    const uint32_t cx = (uint32_t)ucx;
    int cnt = 0;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            int32_t v = nb9[c * 9 + (dy + 1) * 3 + (dx + 1)];
            if (v < 0) continue;
            uint32_t nx = (uint32_t)((int64_t)cx + dx);
            if (!ref_adjacent_col(cx, nx, g.gx)) continue;
            out[cnt++] = v;
        }
    return cnt;
}

// A cell's list keeps only the adjacent runs with a feature above the cell's
// lowest own feature: the join reads a list from an own run's suffix on, and
// the lowest own run's suffix starts past every entry of feature <= its own.
// Most lists are then empty; the cells whose 3x3 mask allows one were queued
// by k_quad_masks (nrl_len is zero for the others).  Grid-stride over the queue.
__global__ void k_nrl_count(const uint32_t* __restrict__ listq, const uint32_t* __restrict__ nlistq,
                            const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
                            const JobGrid* __restrict__ grids, const int32_t* __restrict__ nb9,
                            const uint32_t* __restrict__ crun, const uint32_t* __restrict__ rfeat,
                            uint32_t* __restrict__ nrl_len) {
    const uint32_t n = *nlistq;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t c = listq[i];
        const uint32_t fmin = rfeat[crun[c]];
        int32_t adj[9];
        const int na = adjacent_cells(c, ckey, cjob, grids, nb9, adj);
        uint32_t nr = 0;
        for (int t = 0; t < na; ++t) {
            const uint64_t q0 = crun[adj[t]], q1 = crun[adj[t] + 1];
            nr += (uint32_t)(q1 - lower_bound_dev(rfeat, q0, q1, fmin + 1));
        }
        nrl_len[c] = nr;
    }
}

// The list of cell c (lanes l = 0..G-1 of a group share it).  In the full
// (feature, slot) order a run of feature f in adjacent slot s is at the sum
// over slots of (#runs with feature < f) plus the number of earlier slots
// that also hold f; the kept list drops the off0 entries of feature <= the
// cell's lowest own feature.  Per own run of the cell: the first entry with a
// higher feature and the number of target points from there on (the points
// of each adjacent cell past its runs of features <= f), both from one binary
// search per slot.
template <int G>
__device__ __forceinline__ void nrl_cell(uint64_t c, int l, const uint64_t* __restrict__ ckey,
                                         const uint32_t* __restrict__ cjob, const JobGrid* __restrict__ grids,
                                         const int32_t* __restrict__ nb9, const uint32_t* __restrict__ cstart,
                                         const uint32_t* __restrict__ crun, const uint32_t* __restrict__ rfeat,
                                         const uint32_t* __restrict__ rstart, const uint32_t* __restrict__ cmask,
                                         const uint32_t* __restrict__ rcnt, uint32_t W,
                                         const uint64_t* __restrict__ nrl_off, uint2* __restrict__ nrl_ent,
                                         uint64_t* __restrict__ run_sfx, uint32_t* __restrict__ run_qn,
                                         uint32_t* __restrict__ run_L) {
    int32_t adj[9];
    const int na = adjacent_cells(c, ckey, cjob, grids, nb9, adj);
    const uint32_t fmin = rfeat[crun[c]];
    uint32_t q0[9], q1[9], pre[10];
    uint64_t off0 = 0;
    pre[0] = 0;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        if (t < na) {
            q0[t] = crun[adj[t]];
            q1[t] = crun[adj[t] + 1];
            off0 += lower_bound_dev(rfeat, (uint64_t)q0[t], (uint64_t)q1[t], fmin + 1) - q0[t];
        } else {
            q0[t] = q1[t] = 0;
        }
        pre[t + 1] = pre[t] + (q1[t] - q0[t]);
    }
    const uint64_t base = nrl_off[c] - off0;   // where entry 0 of the full order would be
    for (uint32_t e = l; e < pre[9]; e += G) {
        int sl = 0;
        uint32_t r = 0;
#pragma unroll
        for (int t = 0; t < 9; ++t)
            if (e >= pre[t] && e < pre[t + 1]) {
                sl = t;
                r = q0[t] + (e - pre[t]);
            }
        const uint32_t f = rfeat[r];
        if (f <= fmin) continue;
        uint64_t pos = 0;
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            if (t < na) {
                const uint32_t lb = (uint32_t)lower_bound_dev(rfeat, (uint64_t)q0[t], (uint64_t)q1[t], f);
                pos += lb - q0[t];
                if (t < sl && lb < q1[t] && rfeat[lb] == f) pos += 1;
            }
        }
        nrl_ent[base + pos] = make_uint2(rstart[r], rcnt[r]);
    }
    for (uint32_t r = crun[c] + l; r < crun[c + 1]; r += G) {
        const uint32_t f = rfeat[r];
        uint64_t sfx = base;
        uint32_t L = 0;
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            if (t < na) {
                const uint32_t ub = (uint32_t)lower_bound_dev(rfeat, (uint64_t)q0[t], (uint64_t)q1[t], f + 1);
                sfx += ub - q0[t];
                if (ub < q1[t]) L += cstart[adj[t] + 1] - rstart[ub];
            }
        }
        run_sfx[r] = sfx;
        run_qn[r] = (uint32_t)(nrl_off[c + 1] - sfx);
        run_L[r] = L;
    }
}

constexpr uint32_t kBigList = 512;   // cells with longer lists get a warp each

// One thread per cell: the list is the 9-way merge, by (feature, slot), of
// the adjacent cells' runs above the lowest own feature (each slot ascending
// by feature).  The running point count P gives the suffix counts: the
// cell's own run of feature f gets sfx = the first position after every
// entry of feature <= f and L = (points in the list) - P(sfx).  Cells with
// lists longer than kBigList are queued for k_nrl_fill_big.
__device__ __forceinline__ void nrl_fill_cell(uint64_t c, const uint64_t* __restrict__ ckey,
                                              const uint32_t* __restrict__ cjob, const JobGrid* __restrict__ grids,
                                              const int32_t* __restrict__ nb9, const uint32_t* __restrict__ crun,
                                              const uint32_t* __restrict__ rfeat, const uint32_t* __restrict__ rstart,
                                              const uint32_t* __restrict__ rcnt, const uint64_t* __restrict__ nrl_off,
                                              uint2* __restrict__ nrl_ent, uint64_t* __restrict__ run_sfx,
                                              uint32_t* __restrict__ run_qn, uint32_t* __restrict__ run_L,
                                              uint32_t* __restrict__ big, uint32_t* __restrict__ nbig) {
    const uint64_t base = nrl_off[c], kept = nrl_off[c + 1] - base;
    if (kept == 0) return;   // no own run has targets (run_L is zero)
    const uint32_t r0 = crun[c], r1 = crun[c + 1];
    if (kept > kBigList) {   // the merge below is serial in the list
        big[atomicAdd(nbig, 1u)] = (uint32_t)c;
        return;
    }
    int32_t adj[9];
    const int na = adjacent_cells(c, ckey, cjob, grids, nb9, adj);
    const uint32_t fmin = rfeat[r0];
    // each slot's cursor starts at its first run above the lowest own feature
    uint32_t h[9], e[9], f[9];
    int own = 0;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        if (t < na) {
            e[t] = crun[adj[t] + 1];
            h[t] = (uint32_t)lower_bound_dev(rfeat, (uint64_t)crun[adj[t]], (uint64_t)e[t], fmin + 1);
            f[t] = h[t] < e[t] ? rfeat[h[t]] : 0xffffffffu;
            if ((uint64_t)adj[t] == c) own = t;
        } else {
            h[t] = e[t] = 0;
            f[t] = 0xffffffffu;
        }
    }
    // the lowest own run's suffix is the whole list
    const uint64_t end = base + kept;
    run_sfx[r0] = base;
    run_qn[r0] = (uint32_t)kept;
    run_L[r0] = 0;
    uint64_t pos = base;
    uint32_t P = 0, pend_r = 0, pend_f = 0;
    bool pend = false;
    for (;;) {
        int ts = 0;
        uint32_t fm = f[0];
#pragma unroll
        for (int t = 1; t < 9; ++t)
            if (f[t] < fm) {
                fm = f[t];
                ts = t;
            }
        if (fm == 0xffffffffu) break;
        if (pend && pend_f < fm) {
            run_sfx[pend_r] = pos;
            run_qn[pend_r] = (uint32_t)(end - pos);
            run_L[pend_r] = P;
            pend = false;
        }
        uint32_t r = 0;
#pragma unroll
        for (int t = 0; t < 9; ++t)
            if (t == ts) {
                r = h[t]++;
                f[t] = h[t] < e[t] ? rfeat[h[t]] : 0xffffffffu;
            }
        const uint32_t rc = rcnt[r];
        nrl_ent[pos++] = make_uint2(rstart[r], rc);
        P += rc;
        if (ts == own) {
            pend = true;
            pend_r = r;
            pend_f = fm;
        }
    }
    if (pend) {
        run_sfx[pend_r] = pos;
        run_qn[pend_r] = 0;
        run_L[pend_r] = P;
    }
    for (uint32_t r = r0; r < r1; ++r) run_L[r] = P - run_L[r];
}

// Grid-stride over the queued cells; run_L is zero for every run of the
// others, and run_sfx is read only where run_L > 0.
__global__ void k_nrl_fill(const uint32_t* __restrict__ work, const uint32_t* __restrict__ nwork,
                           const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
                           const JobGrid* __restrict__ grids, const int32_t* __restrict__ nb9,
                           const uint32_t* __restrict__ crun, const uint32_t* __restrict__ rfeat,
                           const uint32_t* __restrict__ rstart, const uint32_t* __restrict__ rcnt,
                           const uint64_t* __restrict__ nrl_off, uint2* __restrict__ nrl_ent,
                           uint64_t* __restrict__ run_sfx, uint32_t* __restrict__ run_qn,
                           uint32_t* __restrict__ run_L, uint32_t* __restrict__ big, uint32_t* __restrict__ nbig) {
    const uint32_t n = *nwork;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        nrl_fill_cell(work[i], ckey, cjob, grids, nb9, crun, rfeat, rstart, rcnt, nrl_off, nrl_ent, run_sfx, run_qn,
                      run_L, big, nbig);
}

// A warp per queued cell (grid-stride over the queue).
__global__ void k_nrl_fill_big(const uint32_t* __restrict__ big, const uint32_t* __restrict__ nbig,
                               const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
                               const JobGrid* __restrict__ grids, const int32_t* __restrict__ nb9,
                               const uint32_t* __restrict__ cstart, const uint32_t* __restrict__ crun,
                               const uint32_t* __restrict__ rfeat, const uint32_t* __restrict__ rstart,
                               const uint32_t* __restrict__ cmask, uint32_t W,
                               const uint32_t* __restrict__ rcnt, const uint64_t* __restrict__ nrl_off,
                               uint2* __restrict__ nrl_ent, uint64_t* __restrict__ run_sfx,
                               uint32_t* __restrict__ run_qn, uint32_t* __restrict__ run_L) {
    const uint32_t n = *nbig;
    const int lane = threadIdx.x & 31;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5)
        nrl_cell<32>(big[i], lane, ckey, cjob, grids, nb9, cstart, crun, rfeat, rstart, cmask, rcnt, W, nrl_off,
                     nrl_ent, run_sfx, run_qn, run_L);
}

inline unsigned grid_for(uint64_t n, int threads) {
    uint64_t g = (n + threads - 1) / threads;
    return (unsigned)(g == 0 ? 1 : g);
}

}  // namespace

// Cell keys, the stable sort by key, the sorted point copies and the cell /
// run compaction, with KT = 32-bit keys when every key fits (less traffic per
// radix pass), else 64-bit.
template <class KT>
void sort_and_compact(Batch& b) {
    cudaStream_t s = b.s;
    const uint64_t n = b.N;
    DevBuf<KT> keys;
    keys.alloc(n, s);
    b.sid.alloc(n, s);
    const int bits = sizeof(KT) == 4 && b.key_bits > 32 ? 32 : (int)b.key_bits;
    const RadixPlan plan = radix_plan(bits);
    DevBuf<unsigned long long> hist;
    hist.alloc((uint64_t)(plan.n > 0 ? plan.n : 1) * kRadixDigits, s);
    hist.zero(s);
    {
    KScope ks("cell_keys");
    b.xy.alloc(n, s);
    const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)b.sms * 8);
    // the ids are written here only when the sort runs no pass (its first pass makes them)
    const bool sorted_ids = n > 1 && bits > 0;
    k_cell_keys<KT><<<(unsigned)(blocks ? blocks : 1), 256, 0, s>>>(n, b.x, b.y, b.F, b.fstart.get(), b.fjob.get(), b.grids.get(),
                                                                    keys.get(), sorted_ids ? nullptr : b.sid.get(),
                                                                    b.xy.get(), b.flags.get(), plan, hist.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    }
    // a look-back timeout lands in the batch's flags, read with the compaction totals
    radix_sort(keys, b.sid, n, bits, s, "radix_sort", hist.get(), &b.flags.get()->timeout, b.test_spin, true);

    b.sxy.alloc(n, s);
    b.sfeat.alloc(n, s);
    const uint64_t tiles = (n + kHeadTile - 1) / kHeadTile;
    DevBuf<uint64_t> part;
    part.alloc(tiles + 1, s);
    uint64_t totals = 0;
    {
        KScope ks("gather_sorted");
        k_gather_heads<KT><<<(unsigned)tiles, kHeadThreads, 0, s>>>(n, b.F, keys.get(), b.sid.get(), b.xy.get(),
                                                                   b.fstart.get(), b.sxy.get(), b.sfeat.get(),
                                                                   part.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    {
        KScope ks("cell_compact");
        // the sort's timeout word comes back with the totals: after a timeout the keys are not
        // a sorted permutation, and nothing past this point may read them
        uint32_t sort_err = 0;
        COLO_CUDA(cudaMemcpyAsync(&sort_err, &b.flags.get()->timeout, 4, cudaMemcpyDeviceToHost, s));
        scan_partials_u64(part.get(), tiles, s, &totals);
        if (sort_err) throw StatusError{COLO_ERR_TIMEOUT, "radix sort: a tile waited too long for its predecessors"};
    }
    const uint32_t M = (uint32_t)(totals >> 32), Rn = (uint32_t)totals;
    b.M = M;
    b.Rn = Rn;
    b.ckey.alloc(M, s);
    b.cstart.alloc(M + 1, s);
    b.crun.alloc(M + 1, s);
    b.cjob.alloc(M, s);
    b.rfeat.alloc(Rn, s);
    b.rstart.alloc(Rn, s);
    b.rcnt.alloc(Rn, s);
    b.rcell.alloc(Rn, s);
    if (b.keep_scell) b.scell.alloc(n, s);
    {
        KScope ks("cell_compact");
        k_head_compact<KT><<<(unsigned)tiles, kHeadThreads, 0, s>>>(
            n, keys.get(), b.sfeat.get(), b.fjob.get(), part.get(), b.ckey.get(), b.cstart.get(), b.crun.get(),
            b.cjob.get(), b.rfeat.get(), b.rstart.get(), b.rcell.get(), b.keep_scell ? b.scell.get() : nullptr);
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    {
        KScope ks("cell_compact");
        k_run_tail<<<grid_for(Rn, 256), 256, 0, s>>>(Rn, M, n, b.rstart.get(), b.rcnt.get(), b.cstart.get(),
                                                      b.crun.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
}

void bucket_points(Batch& b) {
    cudaStream_t s = b.s;
    if (b.key_bits <= 32) sort_and_compact<uint32_t>(b);
    else sort_and_compact<uint64_t>(b);
    const uint64_t M = b.M, Rn = b.Rn;

    b.cmask.alloc((uint64_t)M * b.W, s);
    {
        KScope ks("cell_masks");
        k_cell_masks<<<grid_for(M, 256), 256, 0, s>>>(M, b.crun.get(), b.rfeat.get(), b.cjob.get(), b.grids.get(),
                                                       b.W, b.cmask.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    b.nb9.alloc((uint64_t)M * 9, s);
    b.qfirst.alloc(M, s);
    {
        KScope ks("cell_neighbours");
        // the row table when it is not much larger than the cell list
        const bool table = b.rows < (1ull << 31) && b.rows <= 4 * (uint64_t)M + (1u << 20);
        b.rowstart.release();
        if (table) {
            b.rowstart.alloc(b.rows + 1, s);
            k_row_starts<<<grid_for(b.rows + 1, 256), 256, 0, s>>>(b.rows, b.J, M, b.ckey.get(), b.grids.get(),
                                                                  b.rowstart.get());
            COLO_LAUNCH_CHECK();
            count_launch();
        }
        k_nb9<<<grid_for(M, 128), 128, 0, s>>>(M, b.ckey.get(), b.cjob.get(), b.grids.get(),
                                               table ? b.rowstart.get() : nullptr, b.nb9.get(), b.qfirst.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    b.nbmask.alloc((uint64_t)M * b.W, s);
    b.qmask.alloc((uint64_t)M * 4 * b.W, s);
    b.listq.alloc(M ? M : 1, s);
    b.nlistq.alloc(1, s);
    b.nlistq.zero(s);
    // cells per driver list (3x3 blocks holding each feature), counted with the masks
    DevBuf<uint32_t> dcnt;
    dcnt.alloc(b.F ? b.F : 1, s);
    dcnt.zero(s);
    {
        KScope ks("quad_masks");
        // one wave of resident blocks (each keeps one histogram for all its cells)
#define COLO_QM(WW)                                                                                          \
    do {                                                                                                     \
        int per_sm = 1;                                                                                      \
        COLO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_quad_masks<WW>, kQuadThreads, 0)); \
        const unsigned qblocks = (unsigned)std::max<uint64_t>(                                               \
            1, std::min<uint64_t>(grid_for(M, kQuadThreads), (uint64_t)b.sms * (uint64_t)std::max(per_sm, 1))); \
        k_quad_masks<WW><<<qblocks, kQuadThreads, 0, s>>>(                                                   \
            M, b.ckey.get(), b.cjob.get(), b.grids.get(), b.nb9.get(), b.cmask.get(), b.qmask.get(),         \
            b.nbmask.get(), b.listq.get(), b.nlistq.get(), b.F, dcnt.get());                                 \
    } while (0)
        switch (b.W) {
            case 1: COLO_QM(1); break;
            case 2: COLO_QM(2); break;
            case 3: COLO_QM(3); break;
            case 4: COLO_QM(4); break;
            case 5: COLO_QM(5); break;
            case 6: COLO_QM(6); break;
            case 7: COLO_QM(7); break;
            case 8: COLO_QM(8); break;
            case 12: COLO_QM(12); break;
            case 16: COLO_QM(16); break;
            case 24: COLO_QM(24); break;
            case 32: COLO_QM(32); break;
            default: throw StatusError{COLO_ERR_CAPACITY, "the quad filter handles at most 1024 features per job"};
        }
#undef COLO_QM
        COLO_LAUNCH_CHECK();
        count_launch();
    }

    // runs per feature
    {
        KScope ks("run_index");
        DevBuf<uint32_t> cnt;
        cnt.alloc(b.F ? b.F : 1, s);
        cnt.zero(s);
        const uint64_t blocks = std::min<uint64_t>((Rn + 255) / 256, (uint64_t)b.sms * 4);
        const size_t smem = b.F <= kHistMax ? (size_t)b.F * 4 : 0;
        if (smem > 48 * 1024)
            COLO_CUDA(cudaFuncSetAttribute(k_feature_runs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (Rn) {
            k_feature_runs<<<(unsigned)(blocks ? blocks : 1), 256, smem, s>>>(Rn, b.F, b.rfeat.get(), cnt.get());
            COLO_LAUNCH_CHECK();
            count_launch();
        }
        // the run counts, list sizes and error flags come back with one wait
        std::vector<uint32_t> hc(b.F), hd(b.F);
        DevFlags hf;
        if (b.F) {
            COLO_CUDA(cudaMemcpyAsync(hc.data(), cnt.get(), b.F * 4, cudaMemcpyDeviceToHost, s));
            COLO_CUDA(cudaMemcpyAsync(hd.data(), dcnt.get(), b.F * 4, cudaMemcpyDeviceToHost, s));
        }
        COLO_CUDA(cudaMemcpyAsync(&hf, b.flags.get(), sizeof(hf), cudaMemcpyDeviceToHost, s));
        stream_wait(s);
        b.h_frun_off.assign(b.F + 1, 0);
        for (uint32_t f = 0; f < b.F; ++f) b.h_frun_off[f + 1] = b.h_frun_off[f] + hc[f];
        b.h_dcnt.assign(hd.begin(), hd.end());
        b.h_doff.assign(b.F + 1, 0);
        b.dlist_have.assign(b.F, 0);
        if (hf.timeout) throw StatusError{COLO_ERR_TIMEOUT, "radix sort: a tile waited too long for its predecessors"};
        if (hf.out_of_grid)
            throw StatusError{COLO_ERR_INPUT, std::to_string(hf.out_of_grid) +
                                                  " point(s) fall outside the grid derived from the bounds line"};
    }
}

void build_neighborhoods(Batch& b) {
    cudaStream_t s = b.s;
    const uint64_t M = b.M;
    DevBuf<uint32_t> nrl_len;
    nrl_len.alloc(M ? M : 1, s);
    nrl_len.zero(s);
    const unsigned qgrid = (unsigned)std::min<uint64_t>(grid_for(M, 128), (uint64_t)b.sms * 16);
    {
        KScope ks("nrl_count");
        k_nrl_count<<<qgrid, 128, 0, s>>>(b.listq.get(), b.nlistq.get(), b.ckey.get(), b.cjob.get(), b.grids.get(),
                                          b.nb9.get(), b.crun.get(), b.rfeat.get(), nrl_len.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    b.nrl_off.alloc(M + 1, s);
    uint64_t tr = 0;
    scan_u32_to_u64(nrl_len.get(), b.nrl_off.get(), M, s, &tr);
    COLO_CUDA(cudaMemcpyAsync(b.nrl_off.get() + M, &tr, 8, cudaMemcpyHostToDevice, s));
    b.nrl_total = tr;
    b.nrl_ent.alloc(tr ? tr : 1, s);
    b.run_sfx.alloc(b.Rn, s);
    b.run_qn.alloc(b.Rn, s);
    b.run_L.alloc(b.Rn, s);
    {
        KScope ks("nrl_fill");
        DevBuf<uint32_t> big, nbig;
        big.alloc(M ? M : 1, s);
        nbig.alloc(1, s);
        nbig.zero(s);
        COLO_CUDA(cudaMemsetAsync(b.run_L.get(), 0, b.Rn * 4, s));
        k_nrl_fill<<<qgrid, 128, 0, s>>>(
            b.listq.get(), b.nlistq.get(), b.ckey.get(), b.cjob.get(), b.grids.get(), b.nb9.get(), b.crun.get(),
            b.rfeat.get(), b.rstart.get(), b.rcnt.get(), b.nrl_off.get(), b.nrl_ent.get(), b.run_sfx.get(),
            b.run_qn.get(), b.run_L.get(), big.get(), nbig.get());
        COLO_LAUNCH_CHECK();
        k_nrl_fill_big<<<(unsigned)(b.sms * 8), 256, 0, s>>>(big.get(), nbig.get(), b.ckey.get(), b.cjob.get(),
                                                             b.grids.get(), b.nb9.get(), b.cstart.get(), b.crun.get(),
                                                             b.rfeat.get(), b.rstart.get(), b.cmask.get(), b.W,
                                                             b.rcnt.get(), b.nrl_off.get(), b.nrl_ent.get(),
                                                             b.run_sfx.get(), b.run_qn.get(), b.run_L.get());
        COLO_LAUNCH_CHECK();
        count_launch(2);
    }
}

}  // namespace colo
