// colo_bucket.cu -- grid bucketing: a stable radix sort of points by cell key
// into a cell CSR with (cell, feature) runs, per-cell feature masks and the
// geometric 3x3 occupied-neighbour table; then the per-cell neighbourhood
// run/point lists (NRL / NPL) that the join streams.
//
// Replaces CountCellFeatures (Codes/DeviceProcess.cu:312-369) and
// kernel_CountCellFeatures (Codes/DeviceProcess_Kernel.h:629-647): instead of
// dense totalCells x F count/start arrays, only occupied cells and runs are
// stored, so grids of 10^10 cells cost nothing.
#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

__global__ void k_cell_keys(uint64_t n, const float* __restrict__ x, const float* __restrict__ y,
                            const uint32_t* __restrict__ feat, const uint32_t* __restrict__ fjob,
                            const JobGrid* __restrict__ grids, uint64_t* __restrict__ keys,
                            uint32_t* __restrict__ vals, DevFlags* flags) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const JobGrid g = grids[fjob[feat[i]]];
    uint64_t c = ref_cell(g, x[i], y[i]);
    if (c >= g.total) {
        atomicAdd(&flags->out_of_grid, 1u);
        c = g.total - 1;
    }
    keys[i] = g.key_base + c;
    vals[i] = (uint32_t)i;
}

__global__ void k_gather_sorted(uint64_t n, const uint32_t* __restrict__ sid,
                                const float* __restrict__ x, const float* __restrict__ y,
                                const uint32_t* __restrict__ feat, float* __restrict__ sx,
                                float* __restrict__ sy, uint32_t* __restrict__ sfeat) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t id = sid[p];
    sx[p] = x[id];
    sy[p] = y[id];
    sfeat[p] = feat[id];
}

__global__ void k_heads(uint64_t n, const uint64_t* __restrict__ keys,
                        const uint32_t* __restrict__ sfeat, uint32_t* __restrict__ cell_head,
                        uint32_t* __restrict__ run_head) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    bool ch = (p == 0) || keys[p] != keys[p - 1];
    bool rh = ch || sfeat[p] != sfeat[p - 1];
    cell_head[p] = ch;
    run_head[p] = rh;
}

__global__ void k_compact(uint64_t n, const uint64_t* __restrict__ keys,
                          const uint32_t* __restrict__ sfeat, const uint32_t* __restrict__ fjob,
                          const uint32_t* __restrict__ cell_head, const uint32_t* __restrict__ run_head,
                          const uint32_t* __restrict__ cell_ex, const uint32_t* __restrict__ run_ex,
                          uint64_t* __restrict__ ckey, uint32_t* __restrict__ cstart,
                          uint32_t* __restrict__ crun, uint32_t* __restrict__ cjob,
                          uint32_t* __restrict__ rfeat, uint32_t* __restrict__ rstart,
                          uint32_t* __restrict__ rcell, uint32_t* __restrict__ scell) {
    uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t ch = cell_head[p], rh = run_head[p];
    uint32_t c = cell_ex[p] + ch - 1;
    scell[p] = c;
    if (ch) {
        ckey[c] = keys[p];
        cstart[c] = (uint32_t)p;
        crun[c] = run_ex[p];
        cjob[c] = fjob[sfeat[p]];
    }
    if (rh) {
        uint32_t r = run_ex[p];
        rfeat[r] = sfeat[p];
        rstart[r] = (uint32_t)p;
        rcell[r] = c;
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

__global__ void k_cell_masks(uint64_t Rn, const uint32_t* __restrict__ rfeat,
                             const uint32_t* __restrict__ rcell, const uint32_t* __restrict__ cjob,
                             const JobGrid* __restrict__ grids, uint32_t W,
                             uint32_t* __restrict__ cmask) {
    uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= Rn) return;
    uint32_t c = rcell[r];
    uint32_t lf = rfeat[r] - grids[cjob[c]].f0;
    atomicOr(&cmask[(uint64_t)c * W + (lf >> 5)], 1u << (lf & 31));
}

// nb9[c*9 + (dy+1)*3 + (dx+1)] = occupied index of the geometric neighbour
// (cx+dx, cy+dy) inside the job's grid, or -1.
__global__ void k_nb9(uint64_t M, const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
                      const JobGrid* __restrict__ grids, int32_t* __restrict__ nb9) {
    uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M) return;
    const JobGrid g = grids[cjob[c]];
    uint64_t local = ckey[c] - g.key_base;
    int64_t cx = (int64_t)(local % g.gx), cy = (int64_t)(local / g.gx);
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            int32_t v = -1;
            int64_t nx = cx + dx, ny = cy + dy;
            if (dx == 0 && dy == 0) {
                v = (int32_t)c;
            } else if (nx >= 0 && ny >= 0 && nx < (int64_t)g.gx && ny < (int64_t)g.gy) {
                uint64_t key = g.key_base + (uint64_t)ny * g.gx + (uint64_t)nx;
                uint64_t lo = 0, hi = M;
                // neighbours lie within the job's cells; search the whole list
                lo = lower_bound_dev(ckey, lo, hi, key);
                if (lo < M && ckey[lo] == key) v = (int32_t)lo;
            }
            nb9[c * 9 + (dy + 1) * 3 + (dx + 1)] = v;
        }
}

__global__ void k_frun_count(uint64_t Rn, const uint32_t* __restrict__ rfeat, uint32_t* __restrict__ cnt) {
    uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < Rn) atomicAdd(&cnt[rfeat[r]], 1u);
}

__global__ void k_frun_fill(uint64_t Rn, const uint32_t* __restrict__ rfeat,
                            const uint32_t* __restrict__ off, uint32_t* __restrict__ cursor,
                            uint32_t* __restrict__ frun) {
    uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= Rn) return;
    uint32_t f = rfeat[r];
    frun[off[f] + atomicAdd(&cursor[f], 1u)] = (uint32_t)r;
}

// ---------------------------------------------------------------------------
// Neighbourhood lists.  For cell c the adjacent cells A(c) (the reference's
// stencil, in ascending cell order) contribute their runs; NRL(c) lists them
// ordered by (feature, cell) and NPL(c) lists their points in that order.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int adjacent_cells(uint64_t c, const uint64_t* ckey, const uint32_t* cjob,
                                              const JobGrid* grids, const int32_t* nb9,
                                              int32_t* out) {
    const JobGrid g = grids[cjob[c]];
    uint64_t local = ckey[c] - g.key_base;
    uint32_t cx = (uint32_t)(local % g.gx);
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

__global__ void k_nl_count(uint64_t M, const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
                           const JobGrid* __restrict__ grids, const int32_t* __restrict__ nb9,
                           const uint32_t* __restrict__ cstart, const uint32_t* __restrict__ crun,
                           uint32_t* __restrict__ nrl_len, uint32_t* __restrict__ npl_len) {
    uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M) return;
    int32_t adj[9];
    int na = adjacent_cells(c, ckey, cjob, grids, nb9, adj);
    uint32_t nr = 0, np = 0;
    for (int s = 0; s < na; ++s) {
        nr += crun[adj[s] + 1] - crun[adj[s]];
        np += cstart[adj[s] + 1] - cstart[adj[s]];
    }
    nrl_len[c] = nr;
    npl_len[c] = np;
}

// One warp per cell.  For a run of feature f in adjacent slot s, its NRL
// position is sum over slots of (#runs with feature < f) plus the number of
// earlier slots that also hold f; its NPL position is the same with points.
__global__ void k_nl_fill(uint64_t M, const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cjob,
                          const JobGrid* __restrict__ grids, const int32_t* __restrict__ nb9,
                          const uint32_t* __restrict__ cstart, const uint32_t* __restrict__ crun,
                          const uint32_t* __restrict__ rfeat, const uint32_t* __restrict__ rstart,
                          const uint32_t* __restrict__ rcnt, const uint32_t* __restrict__ sid,
                          const float* __restrict__ sx, const float* __restrict__ sy,
                          const uint64_t* __restrict__ nrl_off, const uint64_t* __restrict__ npl_off,
                          uint32_t* __restrict__ nrl_feat, uint64_t* __restrict__ nrl_pos,
                          uint32_t* __restrict__ npl_id, float* __restrict__ npl_x,
                          float* __restrict__ npl_y) {
    const int lane = threadIdx.x & 31;
    uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= M) return;
    int32_t adj[9];
    int na = adjacent_cells(c, ckey, cjob, grids, nb9, adj);
    uint64_t rbase = nrl_off[c], pbase = npl_off[c];
    for (int s = 0; s < na; ++s) {
        uint32_t r0 = crun[adj[s]], r1 = crun[adj[s] + 1];
        for (uint32_t r = r0; r < r1; ++r) {
            uint32_t f = rfeat[r];
            uint64_t rpos = 0, ppos = 0;
            for (int t = 0; t < na; ++t) {
                uint32_t q0 = crun[adj[t]], q1 = crun[adj[t] + 1];
                uint32_t lb = (uint32_t)lower_bound_dev(rfeat, (uint64_t)q0, (uint64_t)q1, f);
                rpos += lb - q0;
                uint32_t pts_before = (lb < q1 ? rstart[lb] : cstart[adj[t] + 1]) - cstart[adj[t]];
                ppos += pts_before;
                if (t < s && lb < q1 && rfeat[lb] == f) {
                    rpos += 1;
                    ppos += rcnt[lb];
                }
            }
            if (lane == 0) {
                nrl_feat[rbase + rpos] = f;
                nrl_pos[rbase + rpos] = pbase + ppos;
            }
            uint32_t st = rstart[r], ct = rcnt[r];
            for (uint32_t t = lane; t < ct; t += 32) {
                uint64_t q = pbase + ppos + t;
                npl_id[q] = sid[st + t];
                npl_x[q] = sx[st + t];
                npl_y[q] = sy[st + t];
            }
        }
    }
}

inline unsigned grid_for(uint64_t n, int threads) {
    uint64_t g = (n + threads - 1) / threads;
    return (unsigned)(g == 0 ? 1 : g);
}

}  // namespace

void bucket_points(Batch& b) {
    cudaStream_t s = b.s;
    const uint64_t n = b.N;
    DevBuf<uint64_t> keys;
    keys.alloc(n, s);
    b.sid.alloc(n, s);
    {
    KScope ks("cell_keys");
    k_cell_keys<<<grid_for(n, 256), 256, 0, s>>>(n, b.x, b.y, b.feat, b.fjob.get(), b.grids.get(),
                                                  keys.get(), b.sid.get(), b.flags.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    }
    radix_sort_u64_u32(keys.get(), b.sid.get(), n, (int)b.key_bits, s);

    b.sx.alloc(n, s);
    b.sy.alloc(n, s);
    b.sfeat.alloc(n, s);
    k_gather_sorted<<<grid_for(n, 256), 256, 0, s>>>(n, b.sid.get(), b.x, b.y, b.feat, b.sx.get(),
                                                     b.sy.get(), b.sfeat.get());
    COLO_LAUNCH_CHECK();
    count_launch();

    DevBuf<uint32_t> ch, rh, cex, rex;
    ch.alloc(n, s);
    rh.alloc(n, s);
    cex.alloc(n, s);
    rex.alloc(n, s);
    k_heads<<<grid_for(n, 256), 256, 0, s>>>(n, keys.get(), b.sfeat.get(), ch.get(), rh.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    uint32_t M = 0, Rn = 0;
    scan_u32_to_u32(ch.get(), cex.get(), n, s, &M);
    scan_u32_to_u32(rh.get(), rex.get(), n, s, &Rn);
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
    b.scell.alloc(n, s);
    k_compact<<<grid_for(n, 256), 256, 0, s>>>(n, keys.get(), b.sfeat.get(), b.fjob.get(), ch.get(),
                                                rh.get(), cex.get(), rex.get(), b.ckey.get(),
                                                b.cstart.get(), b.crun.get(), b.cjob.get(),
                                                b.rfeat.get(), b.rstart.get(), b.rcell.get(),
                                                b.scell.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    k_run_tail<<<grid_for(Rn, 256), 256, 0, s>>>(Rn, M, n, b.rstart.get(), b.rcnt.get(), b.cstart.get(),
                                                  b.crun.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    keys.release();
    ch.release();
    rh.release();
    cex.release();
    rex.release();

    b.cmask.alloc((uint64_t)M * b.W, s);
    b.cmask.zero(s);
    k_cell_masks<<<grid_for(Rn, 256), 256, 0, s>>>(Rn, b.rfeat.get(), b.rcell.get(), b.cjob.get(),
                                                    b.grids.get(), b.W, b.cmask.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    b.nb9.alloc((uint64_t)M * 9, s);
    k_nb9<<<grid_for(M, 128), 128, 0, s>>>(M, b.ckey.get(), b.cjob.get(), b.grids.get(), b.nb9.get());
    COLO_LAUNCH_CHECK();
    count_launch();

    // feature-major run index
    DevBuf<uint32_t> fcnt, cursor;
    fcnt.alloc(b.F, s);
    fcnt.zero(s);
    cursor.alloc(b.F, s);
    cursor.zero(s);
    b.frun_off.alloc(b.F + 1, s);
    b.frun.alloc(Rn, s);
    k_frun_count<<<grid_for(Rn, 256), 256, 0, s>>>(Rn, b.rfeat.get(), fcnt.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    uint32_t tot = 0;
    scan_u32_to_u32(fcnt.get(), b.frun_off.get(), b.F, s, &tot);
    COLO_CUDA(cudaMemcpyAsync(b.frun_off.get() + b.F, &tot, 4, cudaMemcpyHostToDevice, s));
    k_frun_fill<<<grid_for(Rn, 256), 256, 0, s>>>(Rn, b.rfeat.get(), b.frun_off.get(), cursor.get(),
                                                   b.frun.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    b.h_frun_off.resize(b.F + 1);
    COLO_CUDA(cudaMemcpyAsync(b.h_frun_off.data(), b.frun_off.get(), (b.F + 1) * 4,
                              cudaMemcpyDeviceToHost, s));
    DevFlags hf;
    COLO_CUDA(cudaMemcpyAsync(&hf, b.flags.get(), sizeof(hf), cudaMemcpyDeviceToHost, s));
    COLO_CUDA(cudaStreamSynchronize(s));
    if (hf.out_of_grid)
        throw StatusError{COLO_ERR_INPUT, std::to_string(hf.out_of_grid) +
                                              " point(s) fall outside the grid derived from the bounds line"};
}

void build_neighborhoods(Batch& b) {
    cudaStream_t s = b.s;
    const uint64_t M = b.M;
    DevBuf<uint32_t> nrl_len, npl_len;
    nrl_len.alloc(M, s);
    npl_len.alloc(M, s);
    k_nl_count<<<grid_for(M, 128), 128, 0, s>>>(M, b.ckey.get(), b.cjob.get(), b.grids.get(),
                                                 b.nb9.get(), b.cstart.get(), b.crun.get(),
                                                 nrl_len.get(), npl_len.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    b.nrl_off.alloc(M + 1, s);
    b.npl_off.alloc(M + 1, s);
    uint64_t tr = 0, tp = 0;
    scan_u32_to_u64(nrl_len.get(), b.nrl_off.get(), M, s, &tr);
    scan_u32_to_u64(npl_len.get(), b.npl_off.get(), M, s, &tp);
    COLO_CUDA(cudaMemcpyAsync(b.nrl_off.get() + M, &tr, 8, cudaMemcpyHostToDevice, s));
    COLO_CUDA(cudaMemcpyAsync(b.npl_off.get() + M, &tp, 8, cudaMemcpyHostToDevice, s));
    b.nrl_total = tr;
    b.npl_total = tp;
    b.nrl_feat.alloc(tr, s);
    b.nrl_pos.alloc(tr, s);
    b.npl_id.alloc(tp, s);
    b.npl_x.alloc(tp, s);
    b.npl_y.alloc(tp, s);
    KScope ks("npl_fill");
    k_nl_fill<<<grid_for(M * 32, 256), 256, 0, s>>>(
        M, b.ckey.get(), b.cjob.get(), b.grids.get(), b.nb9.get(), b.cstart.get(), b.crun.get(),
        b.rfeat.get(), b.rstart.get(), b.rcnt.get(), b.sid.get(), b.sx.get(), b.sy.get(),
        b.nrl_off.get(), b.npl_off.get(), b.nrl_feat.get(), b.nrl_pos.get(), b.npl_id.get(),
        b.npl_x.get(), b.npl_y.get());
    COLO_LAUNCH_CHECK();
    count_launch();
    // the tiny host copies above must complete before the temporaries go
    COLO_CUDA(cudaStreamSynchronize(s));
}

}  // namespace colo
