// colo_level.cu -- level-wise instance tables and participation bitmaps.
//
// Reference semantics (generalInstanceTableSlotCounter_Kernel and
// generateInstanceTableGeneral_Kernel, Codes/DeviceProcess_Kernel.h:255-385;
// degree 2: 12-100): for a candidate (c_0..c_{k-1}) with parent table
// T(c_0..c_{k-2}), row r extends by b when b is an instance of c_{k-1} in a
// cell adjacent to r[0]'s cell with sq(r[i], b) <= R^2 for every i.  The
// candidates b of r are exactly N+_{c_{k-1}}(r[0]), a contiguous slice of the
// neighbour CSR (features ascend along each list), so the cell test and the
// r[0] distance test are already done; rows check the other k-2 members.
//
// Work decomposition: a warp owns 32 parent rows.  Their slices are
// flattened with a warp prefix sum and the warp walks the flattened items 32
// at a time, so a row with 10^4 candidates and a row with none cost the same
// per item (load-balanced expand).  Hits are compacted with one ballot per
// step; output rows are written column-major (one coalesced stream per
// column).  Participation bits are set with atomicOr on 32-bit words.
//
// The single pass (presized tables, COLO_MODE_LEARNED) writes rows in the
// same order as count + fill: a warp takes its chunk by ticket (chunks of
// warps already running come first), counts its hits, publishes the count,
// and looks back over the candidate's earlier chunks (decoupled look-back,
// every wait bounded) for the rows before it; it then writes its rows at
// their exact offsets, replaying the ballots it kept (steps beyond the kept
// ones are evaluated again).
#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

enum { MODE_COUNT = 0, MODE_FILL = 1, MODE_SINGLE = 2 };

// Participation bits: a word is read (from L2) before the atomic, so a bit
// already set costs a load, not another atomic on the same address -- in
// dense data thousands of rows hit the same few words.  A stale read only
// costs an extra (idempotent) atomic.
__device__ __forceinline__ void set_bit(uint32_t* words, uint32_t bit) {
    uint32_t* w = &words[bit >> 5];
    const uint32_t m = 1u << (bit & 31);
    if (!(__ldcg(w) & m)) atomicOr(w, m);
}

constexpr unsigned long long kChunkA = 1ull << 62;   // chunk count published
constexpr unsigned long long kChunkP = 2ull << 62;   // inclusive prefix published
constexpr unsigned long long kChunkVal = (1ull << 62) - 1;
constexpr uint32_t kChunkSpin = 1u << 22;

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Word offset of member j's participation bitmap in the level's bitmap arena.
__device__ __forceinline__ uint64_t bm_offset(const CandDesc& d, uint32_t j, const uint32_t* __restrict__ fcount) {
    uint64_t o = d.bm_base;
    for (uint32_t i = 0; i < j; ++i) o += (fcount[d.m[i]] + 31u) / 32u;
    return o;
}

// K = pattern size (2..8), or 0 for a runtime size read from the descriptor
// (members kept in global memory, slower; only reached for k > 8).  The kernel
// is latency-bound (a chain of dependent loads per warp), so the count and fill
// forms are held to fewer registers for more resident warps: pairs' count at
// eight 256-thread blocks per SM and their fill at six, size 3 at five, size 4
// at four (a few registers spill; larger sizes would spill more).  On the 20M
// workload the fills went 0.173 -> 0.158 ms and the counts 0.478 -> 0.466 ms per
// step.
template <int K, int MODE>
__global__ void __launch_bounds__(256, (MODE == MODE_COUNT && K == 2) ? 8 : (MODE == MODE_FILL && K == 2) ? 6 : (MODE != MODE_SINGLE && K == 3) ? 5 : (MODE != MODE_SINGLE && K == 4) ? 4 : 1) k_level(
    const CandDesc* __restrict__ cands, const uint64_t* __restrict__ chunk_off, uint64_t ncand,
    uint64_t nchunks, const uint64_t* __restrict__ nb_beg, const uint32_t* __restrict__ nb_cnt,
    const uint32_t* __restrict__ nb,
    const float2* __restrict__ xy, const uint32_t* __restrict__ fstart,
    const uint32_t* __restrict__ fcount, const JobGrid* __restrict__ grids,
    uint32_t* __restrict__ overflow, unsigned long long* __restrict__ items,
    unsigned long long* __restrict__ chunk_status, unsigned long long* __restrict__ ticket,
    uint32_t* __restrict__ timeout, int persistent) {
    constexpr int KR = (K == 0) ? 1 : K;   // register members kept for K > 0
    const int lane = threadIdx.x & 31;
    // one chunk per warp, or (persistent) warps that take chunk tickets until none is left; the
    // single pass always takes tickets, so its chunks run in the order warps start them
    const bool by_ticket = MODE == MODE_SINGLE || persistent;
    for (bool first = true;; first = false) {
    uint64_t ch = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (by_ticket) {
        unsigned long long tk = 0;
        if (lane == 0) tk = atomicAdd(ticket, 1ull);
        ch = __shfl_sync(0xffffffffu, tk, 0);
    } else if (!first) {
        break;
    }
    if (ch >= nchunks) break;
    // candidate of this chunk: the last c with chunk_off[c] <= ch, by a 32-way search (the
    // lanes probe 32 evenly spaced prefixes per round, so a few dependent loads instead of
    // one per halving)
    uint64_t lo = 0, hi = ncand;   // answer in [lo, hi)
    while (hi - lo > 1) {
        const uint64_t span = hi - lo;
        const uint64_t step = span <= 32 ? 1 : (span + 31) / 32;
        const uint64_t probe = lo + (uint64_t)lane * step;
        const bool le = probe < hi && chunk_off[probe] <= ch;
        const uint32_t bal = __ballot_sync(0xffffffffu, le);   // lane 0 (probe lo) is always set
        const int last = 31 - __clz(bal);
        const uint64_t nlo = lo + (uint64_t)last * step;
        hi = nlo + step < hi ? nlo + step : hi;
        lo = nlo;
    }
    const CandDesc& d = cands[lo];
    const uint32_t k = (K == 0) ? d.k : (uint32_t)K;
    const uint64_t row = (ch - chunk_off[lo]) * 32 + lane;
    const bool valid = row < d.prow;
    const uint32_t flast = d.m[k - 1];
    const uint64_t bm_last = (MODE == MODE_FILL) ? 0 : bm_offset(d, k - 1, fcount);
    const uint32_t last_start = fstart[flast];
    const uint32_t last_end = last_start + fcount[flast];
    const float R2 = grids[d.job].R2, hu = grids[d.job].R2hu;

    // row members (ids) and coordinates of members 1..k-2
    uint32_t rid[KR];
    float rx[KR], ry[KR];
#pragma unroll
    for (int i = 0; i < KR; ++i) {
        rid[i] = 0;
        rx[i] = 0.f;
        ry[i] = 0.f;
    }
    uint32_t a0 = 0;
    uint64_t slo = 0, shi = 0;
    if (valid) {
        a0 = d.parent ? d.parent[row] : fstart[d.m[0]] + (uint32_t)row;
        if (K > 0) {
            rid[0] = a0;
#pragma unroll
            for (int i = 1; i < KR - 1; ++i) {
                rid[i] = d.parent[(uint64_t)i * d.pstride + row];
                const float2 pi = xy[rid[i]];
                rx[i] = pi.x;
                ry[i] = pi.y;
            }
        }
        uint64_t o0 = nb_beg[a0], o1 = o0 + nb_cnt[a0];
        slo = lower_bound_dev(nb, o0, o1, last_start);
        shi = lower_bound_dev(nb, slo, o1, last_end);
    }
    // flatten the 32 slices
    uint32_t len = (uint32_t)(shi - slo);
    uint32_t incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const uint32_t excl = incl - len;
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (items && lane == 0 && total && MODE != MODE_FILL) atomicAdd(items, (unsigned long long)total);
    uint32_t mine = 0;               // hits of this lane's row so far
    uint64_t out0 = 0;
    if (MODE == MODE_FILL && valid) out0 = d.offs[row] - d.offs[0];   // offsets may be a slice of a longer scan
    const uint32_t lt = (1u << lane) - 1u;
    bool ovf = false;
    const uint64_t chunk_row0 = (ch - chunk_off[lo]) * 32;

    // item t0 + lane: its owner row (lane j), the row's first item and slice, and whether b
    // extends the row (the other k-2 members within R)
    struct Item {
        int j;
        uint32_t ex_j, in_j, b;
        bool active;
    };
    auto locate = [&](uint32_t t0) {
        Item it;
        const uint32_t item = t0 + lane;
        it.active = item < total;
        int j = 0;
#pragma unroll
        for (int bstep = 16; bstep > 0; bstep >>= 1) {
            uint32_t ev = __shfl_sync(0xffffffffu, excl, j + bstep);
            if (ev <= item) j += bstep;
        }
        it.j = j;
        it.ex_j = __shfl_sync(0xffffffffu, excl, j);
        it.in_j = __shfl_sync(0xffffffffu, incl, j);
        const uint64_t lo_j = __shfl_sync(0xffffffffu, slo, j);
        it.b = it.active ? nb[lo_j + (item - it.ex_j)] : 0u;
        return it;
    };
    auto extends = [&](const Item& it) {
        bool ok = it.active;
        if (K == 0) {
            if (it.active && k > 2) {
                const float2 pb = xy[it.b];
                const uint64_t prow_j = chunk_row0 + (uint64_t)it.j;
                for (uint32_t i = 1; i + 1 < k && ok; ++i) {
                    uint32_t ri = d.parent[(uint64_t)i * d.pstride + prow_j];
                    const float2 pr = xy[ri];
                    ok = ref_within(pr.x, pr.y, pb.x, pb.y, R2, hu);
                }
            }
        } else if (K > 2) {
            float xb = 0.f, yb = 0.f;
            if (it.active) {
                const float2 pb = xy[it.b];
                xb = pb.x;
                yb = pb.y;
            }
#pragma unroll
            for (int i = 1; i < KR - 1; ++i) {
                float xi = __shfl_sync(0xffffffffu, rx[i], it.j);
                float yi = __shfl_sync(0xffffffffu, ry[i], it.j);
                ok = ok && ref_within(xi, yi, xb, yb, R2, hu);
            }
        }
        return ok;
    };
    // lanes of step t0 that belong to my own row
    auto own_mask = [&](uint32_t t0) {
        int r0 = (int)excl - (int)t0, r1 = (int)incl - (int)t0;
        r0 = r0 < 0 ? 0 : r0;
        r1 = r1 > 32 ? 32 : r1;
        return (r1 > r0) ? ((r1 - r0 == 32) ? 0xffffffffu : (((1u << (r1 - r0)) - 1u) << r0)) : 0u;
    };
    // writes the hits of one step: rows of owner j go to out_j + (j's rows written so far)
    auto write_step = [&](const Item& it, bool ok, uint32_t bal, uint32_t t0, uint64_t col_stride, bool capped) {
        const uint32_t before_j = __shfl_sync(0xffffffffu, mine, it.j);
        const uint64_t out_j = __shfl_sync(0xffffffffu, out0, it.j);
        int q0 = (int)it.ex_j - (int)t0, q1 = (int)it.in_j - (int)t0;
        q0 = q0 < 0 ? 0 : q0;
        q1 = q1 > 32 ? 32 : q1;
        const uint32_t jmask = (q1 > q0) ? ((q1 - q0 == 32) ? 0xffffffffu : (((1u << (q1 - q0)) - 1u) << q0)) : 0u;
        const uint64_t pos = out_j + before_j + __popc(bal & jmask & lt);
        const bool room = !capped || pos < d.out_cap;
        if (ok && !room) ovf = true;
        const bool wr = ok && room;
        if (K > 0) {
#pragma unroll
            for (int i = 0; i < KR - 1; ++i) {
                uint32_t v = __shfl_sync(0xffffffffu, rid[i], it.j);
                if (wr) d.out[(uint64_t)i * col_stride + pos] = v;
            }
        } else if (wr) {
            const uint64_t prow_j = chunk_row0 + (uint64_t)it.j;
            d.out[pos] = d.parent ? d.parent[prow_j] : fstart[d.m[0]] + (uint32_t)prow_j;
            for (uint32_t i = 1; i + 1 < k; ++i)
                d.out[(uint64_t)i * col_stride + pos] = d.parent[(uint64_t)i * d.pstride + prow_j];
        }
        if (wr) d.out[(uint64_t)(k - 1) * col_stride + pos] = it.b;
    };

    uint32_t bal_lo = 0, bal_hi = 0;   // single pass: ballot of step s kept in lane s % 32 (s < 64)
    for (uint32_t t0 = 0; t0 < total; t0 += 32) {
        const Item it = locate(t0);
        const bool ok = extends(it);
        const uint32_t bal = __ballot_sync(0xffffffffu, ok);
        const uint32_t my_hits = __popc(bal & own_mask(t0));
        if (MODE == MODE_COUNT || MODE == MODE_SINGLE) {
            if (ok) set_bit(d.bitmap + bm_last, it.b - last_start);
        }
        if (MODE == MODE_SINGLE) {
            const uint32_t step = t0 >> 5;
            if (step < 32 && lane == (int)step) bal_lo = bal;
            else if (step >= 32 && step < 64 && lane == (int)(step - 32)) bal_hi = bal;
        }
        if (MODE == MODE_FILL) write_step(it, ok, bal, t0, d.out_rows, false);
        mine += my_hits;
    }
    if (MODE == MODE_SINGLE) {
        // the chunk's rows, then the rows of the candidate's earlier chunks: the warp reads 32
        // predecessors' words at once, back to the nearest published prefix
        const uint32_t wsum = __reduce_add_sync(0xffffffffu, mine);
        const uint64_t first = chunk_off[lo];
        unsigned long long prefix = 0;
        if (lane == 0) *(volatile unsigned long long*)(chunk_status + ch) = (first == ch ? kChunkP : kChunkA) | wsum;
        if (first != ch) {
            uint32_t spins = 0;
            int64_t base = (int64_t)ch - 1;
            while (true) {
                const int64_t t = base - lane;
                // words before the candidate's first chunk read as an empty published prefix
                const unsigned long long v =
                    t >= (int64_t)first ? *(volatile const unsigned long long*)(chunk_status + t) : kChunkP;
                const unsigned long long flag = v & ~kChunkVal;
                const uint32_t pm = __ballot_sync(0xffffffffu, flag == kChunkP);
                const uint32_t zm = __ballot_sync(0xffffffffu, flag == 0);
                const int fp = pm ? __ffs(pm) - 1 : 32;                 // nearest published prefix
                const uint32_t upto = fp == 32 ? 0xffffffffu : ((2u << fp) - 1u);
                if (zm & upto) {                                         // a chunk before it not counted yet
                    if (++spins > kChunkSpin) {                          // give up: report it, write with what we have
                        if (lane == 0) atomicOr(timeout, 1u);
                        break;
                    }
                    __nanosleep(64);
                    continue;
                }
                prefix += warp_sum_u64(((upto >> lane) & 1u) ? (v & kChunkVal) : 0ull);
                if (fp < 32) break;
                base -= 32;
            }
            if (lane == 0) *(volatile unsigned long long*)(chunk_status + ch) = kChunkP | (prefix + wsum);
        }
        // my row's first output row: the chunk's prefix plus the rows of the chunk's earlier rows
        uint32_t rincl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, rincl, o);
            if (lane >= o) rincl += t;
        }
        const uint32_t slots = mine;
        out0 = prefix + (rincl - mine);
        mine = 0;
        for (uint32_t t0 = 0; t0 < total; t0 += 32) {
            const Item it = locate(t0);
            const uint32_t step = t0 >> 5;
            bool ok;
            if (step < 64) {
                const uint32_t kept = __shfl_sync(0xffffffffu, step < 32 ? bal_lo : bal_hi, (int)(step & 31));
                ok = it.active && ((kept >> lane) & 1u);
            } else {
                ok = extends(it);
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, ok);
            write_step(it, ok, bal, t0, d.out_cap, true);
            mine += __popc(bal & own_mask(t0));
        }
        mine = slots;
    }
    if (MODE == MODE_SINGLE) {
        if (__any_sync(0xffffffffu, ovf) && lane == 0) atomicOr(&overflow[lo], 1u);
    }
    if (MODE == MODE_COUNT || MODE == MODE_SINGLE) {
        const uint32_t wsum = __reduce_add_sync(0xffffffffu, mine);
        if (lane == 0 && wsum) atomicAdd(d.rows, (unsigned long long)wsum);
    }
    if ((MODE == MODE_COUNT || MODE == MODE_SINGLE) && valid) {
        d.slots[row] = mine;
        if (mine) {
            set_bit(d.bitmap + d.bm_base, a0 - fstart[d.m[0]]);
            if (K > 0) {
                uint64_t o = d.bm_base + (fcount[d.m[0]] + 31u) / 32u;
#pragma unroll
                for (int q = 1; q < KR - 1; ++q) {
                    set_bit(d.bitmap + o, rid[q] - fstart[d.m[q]]);
                    o += (fcount[d.m[q]] + 31u) / 32u;
                }
            } else {
                for (uint32_t i = 1; i + 1 < k; ++i) {
                    uint32_t ri = d.parent[(uint64_t)i * d.pstride + row];
                    set_bit(d.bitmap + bm_offset(d, i, fcount), ri - fstart[d.m[i]]);
                }
            }
        }
    }
    }   // chunks of this warp
}

// Participation statistics: per (candidate, member) [A, last, first, full]
// where A counts set bits in [0, n-2] (the window getParticipationIndex sums,
// Codes/DeviceProcess.cu:108-132).  A block takes one (candidate, member)
// pair (blockIdx.x) and one span of kPiSpan bitmap words (blockIdx.y; spans
// past the member's bitmap leave at once) and adds its counts to the zeroed
// statistics; the spans holding bit 0 and bit n-1 also record first and last.
constexpr uint32_t kPiSpan = 16384;

__global__ void __launch_bounds__(256) k_level_pi(const CandDesc* __restrict__ cands, uint32_t k,
                                                  const uint32_t* __restrict__ fcount, uint64_t* __restrict__ stats) {
    const uint64_t c = blockIdx.x / k;
    const uint32_t j = blockIdx.x - (uint32_t)(c * k);
    const CandDesc& d = cands[c];
    const uint32_t n = fcount[d.m[j]];
    const uint32_t nw = (n + 31) / 32;
    const uint32_t w0 = blockIdx.y * kPiSpan;
    if (w0 >= nw) return;
    const uint32_t w1 = w0 + kPiSpan < nw ? w0 + kPiSpan : nw;
    const uint32_t* w = d.bitmap + bm_offset(d, j, fcount);
    const uint32_t lim = n - 1;   // bits in the window [0, n-2]
    unsigned long long cntA = 0, cntFull = 0;
    for (uint32_t i = w0 + threadIdx.x; i < w1; i += blockDim.x) {
        const uint32_t v = w[i];
        cntFull += __popc(v);
        const uint32_t wb = i * 32;
        const uint32_t mask = wb + 32 <= lim ? 0xffffffffu : (wb >= lim ? 0u : (1u << (lim - wb)) - 1u);
        cntA += __popc(v & mask);
    }
    __shared__ unsigned long long red[8];
    for (int o = 16; o > 0; o >>= 1) {
        cntA += __shfl_down_sync(0xffffffffu, cntA, o);
        cntFull += __shfl_down_sync(0xffffffffu, cntFull, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = cntA | (cntFull << 32);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long A = 0, Fu = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
            A += red[q] & 0xffffffffull;
            Fu += red[q] >> 32;
        }
        uint64_t* o = stats + (c * k + j) * 4;
        if (A) atomicAdd(reinterpret_cast<unsigned long long*>(o + 0), A);
        if (Fu) atomicAdd(reinterpret_cast<unsigned long long*>(o + 3), Fu);
        if (w0 == 0) o[2] = w[0] & 1u;
        if ((lim >> 5) >= w0 && (lim >> 5) < w1) o[1] = (w[lim >> 5] >> (lim & 31)) & 1u;
    }
}

template <int MODE>
void launch_level(Batch& b, const LevelWork& w, uint32_t k, uint32_t* ovf) {
    if (w.nchunks == 0) return;
    KScope ks(MODE == MODE_COUNT ? "level_count" : MODE == MODE_FILL ? "level_fill" : "level_single");
    const unsigned block = (b.level_block == 64 || b.level_block == 128) ? (unsigned)b.level_block : 256u;
    uint64_t threads = w.nchunks * 32;
    unsigned grid = (unsigned)((threads + block - 1) / block);
    // persistent queue: as many blocks as are resident at once (64 registers a thread: 32 warps
    // an SM), their warps taking chunk tickets (the ticket word follows the chunk words)
    const int persistent = (b.level_queue && MODE != MODE_SINGLE && w.ticket) ? 1 : 0;
    if (persistent) {
        const uint64_t cap = (uint64_t)b.sms * (32u * 32u / block);
        if (grid > cap) grid = (unsigned)cap;
    }
#define COLO_LVL(KK)                                                                              \
    k_level<KK, MODE><<<grid, block, 0, b.s>>>(w.cands, w.chunk_off, w.ncand, w.nchunks, b.nb_beg.get(), b.nb_cnt.get(), \
                                            b.nb.get(), b.xy.get(), b.fstart.get(), b.fcount.get(),  \
                                            b.grids.get(), ovf, w.items, w.chunk_status, w.ticket,    \
                                            &b.flags.get()->timeout, persistent)
    switch (k) {
        case 2: COLO_LVL(2); break;
        case 3: COLO_LVL(3); break;
        case 4: COLO_LVL(4); break;
        case 5: COLO_LVL(5); break;
        case 6: COLO_LVL(6); break;
        case 7: COLO_LVL(7); break;
        case 8: COLO_LVL(8); break;
        default: COLO_LVL(0); break;
    }
#undef COLO_LVL
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace

void level_count(Batch& b, const LevelWork& w, uint32_t k) { launch_level<MODE_COUNT>(b, w, k, nullptr); }
void level_fill(Batch& b, const LevelWork& w, uint32_t k) { launch_level<MODE_FILL>(b, w, k, nullptr); }
void level_single(Batch& b, const LevelWork& w, uint32_t k, uint32_t* d_overflow) {
    launch_level<MODE_SINGLE>(b, w, k, d_overflow);
}

void level_pi(Batch& b, const CandDesc* d_cands, uint64_t ncand, uint32_t k, uint64_t* d_stats) {
    if (ncand == 0) return;
    if (ncand * k >= (1ull << 31)) throw StatusError{COLO_ERR_CAPACITY, "too many candidates in one level"};
    KScope ks("level_pi");
    // spans per member: enough for the largest feature of the batch
    uint32_t fmax = 0;
    for (uint32_t f = 0; f < b.F; ++f) fmax = std::max(fmax, b.h_fcount[f]);
    const uint32_t spans = std::max<uint32_t>(1, ((fmax + 31) / 32 + kPiSpan - 1) / kPiSpan);
    k_level_pi<<<dim3((unsigned)(ncand * k), spans), 256, 0, b.s>>>(d_cands, k, b.fcount.get(), d_stats);
    COLO_LAUNCH_CHECK();
    count_launch();
}

}  // namespace colo
