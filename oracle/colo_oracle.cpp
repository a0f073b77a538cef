/*
 * colo_oracle.cpp -- CPU restatement of the reference's colocation-mining
 * semantics.  TEST INFRASTRUCTURE ONLY (see colo_oracle.h): used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs, never by the product.
 *
 * Parity status of this oracle
 *  - Float squared-distance form: pinned against the reference's own device
 *    expression evaluated on a GB300 (tests/test_gpu_sqdist.py).
 *  - Integer/host semantics (parse, grid, cells, neighbour-cell rule, filter,
 *    tables, bitmap windows, PI, Apriori): pinned against golden vectors that
 *    the reference's own sources produced when compiled and run on the CPU
 *    (oracle/ref_emu/, fixtures in tests/golden/).
 *
 * All citations are paths inside the reference project.
 */
#include "colo_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#ifdef _OPENMP
#include <parallel/algorithm>
#endif
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* ------------------------------------------------------------------------ */
/* Float arithmetic                                                          */
/* ------------------------------------------------------------------------ */

/* Codes/Utility_Inline.h:25-33: squareDistance = pow(x2-x1,2) + pow(y2-y1,2)
 * with float differences and the result stored in a float.  Measured on a
 * GB300 (see tests/test_gpu_sqdist.py), the device value is the correctly
 * rounded float of the exact sum S = dx^2 + dy^2, except when S lies on (or
 * within a few double ulps of) a rounding midpoint between two floats, where
 * either neighbour can come out -- the behaviour of pow evaluated in double
 * and rounded to float once.  CUDA's pow itself is not restated here: the
 * host computes S exactly (double-double) and calls a comparison "ambiguous"
 * when such a midpoint could flip it; ambiguous pairs are resolved by a
 * device evaluation of the reference expression supplied by the caller. */
struct SqDecision {
    bool le;          /* sq <= R2 (for ambiguous pairs: the round-to-even guess) */
    bool ambiguous;
};

struct ExactSq {
    float rn;         /* correctly rounded float of S (ties to even) */
    float other;      /* the other neighbour when S is near a midpoint */
    bool near_mid;
};

inline ExactSq exact_sq(float x1, float y1, float x2, float y2) {
    float dx = x2 - x1;
    float dy = y2 - y1;
    double a = (double)dx * (double)dx;          /* exact */
    double b = (double)dy * (double)dy;          /* exact */
    double hi = a + b;                           /* TwoSum: S = hi + lo exactly */
    double bb = hi - a;
    double lo = (a - (hi - bb)) + (b - bb);
    ExactSq r;
    r.near_mid = false;
    r.rn = (float)hi;
    r.other = r.rn;
    if (!(hi < 3.0e38)) return r;                /* overflow range: never near R^2 */
    /* neighbours of S and their midpoint (exact in double) */
    float l = (double)r.rn <= hi ? r.rn : std::nextafter(r.rn, -INFINITY);
    float h = std::nextafter(l, INFINITY);
    if ((double)l == hi && lo == 0.0) return r;  /* S is a float */
    double mid = 0.5 * ((double)l + (double)h);
    double d = hi - mid;                         /* exact (Sterbenz) */
    /* sign of S - mid = d + lo */
    bool above = d > 0 || (d == 0 && lo > 0);
    bool below = d < 0 || (d == 0 && lo < 0);
    if (above) {
        r.rn = h;
    } else if (below) {
        r.rn = l;
    } else {                                     /* exact midpoint: ties to even */
        uint32_t lbits;
        std::memcpy(&lbits, &l, 4);
        r.rn = (lbits & 1u) ? h : l;
    }
    double gap = std::fabs(d + lo);
    if (gap <= std::ldexp(hi, -44)) {            /* within ~256 double ulps of the midpoint */
        r.near_mid = true;
        r.other = (r.rn == l) ? h : l;
    }
    return r;
}

inline SqDecision sq_decide(float x1, float y1, float x2, float y2, float R2) {
    ExactSq e = exact_sq(x1, y1, x2, y2);
    SqDecision out;
    out.le = e.rn <= R2;
    out.ambiguous = e.near_mid && ((e.other <= R2) != out.le);
    return out;
}

/* Squared distance value away from rounding midpoints (used by oracle_sqdist). */
inline float sqdist(float x1, float y1, float x2, float y2) { return exact_sq(x1, y1, x2, y2).rn; }

/* Device float -> u32 conversion (cvt.rzi.u32.f32 clamps to the range). */
inline uint32_t f2u_sat(float f) {
    if (!(f > 0.0f)) return 0u;                 /* negative, zero, NaN */
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

/* ------------------------------------------------------------------------ */
/* Grid                                                                      */
/* ------------------------------------------------------------------------ */

/* colocationFinder.cpp:102-115 (setGrid). */
int make_grid(float minX, float minY, float maxX, float maxY, float R, oracle_grid* g) {
    std::memset(g, 0, sizeof(*g));
    if (!(R > 0.0f) || !std::isfinite(R)) return 1;
    g->min_x = minX;
    g->min_y = minY;
    g->max_x = maxX;
    g->max_y_ext = maxY + R;              /* computeZone.maxBound.y = maxY + R */
    g->cell_width = R;
    float gsx = (g->max_x - g->min_x) / g->cell_width;
    float gsy = (g->max_y_ext - g->min_y) / g->cell_width;
    if (!std::isfinite(gsx) || !std::isfinite(gsy)) return 1;
    float cx = std::ceil(gsx), cy = std::ceil(gsy);
    if (!(cx >= 1.0f) || !(cy >= 1.0f)) return 1;
    if (cx >= 4294967296.0f || cy >= 4294967296.0f) return 1;
    g->gx = (uint32_t)cx;
    g->gy = (uint32_t)cy;
    g->total_cells = (uint64_t)g->gx * (uint64_t)g->gy;
    /* The reference keeps cell ids in u32 and neighbour ids in i32
     * (Utility_Inline.h:35-37).  Both are exact while total + gx < 2^31. */
    g->compat32 = (g->total_cells + g->gx) < (1ull << 31) ? 1 : 0;
    return 0;
}

/* Codes/DeviceProcess_Kernel.h:615-625 (getCellID), u32 arithmetic. */
inline uint64_t cell_of(const oracle_grid& g, float x, float y) {
    float rx = x - g.min_x;
    float ry = y - g.min_y;
    rx /= g.cell_width;
    ry /= g.cell_width;
    uint64_t i = f2u_sat(rx), j = f2u_sat(ry);
    uint64_t c = (uint64_t)g.gx * j + i;
    if (g.compat32) c = (uint32_t)c;      /* const Integer CellID = gx*j + i */
    return c;
}

/* Codes/Utility_Inline.h:35-53 (getNeighborCellID) plus the caller's range
 * check (e.g. DeviceProcess_Kernel.h:28-32).  Returns -1 for "skip". */
inline int64_t neighbor_cell32(uint32_t x, uint32_t y, uint32_t tid, uint32_t gx,
                               uint64_t total) {
    int32_t ncid = (int32_t)(y * gx + x);
    int32_t r;
    if (tid % gx == 0) {
        r = (((uint32_t)ncid + 1u) % gx == 0) ? -1 : ncid;
    } else if ((tid + 1u) % gx == 0) {
        r = (((uint32_t)ncid) % gx == 0) ? -1 : ncid;
    } else {
        r = ncid;
    }
    if (r < 0 || (uint64_t)(uint32_t)r >= total) return -1;
    return r;
}

/* The same rule with 64-bit signed arithmetic, used where the reference's
 * 32-bit ids overflow (total + gx >= 2^31). */
inline int64_t neighbor_cell64(int64_t x, int64_t y, uint64_t cell, uint32_t gx,
                               uint64_t total) {
    int64_t ncid = y * (int64_t)gx + x;
    if (ncid < 0 || (uint64_t)ncid >= total) return -1;
    uint64_t cx = cell % gx;
    if (cx == 0) {
        if (((uint64_t)ncid + 1) % gx == 0) return -1;
    } else if (cx == (uint64_t)gx - 1) {
        if ((uint64_t)ncid % gx == 0) return -1;
    }
    return ncid;
}

/* Visit the up-to-9 neighbour cells of `cell` in the reference's order
 * (j outer, i inner: DeviceProcess_Kernel.h:24-28). */
template <class F>
inline void for_neighbor_cells(const oracle_grid& g, uint64_t cell, F&& fn) {
    if (g.compat32) {
        uint32_t cur = (uint32_t)cell;
        uint32_t cidy = cur / g.gx;
        uint32_t cidx = cur - g.gx * cidy;
        for (int j = -1; j <= 1; ++j)
            for (int i = -1; i <= 1; ++i) {
                int64_t nc = neighbor_cell32(cidx + (uint32_t)i, cidy + (uint32_t)j, cur,
                                             g.gx, g.total_cells);
                if (nc >= 0) fn((uint64_t)nc);
            }
    } else {
        int64_t cidy = (int64_t)(cell / g.gx);
        int64_t cidx = (int64_t)(cell % g.gx);
        for (int j = -1; j <= 1; ++j)
            for (int i = -1; i <= 1; ++i) {
                int64_t nc = neighbor_cell64(cidx + i, cidy + j, cell, g.gx, g.total_cells);
                if (nc >= 0) fn((uint64_t)nc);
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Bucketed data (CountCellFeatures, Codes/DeviceProcess.cu:312-369)         */
/* ------------------------------------------------------------------------ */

struct Data {
    uint64_t n = 0;
    uint32_t F = 0;
    const float* x = nullptr;
    const float* y = nullptr;
    const uint32_t* feat = nullptr;
    std::vector<uint32_t> fstart, fcount;
    oracle_grid g{};
    float R2 = 0.0f;
    float thr = 0.0f;
    std::vector<uint64_t> cellOf;
    std::vector<uint32_t> sorted;      /* point ids sorted by (cell, id) */
    /* (cell, feature) runs in sorted order: key = cell*F + f */
    std::vector<uint64_t> runKey;
    std::vector<uint64_t> runStart;
    std::vector<uint32_t> runCount;
    std::vector<uint64_t> cellKeys;    /* distinct occupied cells, ascending */
    std::vector<std::vector<uint32_t>> cellFeatRuns; /* per occupied cell: run indices */
    /* device outcomes for ambiguous pairs: key = min(a,b) << 32 | max(a,b) */
    const uint64_t* res_keys = nullptr;
    const uint8_t* res_le = nullptr;
    uint64_t nres = 0;
    mutable std::atomic<uint64_t> unresolved{0};

    /* The reference's neighbour test sq(a, b) <= R^2 (a = first instance). */
    bool near(uint32_t a, uint32_t b) const {
        SqDecision dc = sq_decide(x[a], y[a], x[b], y[b], R2);
        if (!dc.ambiguous) return dc.le;
        uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
        const uint64_t* it = std::lower_bound(res_keys, res_keys + nres, key);
        if (it != res_keys + nres && *it == key) return res_le[it - res_keys] != 0;
        unresolved.fetch_add(1, std::memory_order_relaxed);
        return dc.le;
    }

    /* run lookup: index of run (cell, f) or -1 */
    int64_t run(uint64_t cell, uint32_t f) const {
        uint64_t key = cell * (uint64_t)F + f;
        auto it = std::lower_bound(runKey.begin(), runKey.end(), key);
        if (it == runKey.end() || *it != key) return -1;
        return it - runKey.begin();
    }
    uint32_t count(uint64_t cell, uint32_t f) const {
        int64_t r = run(cell, f);
        return r < 0 ? 0u : runCount[r];
    }
};

int build_data(Data& d, const float* x, const float* y, const uint32_t* feat, uint64_t n,
               uint32_t F, const float bounds[4], float R, float thr) {
    d.n = n;
    d.F = F;
    d.x = x;
    d.y = y;
    d.feat = feat;
    d.thr = thr;
    d.R2 = R * R;                        /* colocationFinder.cpp:73 */
    if (make_grid(bounds[0], bounds[1], bounds[2], bounds[3], R, &d.g)) return 2;
    d.fstart.assign(F, 0);
    d.fcount.assign(F, 0);
    /* featureInstanceStart / Count (colocationFinder.cpp:168-229) */
    for (uint64_t i = 0; i < n; ++i) {
        if (feat[i] >= F) return 3;
        if (i > 0 && feat[i] < feat[i - 1]) return 3;
        if (d.fcount[feat[i]] == 0) d.fstart[feat[i]] = (uint32_t)i;
        d.fcount[feat[i]]++;
    }
    for (uint32_t f = 0; f < F; ++f)
        if (d.fcount[f] == 0) return 3;
    d.cellOf.resize(n);
    for (uint64_t i = 0; i < n; ++i) {
        if (!std::isfinite(x[i]) || !std::isfinite(y[i])) return 4;
        d.cellOf[i] = cell_of(d.g, x[i], y[i]);
        if (d.cellOf[i] >= d.g.total_cells) return 4;
    }
    /* thrust::sort_by_key on cell ids is stable (DeviceProcess.cu:342). */
    d.sorted.resize(n);
    for (uint64_t i = 0; i < n; ++i) d.sorted[i] = (uint32_t)i;
    std::stable_sort(d.sorted.begin(), d.sorted.end(),
                     [&](uint32_t a, uint32_t b) { return d.cellOf[a] < d.cellOf[b]; });
    for (uint64_t p = 0; p < n; ++p) {
        uint32_t id = d.sorted[p];
        uint64_t key = d.cellOf[id] * (uint64_t)F + feat[id];
        if (d.runKey.empty() || d.runKey.back() != key) {
            d.runKey.push_back(key);
            d.runStart.push_back(p);
            d.runCount.push_back(0);
        }
        d.runCount.back()++;
    }
    for (size_t r = 0; r < d.runKey.size(); ++r) {
        uint64_t cell = d.runKey[r] / F;
        if (d.cellKeys.empty() || d.cellKeys.back() != cell) {
            d.cellKeys.push_back(cell);
            d.cellFeatRuns.emplace_back();
        }
        d.cellFeatRuns.back().push_back((uint32_t)r);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Filter: cell-aggregate upper bound (DeviceProcess_Kernel.h:469-509 and    */
/* threshold_Kernel 545-573).  The reference's degree-2 variant             */
/* (filter2_2_Kernel, 512-543) reads an uninitialised index; the degree>=3  */
/* rule is applied to pairs as well.                                        */
/* ------------------------------------------------------------------------ */

struct FilterOut {
    std::vector<uint64_t> ub;   /* k entries */
    bool pass = false;
};

/* Threshold step, DeviceProcess_Kernel.h:545-573: per member
 * PI = (float)(countMap * 1.0 / (float)n_j), minimum, compare >= thr.
 * Only members j < 8 are ever counted (block (8,2,2) in
 * DeviceProcess.cu:223); the others keep countMap = 0. */
bool threshold_pass(const Data& d, const uint32_t* c, uint32_t k, const uint64_t* ub) {
    float pi0 = 1.0f;
    for (uint32_t j = 0; j < k; ++j) {
        float pr = (float)((double)ub[j] / (double)(float)d.fcount[c[j]]);
        if (j == 0) pi0 = pr;
        else if (pi0 > pr) pi0 = pr;
    }
    return pi0 >= d.thr;
}

/* Sparse restatement: a quad can be full only if it holds member 0, so the
 * quads of member-0 cells are the only ones examined. */
FilterOut filter_sparse(const Data& d, const uint32_t* c, uint32_t k) {
    FilterOut out;
    out.ub.assign(k, 0);
    const oracle_grid& g = d.g;
    uint32_t m = k < 8 ? k : 8;
    if (g.gx >= 2 && g.gy >= 2) {
        std::unordered_set<uint64_t> quads;   /* key = by*gx + bx */
        std::unordered_set<uint64_t> cells;
        for (size_t ci = 0; ci < d.cellKeys.size(); ++ci) {
            uint64_t cell = d.cellKeys[ci];
            if (d.count(cell, c[0]) == 0) continue;
            uint64_t cx = cell % g.gx, cy = cell / g.gx;
            for (int dy = -1; dy <= 0; ++dy)
                for (int dx = -1; dx <= 0; ++dx) {
                    int64_t bx = (int64_t)cx + dx, by = (int64_t)cy + dy;
                    if (bx < 0 || by < 0 || bx > (int64_t)g.gx - 2 || by > (int64_t)g.gy - 2)
                        continue;
                    uint64_t qk = (uint64_t)by * g.gx + (uint64_t)bx;
                    if (quads.count(qk)) continue;
                    quads.insert(qk);
                    bool full = true;
                    for (uint32_t j = 0; j < m && full; ++j) {
                        uint64_t s = 0;
                        for (int yy = 0; yy < 2; ++yy)
                            for (int xx = 0; xx < 2; ++xx)
                                s += d.count((uint64_t)(by + yy) * g.gx + (uint64_t)(bx + xx), c[j]);
                        if (s == 0) full = false;
                    }
                    if (!full) continue;
                    for (int yy = 0; yy < 2; ++yy)
                        for (int xx = 0; xx < 2; ++xx)
                            cells.insert((uint64_t)(by + yy) * g.gx + (uint64_t)(bx + xx));
                }
        }
        for (uint64_t cell : cells)
            for (uint32_t j = 0; j < m; ++j) out.ub[j] += d.count(cell, c[j]);
    }
    out.pass = threshold_pass(d, c, k, out.ub.data());
    return out;
}

/* Literal dense restatement (every quad of the grid, claim flags per cell). */
FilterOut filter_dense(const Data& d, const uint32_t* c, uint32_t k) {
    FilterOut out;
    out.ub.assign(k, 0);
    const oracle_grid& g = d.g;
    uint32_t m = k < 8 ? k : 8;
    std::vector<uint8_t> processed(g.total_cells, 0);
    for (uint64_t by = 0; by + 1 < g.gy; ++by)
        for (uint64_t bx = 0; bx + 1 < g.gx; ++bx) {
            uint64_t cnt[8][2][2];
            bool done = false;
            for (uint32_t j = 0; j < m; ++j) {
                uint64_t s = 0;
                for (int yy = 0; yy < 2; ++yy)
                    for (int xx = 0; xx < 2; ++xx) {
                        cnt[j][xx][yy] = d.count((by + yy) * g.gx + bx + xx, c[j]);
                        s += cnt[j][xx][yy];
                    }
                if (s == 0) done = true;
            }
            if (done) continue;
            for (int yy = 0; yy < 2; ++yy)
                for (int xx = 0; xx < 2; ++xx) {
                    uint64_t cid = (by + yy) * g.gx + bx + xx;
                    if (processed[cid]) continue;
                    processed[cid] = 1;
                    for (uint32_t j = 0; j < m; ++j) out.ub[j] += cnt[j][xx][yy];
                }
        }
    out.pass = threshold_pass(d, c, k, out.ub.data());
    return out;
}

/* ------------------------------------------------------------------------ */
/* Refinement: slot counting with bitmaps and participation index           */
/* ------------------------------------------------------------------------ */

struct Refined {
    uint64_t rows = 0;
    std::vector<uint64_t> num;   /* k numerators as getParticipationIndex sums them */
    float pi = 1.0f;
    uint32_t argmin = 0;
    std::vector<uint32_t> slots; /* per parent row (or per anchor for k = 2) */
};

/* Codes/DeviceProcess.cu:108-132 (getParticipationIndex): window sums over a
 * word-per-bit bitmap, float ratio, strict-< minimum starting at 1.0. */
void participation(const Data& d, const uint32_t* c, uint32_t k, const std::vector<uint8_t>& bm,
                   Refined& out) {
    out.num.assign(k, 0);
    float PI = 1.0f;
    uint32_t from = 0, to = 0;
    out.argmin = 0;
    for (uint32_t j = 0; j < k; ++j) {
        uint32_t total = d.fcount[c[j]];
        if (j == 0) {
            from = 0;
            to = total;
        } else {
            from = to - 1;
            to = from + total + 1;
        }
        uint64_t s = 0;
        for (uint64_t p = from; p + 1 < (uint64_t)to; ++p) s += bm[p];   /* reduce(from, to-1) */
        out.num[j] = s;
        float pr = (float)s / (float)total;
        if (pr < PI) {
            PI = pr;
            out.argmin = j;
        }
    }
    out.pi = PI;
}

inline void set_bit(std::vector<uint8_t>& bm, uint64_t i) {
    __atomic_store_n(&bm[i], (uint8_t)1, __ATOMIC_RELAXED);
}

/* Degree 2: degree2TableSlotCounter_Kernel (DeviceProcess_Kernel.h:12-55).
 * Bitmap layout: first feature at TID, second at b - secondstart + (n0-1). */
Refined refine2(const Data& d, uint32_t f0, uint32_t f1) {
    Refined out;
    uint32_t start = d.fstart[f0], n0 = d.fcount[f0], n1 = d.fcount[f1];
    uint32_t secondstart = d.fstart[f1];
    std::vector<uint8_t> bm((size_t)n0 + n1, 0);
    out.slots.assign(n0, 0);
    uint64_t rows = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : rows)
    for (int64_t tid = 0; tid < (int64_t)n0; ++tid) {
        uint32_t a = start + (uint32_t)tid;
        uint32_t cnt = 0;
        for_neighbor_cells(d.g, d.cellOf[a], [&](uint64_t nc) {
            int64_t r = d.run(nc, f1);
            if (r < 0) return;
            for (uint64_t p = d.runStart[r]; p < d.runStart[r] + d.runCount[r]; ++p) {
                uint32_t b = d.sorted[p];
                if (d.near(a, b)) {
                    cnt++;
                    set_bit(bm, (uint64_t)tid);
                    set_bit(bm, (uint64_t)(b - secondstart) + (n0 - 1));
                }
            }
        });
        out.slots[tid] = cnt;
        rows += cnt;
    }
    out.rows = rows;
    uint32_t c[2] = {f0, f1};
    participation(d, c, 2, bm, out);
    return out;
}

/* degree2TableGenerator_Kernel (DeviceProcess_Kernel.h:56-100): rows (a,b)
 * ordered by anchor, neighbour cell, then b. */
std::vector<uint32_t> fill2(const Data& d, uint32_t f0, uint32_t f1, const Refined& ref) {
    uint32_t start = d.fstart[f0], n0 = d.fcount[f0];
    std::vector<uint64_t> off((size_t)n0 + 1, 0);
    for (uint32_t t = 0; t < n0; ++t) off[t + 1] = off[t] + ref.slots[t];
    std::vector<uint32_t> tab(off[n0] * 2);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t tid = 0; tid < (int64_t)n0; ++tid) {
        uint32_t a = start + (uint32_t)tid;
        uint64_t o = off[tid] * 2;
        for_neighbor_cells(d.g, d.cellOf[a], [&](uint64_t nc) {
            int64_t r = d.run(nc, f1);
            if (r < 0) return;
            for (uint64_t p = d.runStart[r]; p < d.runStart[r] + d.runCount[r]; ++p) {
                uint32_t b = d.sorted[p];
                if (d.near(a, b)) {
                    tab[o++] = a;
                    tab[o++] = b;
                }
            }
        });
    }
    return tab;
}

/* Degree k >= 3: generalInstanceTableSlotCounter_Kernel
 * (DeviceProcess_Kernel.h:255-316).  Bitmap offsets are the running sums of
 * member counts. */
Refined refinek(const Data& d, const uint32_t* c, uint32_t k, const std::vector<uint32_t>& parent) {
    Refined out;
    uint32_t km1 = k - 1;
    uint64_t prow = parent.size() / km1;
    uint64_t bmsize = 0;
    for (uint32_t j = 0; j < k; ++j) bmsize += d.fcount[c[j]];
    std::vector<uint8_t> bm(bmsize, 0);
    std::vector<uint64_t> offs(k, 0);
    for (uint32_t j = 1; j < k; ++j) offs[j] = offs[j - 1] + d.fcount[c[j - 1]];
    uint32_t last = c[k - 1];
    out.slots.assign(prow, 0);
    uint64_t rows = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : rows)
    for (int64_t tid = 0; tid < (int64_t)prow; ++tid) {
        const uint32_t* r = &parent[(size_t)tid * km1];
        uint32_t cnt = 0;
        for_neighbor_cells(d.g, d.cellOf[r[0]], [&](uint64_t nc) {
            int64_t ru = d.run(nc, last);
            if (ru < 0) return;
            for (uint64_t p = d.runStart[ru]; p < d.runStart[ru] + d.runCount[ru]; ++p) {
                uint32_t b = d.sorted[p];
                bool ok = true;
                for (uint32_t i = 0; i < km1 && ok; ++i)
                    if (!d.near(r[i], b)) ok = false;
                if (!ok) continue;
                cnt++;
                for (uint32_t i = 0; i < km1; ++i)
                    set_bit(bm, (uint64_t)(r[i] - d.fstart[c[i]]) + offs[i]);
                set_bit(bm, (uint64_t)(b - d.fstart[last]) + offs[km1]);
            }
        });
        out.slots[tid] = cnt;
        rows += cnt;
    }
    out.rows = rows;
    participation(d, c, k, bm, out);
    return out;
}

/* generateInstanceTableGeneral_Kernel (DeviceProcess_Kernel.h:318-385). */
std::vector<uint32_t> fillk(const Data& d, const uint32_t* c, uint32_t k,
                            const std::vector<uint32_t>& parent, const Refined& ref) {
    uint32_t km1 = k - 1;
    uint64_t prow = parent.size() / km1;
    std::vector<uint64_t> off(prow + 1, 0);
    for (uint64_t t = 0; t < prow; ++t) off[t + 1] = off[t] + ref.slots[t];
    std::vector<uint32_t> tab(off[prow] * k);
    uint32_t last = c[k - 1];
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t tid = 0; tid < (int64_t)prow; ++tid) {
        if (ref.slots[tid] == 0) continue;
        const uint32_t* r = &parent[(size_t)tid * km1];
        uint64_t o = off[tid] * k;
        for_neighbor_cells(d.g, d.cellOf[r[0]], [&](uint64_t nc) {
            int64_t ru = d.run(nc, last);
            if (ru < 0) return;
            for (uint64_t p = d.runStart[ru]; p < d.runStart[ru] + d.runCount[ru]; ++p) {
                uint32_t b = d.sorted[p];
                bool ok = true;
                for (uint32_t i = 0; i < km1 && ok; ++i)
                    if (!d.near(r[i], b)) ok = false;
                if (!ok) continue;
                for (uint32_t i = 0; i < km1; ++i) tab[o++] = r[i];
                tab[o++] = b;
            }
        });
    }
    return tab;
}

/* ------------------------------------------------------------------------ */
/* Apriori candidate generation                                             */
/* ------------------------------------------------------------------------ */

/* subsetGen (colocationFinder.cpp:598-616) emits the (n-1)-subsets of a
 * candidate in lexicographic position order: subset i drops position n-1-i. */
void subsets_lex(const std::vector<uint32_t>& inter, std::vector<std::vector<uint32_t>>& out) {
    size_t n = inter.size();
    out.clear();
    for (size_t i = 0; i < n; ++i) {
        size_t drop = n - 1 - i;
        std::vector<uint32_t> s;
        for (size_t t = 0; t < n; ++t)
            if (t != drop) s.push_back(inter[t]);
        out.push_back(s);
    }
}

/* checkSubset (colocationFinder.cpp:618-634): linear search. */
bool check_subset(const std::vector<uint32_t>& prev, size_t nprev, const std::vector<uint32_t>& s) {
    size_t deg = s.size();
    for (size_t i = 0; i < nprev; ++i) {
        bool eq = true;
        for (size_t j = 0; j < deg; ++j)
            if (prev[i * deg + j] != s[j]) {
                eq = false;
                break;
            }
        if (eq) return true;
    }
    return nprev == 0;   /* the reference's flag starts true */
}

/* candidateColocationGeneral (colocationFinder.cpp:517-557): join on equal
 * (k-2)-prefix, check subsets 2..k-1 (generateandCheckSubsets, 669-679),
 * and BREAK out of the inner loop on the first failing subset check. */
std::vector<uint32_t> apriori(const std::vector<uint32_t>& prev, size_t nprev, uint32_t degree) {
    std::vector<uint32_t> cand;
    uint32_t lastIndex = degree - 2;
    std::vector<std::vector<uint32_t>> subs;
    for (size_t i = 0; i < nprev; ++i) {
        bool flag = true;
        for (size_t j = i + 1; j < nprev; ++j) {
            for (size_t k = 0; k < lastIndex; ++k)
                if (prev[i * (degree - 1) + k] != prev[j * (degree - 1) + k]) {
                    flag = false;
                    break;
                }
            if (flag && prev[i * (degree - 1) + lastIndex] < prev[j * (degree - 1) + lastIndex]) {
                std::vector<uint32_t> inter(prev.begin() + i * (degree - 1),
                                            prev.begin() + (i + 1) * (degree - 1));
                inter.push_back(prev[j * (degree - 1) + lastIndex]);
                subsets_lex(inter, subs);
                flag = true;
                for (size_t s = 2; s < degree; ++s) {
                    flag = check_subset(prev, nprev, subs[s]);
                    if (!flag) break;
                }
                if (!flag) break;
                cand.insert(cand.end(), inter.begin(), inter.end());
            } else {
                break;
            }
        }
    }
    return cand;
}

/* getIndex (colocationFinder.cpp:703-718) */
int64_t find_pattern(const std::vector<uint32_t>& list, size_t cnt, uint32_t deg, const uint32_t* p) {
    for (size_t i = 0; i < cnt; ++i) {
        bool eq = true;
        for (uint32_t j = 0; j < deg; ++j)
            if (list[i * deg + j] != p[j]) {
                eq = false;
                break;
            }
        if (eq) return (int64_t)i;
    }
    return -1;
}

}  // namespace

/* ------------------------------------------------------------------------ */
/* Result                                                                   */
/* ------------------------------------------------------------------------ */

struct OLevel {
    uint32_t k = 0;
    std::vector<uint32_t> cand;
    std::vector<uint64_t> ub, num, rows;
    std::vector<uint8_t> pass, prevalent;
    std::vector<float> pi;
    std::vector<uint32_t> argmin;
    std::vector<std::vector<uint32_t>> tables;   /* per candidate (kept on request) */
    std::vector<uint8_t> has_table;
};

struct oracle_result {
    int status = 0;
    uint64_t unresolved = 0;    /* ambiguous comparisons without a device outcome */
    std::vector<OLevel> levels;
    double phase_ms[6] = {0, 0, 0, 0, 0, 0};   /* oracle_mine_fast: bucketing, join, filter, refine, fill, Apriori */
};

extern "C" {

int oracle_make_grid(float min_x, float min_y, float max_x, float max_y, float R, oracle_grid* g) {
    return make_grid(min_x, min_y, max_x, max_y, R, g);
}

uint64_t oracle_cell_ids(const oracle_grid* g, const float* x, const float* y, uint64_t n,
                         uint64_t* cell_out) {
    uint64_t bad = 0;
    for (uint64_t i = 0; i < n; ++i) {
        cell_out[i] = cell_of(*g, x[i], y[i]);
        if (cell_out[i] >= g->total_cells) bad++;
    }
    return bad;
}

float oracle_sqdist(float x1, float y1, float x2, float y2) { return sqdist(x1, y1, x2, y2); }

int oracle_cell_adjacent(const oracle_grid* g, uint64_t c, uint64_t nb) {
    int hit = 0;
    for_neighbor_cells(*g, c, [&](uint64_t nc) {
        if (nc == nb) hit = 1;
    });
    return hit;
}

int oracle_mine(const float* x, const float* y, const uint32_t* feat, uint64_t n, uint32_t nfeat,
                const float bounds[4], float R, float thr, uint32_t max_k, int threads,
                int keep_tables, const uint64_t* res_keys, const uint8_t* res_le, uint64_t nres,
                oracle_result** out) {
    oracle_result* res = new oracle_result();
    *out = res;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    if (n == 0 || nfeat < 2) return res->status = 0;
    Data d;
    int st = build_data(d, x, y, feat, n, nfeat, bounds, R, thr);
    if (st) return res->status = st;
    d.res_keys = res_keys;
    d.res_le = res_le;
    d.nres = res_keys ? nres : 0;
    struct Tally {
        oracle_result* r;
        const Data& d;
        ~Tally() { r->unresolved = d.unresolved.load(); }
    } tally{res, d};

    /* ---- degree 2 (degree2Processing, colocationFinder.cpp:256-425) ---- */
    std::vector<uint32_t> cands;
    for (uint32_t i = 0; i + 1 < nfeat; ++i)       /* 75-82 */
        for (uint32_t j = i + 1; j < nfeat; ++j) {
            cands.push_back(i);
            cands.push_back(j);
        }
    uint32_t k = 2;
    std::vector<uint32_t> prev;                    /* prevalent patterns of level k */
    std::vector<size_t> prevIdx;                   /* their candidate index */
    std::vector<std::vector<uint32_t>> prevTables; /* table per prevalent pattern (if built) */
    std::vector<std::vector<uint32_t>> parentTables;
    std::vector<uint32_t> parentList;              /* prevalent (k-1)-patterns */
    while (true) {
        size_t C = cands.size() / k;
        OLevel L;
        L.k = k;
        L.cand = cands;
        L.ub.assign(C * k, 0);
        L.num.assign(C * k, 0);
        L.rows.assign(C, 0);
        L.pass.assign(C, 0);
        L.prevalent.assign(C, 0);
        L.pi.assign(C, -1.0f);
        L.argmin.assign(C, 0);
        std::vector<Refined> refs(C);
        /* filter (2 in the order of the candidates) */
        std::vector<FilterOut> fo(C);
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t c = 0; c < (int64_t)C; ++c) fo[c] = filter_sparse(d, &cands[c * k], k);
        for (size_t c = 0; c < C; ++c) {
            for (uint32_t j = 0; j < k; ++j) L.ub[c * k + j] = fo[c].ub[j];
            L.pass[c] = fo[c].pass;
        }
        /* refinement per surviving candidate */
        prev.clear();
        prevIdx.clear();
        for (size_t c = 0; c < C; ++c) {
            if (!L.pass[c]) continue;
            const uint32_t* cc = &cands[c * k];
            if (k == 2) {
                refs[c] = refine2(d, cc[0], cc[1]);
            } else {
                int64_t pi = find_pattern(parentList, parentList.size() / (k - 1), k - 1, cc);
                if (pi < 0) return res->status = 5;
                refs[c] = refinek(d, cc, k, parentTables[pi]);
            }
            L.rows[c] = refs[c].rows;
            for (uint32_t j = 0; j < k; ++j) L.num[c * k + j] = refs[c].num[j];
            L.pi[c] = refs[c].pi;
            L.argmin[c] = refs[c].argmin;
            if (!(refs[c].pi < thr)) {                   /* cpp:335, cpp:827 */
                L.prevalent[c] = 1;
                prev.insert(prev.end(), cc, cc + k);
                prevIdx.push_back(c);
            }
        }
        size_t P = prevIdx.size();
        /* next-level candidates (candidateColocationGeneral(k+1)) */
        std::vector<uint32_t> next;
        if (P > 0 && (max_k == 0 || k + 1 <= max_k) && k + 1 <= nfeat) next = apriori(prev, P, k + 1);
        size_t Cn = next.size() / (k + 1);
        /* tables for prevalent patterns that prefix a next candidate
         * (calcInstanceTablePatternIndexes, cpp:1042-1066 / cpp:364-372) */
        std::vector<uint8_t> need(P, 0);
        for (size_t i = 0; i < Cn; ++i) {
            int64_t ix = find_pattern(prev, P, k, &next[i * (k + 1)]);
            if (ix >= 0) need[ix] = 1;
        }
        std::vector<std::vector<uint32_t>> newTables(P);
        L.tables.assign(keep_tables ? C : 0, {});
        L.has_table.assign(C, 0);
        for (size_t p = 0; p < P; ++p) {
            if (!need[p]) continue;
            size_t c = prevIdx[p];
            const uint32_t* cc = &cands[c * k];
            if (k == 2) {
                newTables[p] = fill2(d, cc[0], cc[1], refs[c]);
            } else {
                int64_t pi = find_pattern(parentList, parentList.size() / (k - 1), k - 1, cc);
                newTables[p] = fillk(d, cc, k, parentTables[pi], refs[c]);
            }
            L.has_table[c] = 1;
            if (keep_tables) L.tables[c] = newTables[p];
        }
        res->levels.push_back(std::move(L));
        if (Cn == 0) break;
        parentTables.swap(newTables);
        parentList = prev;
        cands = next;
        k++;
    }
    return res->status = 0;
}

void oracle_free(oracle_result* r) { delete r; }
void oracle_phase_ms(const oracle_result* r, double* ms6) { std::memcpy(ms6, r->phase_ms, sizeof(r->phase_ms)); }
int oracle_status(const oracle_result* r) { return r->status; }
uint64_t oracle_unresolved(const oracle_result* r) { return r->unresolved; }
uint32_t oracle_num_levels(const oracle_result* r) { return (uint32_t)r->levels.size(); }
uint32_t oracle_level_k(const oracle_result* r, uint32_t li) { return r->levels[li].k; }
uint64_t oracle_level_ncand(const oracle_result* r, uint32_t li) {
    return r->levels[li].cand.size() / r->levels[li].k;
}

void oracle_level_get(const oracle_result* r, uint32_t li, uint32_t* cand, uint64_t* ub, uint8_t* pass,
                      uint64_t* rows, uint64_t* num, float* pi, uint8_t* prevalent, uint32_t* argmin) {
    const OLevel& L = r->levels[li];
    size_t C = L.cand.size() / L.k;
    if (cand) std::memcpy(cand, L.cand.data(), L.cand.size() * 4);
    if (ub) std::memcpy(ub, L.ub.data(), L.ub.size() * 8);
    if (pass) std::memcpy(pass, L.pass.data(), C);
    if (rows) std::memcpy(rows, L.rows.data(), C * 8);
    if (num) std::memcpy(num, L.num.data(), L.num.size() * 8);
    if (pi) std::memcpy(pi, L.pi.data(), C * 4);
    if (prevalent) std::memcpy(prevalent, L.prevalent.data(), C);
    if (argmin) std::memcpy(argmin, L.argmin.data(), C * 4);
}

uint64_t oracle_table(const oracle_result* r, uint32_t li, uint64_t ci, uint32_t* out) {
    const OLevel& L = r->levels[li];
    if (ci >= L.tables.size() || !L.has_table[ci]) return UINT64_MAX;
    const auto& t = L.tables[ci];
    if (out) std::memcpy(out, t.data(), t.size() * 4);
    return t.size() / L.k;
}

uint64_t oracle_neighbors(const float* x, const float* y, const uint32_t* feat, uint64_t n,
                          uint32_t nfeat, const float bounds[4], float R, const uint64_t* res_keys,
                          const uint8_t* res_le, uint64_t nres, uint64_t* offs, uint32_t* nbr,
                          uint64_t* n_unresolved) {
    Data d;
    if (build_data(d, x, y, feat, n, nfeat, bounds, R, 0.0f)) return UINT64_MAX;
    d.res_keys = res_keys;
    d.res_le = res_le;
    d.nres = res_keys ? nres : 0;
    std::vector<std::vector<uint32_t>> lists(n);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t a = 0; a < (int64_t)n; ++a) {
        for (uint32_t f = feat[a] + 1; f < nfeat; ++f) {
            for_neighbor_cells(d.g, d.cellOf[a], [&](uint64_t nc) {
                int64_t r = d.run(nc, f);
                if (r < 0) return;
                for (uint64_t p = d.runStart[r]; p < d.runStart[r] + d.runCount[r]; ++p) {
                    uint32_t b = d.sorted[p];
                    if (d.near((uint32_t)a, b)) lists[a].push_back(b);
                }
            });
        }
    }
    uint64_t tot = 0;
    for (uint64_t a = 0; a < n; ++a) {
        if (offs) offs[a] = tot;
        if (nbr) std::memcpy(nbr + tot, lists[a].data(), lists[a].size() * 4);
        tot += lists[a].size();
    }
    if (offs) offs[n] = tot;
    if (n_unresolved) *n_unresolved = d.unresolved.load();
    return tot;
}

void oracle_sq_decide_batch(const float* x1, const float* y1, const float* x2, const float* y2, uint64_t n,
                            float R2, uint8_t* le, uint8_t* ambiguous, float* value, uint8_t* near_mid) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        SqDecision dc = sq_decide(x1[i], y1[i], x2[i], y2[i], R2);
        le[i] = dc.le;
        ambiguous[i] = dc.ambiguous;
        ExactSq e = exact_sq(x1[i], y1[i], x2[i], y2[i]);
        if (value) value[i] = e.rn;
        if (near_mid) near_mid[i] = e.near_mid;
    }
}

int oracle_sq_decide(float x1, float y1, float x2, float y2, float R2, int* ambiguous) {
    SqDecision dc = sq_decide(x1, y1, x2, y2, R2);
    if (ambiguous) *ambiguous = dc.ambiguous ? 1 : 0;
    return dc.le ? 1 : 0;
}

/* Every pair of points of different features whose comparison with R^2 an
 * exact tie could flip.  Candidate pairs come from a uniform grid of cell
 * size R over the true coordinates (a 5x5 stencil covers every pair at
 * distance <= 2R), so the set does not depend on the reference grid.  Each
 * unordered pair of grid cells is visited once, in parallel; within a pair
 * of cells only points of different features are compared, and only sums
 * within 2^-20 of R^2 go through the exact test. */
uint64_t oracle_ambiguous_pairs(const float* x, const float* y, const uint32_t* feat, uint64_t n,
                                float R, uint64_t* keys, uint64_t cap) {
    const float R2 = R * R;
    const double w = (double)R, R2d = (double)R2, win = std::ldexp(R2d, -20);
    struct P {
        int64_t cy, cx;
        uint32_t f, id;
    };
    std::vector<P> pts(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i)
        pts[i] = {(int64_t)std::floor((double)y[i] / w), (int64_t)std::floor((double)x[i] / w), feat[i], (uint32_t)i};
    auto less = [](const P& a, const P& b) {
        if (a.cy != b.cy) return a.cy < b.cy;
        if (a.cx != b.cx) return a.cx < b.cx;
        if (a.f != b.f) return a.f < b.f;
        return a.id < b.id;
    };
#ifdef _OPENMP
    __gnu_parallel::sort(pts.begin(), pts.end(), less);
#else
    std::sort(pts.begin(), pts.end(), less);
#endif
    std::vector<uint64_t> cb;            /* first point of each grid cell */
    std::vector<uint64_t> rb;            /* first cell of each grid row */
    for (uint64_t p = 0; p < n; ++p)
        if (p == 0 || pts[p].cx != pts[p - 1].cx || pts[p].cy != pts[p - 1].cy) {
            if (cb.empty() || pts[p].cy != pts[cb.back()].cy) rb.push_back(cb.size());
            cb.push_back(p);
        }
    const uint64_t NC = cb.size(), NR = rb.size();
    cb.push_back(n);
    rb.push_back(NC);
    std::vector<uint64_t> crow(NC);
    for (uint64_t r = 0; r < NR; ++r)
        for (uint64_t c = rb[r]; c < rb[r + 1]; ++c) crow[c] = r;
    auto pair_cells = [&](uint64_t A, uint64_t B, std::vector<uint64_t>& out) {
        for (uint64_t i = cb[A]; i < cb[A + 1]; ++i) {
            const P& a = pts[i];
            for (uint64_t j = (A == B ? i + 1 : cb[B]); j < cb[B + 1]; ++j) {
                const P& b = pts[j];
                if (a.f == b.f) continue;
                const float dx = x[b.id] - x[a.id], dy = y[b.id] - y[a.id];
                const double S = (double)dx * (double)dx + (double)dy * (double)dy;
                if (std::fabs(S - R2d) > win) continue;
                if (!sq_decide(x[a.id], y[a.id], x[b.id], y[b.id], R2).ambiguous) continue;
                const uint32_t lo = a.id < b.id ? a.id : b.id, hi = a.id < b.id ? b.id : a.id;
                out.push_back(((uint64_t)lo << 32) | hi);
            }
        }
    };
    std::vector<uint64_t> found;
#pragma omp parallel
    {
        std::vector<uint64_t> loc;
#pragma omp for schedule(dynamic, 256)
        for (int64_t A = 0; A < (int64_t)NC; ++A) {
            const int64_t ay = pts[cb[A]].cy, ax = pts[cb[A]].cx;
            for (uint64_t r = crow[A]; r < NR && r <= crow[A] + 2; ++r) {
                const int64_t ry = pts[cb[rb[r]]].cy;
                if (ry > ay + 2) break;
                const int64_t x0 = ry == ay ? ax : ax - 2;   /* same row: this cell and the ones after it */
                uint64_t lo = rb[r], hi = rb[r + 1];
                while (lo < hi) {                          /* first cell of the row with cx >= x0 */
                    const uint64_t mid = (lo + hi) / 2;
                    if (pts[cb[mid]].cx < x0) lo = mid + 1;
                    else hi = mid;
                }
                for (uint64_t B = lo; B < rb[r + 1] && pts[cb[B]].cx <= ax + 2; ++B) pair_cells((uint64_t)A, B, loc);
            }
        }
#pragma omp critical
        found.insert(found.end(), loc.begin(), loc.end());
    }
    std::sort(found.begin(), found.end());
    if (keys) std::memcpy(keys, found.data(), std::min<uint64_t>(found.size(), cap) * 8);
    return found.size();
}

int oracle_filter_dense(const float* x, const float* y, const uint32_t* feat, uint64_t n,
                        uint32_t nfeat, const float bounds[4], float R, float thr,
                        const uint32_t* cand, uint64_t ncand, uint32_t k, uint64_t* ub,
                        uint8_t* pass) {
    Data d;
    int st = build_data(d, x, y, feat, n, nfeat, bounds, R, thr);
    if (st) return st;
    for (uint64_t c = 0; c < ncand; ++c) {
        FilterOut f = filter_dense(d, cand + c * k, k);
        for (uint32_t j = 0; j < k; ++j) ub[c * k + j] = f.ub[j];
        pass[c] = f.pass;
    }
    return 0;
}

uint64_t oracle_apriori(const uint32_t* prev, uint64_t nprev, uint32_t k, uint32_t* out,
                        uint64_t out_cap) {
    std::vector<uint32_t> p(prev, prev + nprev * (k - 1));
    std::vector<uint32_t> c = apriori(p, nprev, k);
    uint64_t nc = c.size() / k;
    if (out) std::memcpy(out, c.data(), std::min<uint64_t>(nc, out_cap) * k * 4);
    return nc;
}

/* ------------------------------------------------------------------------ */
/* Parsing                                                                  */
/* ------------------------------------------------------------------------ */

namespace {
/* boost::escaped_list_separator<char> defaults: separator ',', quote '"',
 * escape '\\' (the tokenizer used at colocationFinder.cpp:156). */
std::vector<std::string> split_csv(const std::string& line) {
    std::vector<std::string> out;
    std::string cur;
    bool inq = false;
    for (size_t i = 0; i < line.size(); ++i) {
        char ch = line[i];
        if (ch == '\\' && i + 1 < line.size()) {
            char nx = line[++i];
            cur.push_back(nx == 'n' ? '\n' : nx);
        } else if (ch == '"') {
            inq = !inq;
        } else if (ch == ',' && !inq) {
            out.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(ch);
        }
    }
    out.push_back(cur);
    return out;
}
bool to_float(const std::string& s, float* v) {          /* std::stof */
    const char* b = s.c_str();
    char* e = nullptr;
    *v = std::strtof(b, &e);
    return e != b;
}
bool to_int(const std::string& s, long* v) {             /* std::stoi */
    const char* b = s.c_str();
    char* e = nullptr;
    *v = std::strtol(b, &e, 10);
    return e != b && *v >= INT32_MIN && *v <= INT32_MAX;
}
bool next_line(std::ifstream& in, std::string& line) {
    bool ok = (bool)std::getline(in, line);
    if (!line.empty() && line.back() == '\r') line.pop_back();
    return ok;
}
}  // namespace

int oracle_parse_csv(const char* path, uint64_t* n, uint32_t* nfeat, float* x, float* y,
                     uint32_t* feat, float bounds[4], char* names, uint64_t names_cap) {
    std::ifstream in(path);
    if (!in.is_open()) return 1;
    std::string line;
    next_line(in, line);
    long N;
    if (!to_int(line, &N) || N < 0) return 2;
    uint64_t cnt = 0;
    uint32_t F = 0;
    size_t last = (size_t)-1;
    std::string nm;
    next_line(in, line);
    while (!line.empty()) {
        std::vector<std::string> v = split_csv(line);
        if (v.size() < 3) return 2;
        long fid;
        if (!to_int(v[0], &fid) || fid == -1) return 2;
        if (last == (size_t)-1 || (size_t)fid != last) {
            last = (size_t)fid;
            if (F > 0) nm.push_back('\n');
            nm += v[0];
            F++;
        }
        float xv, yv;
        if (!to_float(v[1], &xv) || !to_float(v[2], &yv)) return 2;
        if (x && cnt < (uint64_t)N) {
            feat[cnt] = F - 1;
            x[cnt] = xv;
            y[cnt] = yv;
        }
        cnt++;
        line.clear();
        next_line(in, line);
    }
    if (cnt != (uint64_t)N) return 3;
    line.clear();
    next_line(in, line);
    std::vector<std::string> v = split_csv(line);
    if (v.size() < 4) return 2;
    float bb[4];
    for (int i = 0; i < 4; ++i)
        if (!to_float(v[i], &bb[i])) return 2;
    if (bounds) std::memcpy(bounds, bb, sizeof(bb));
    *n = cnt;
    *nfeat = F;
    if (names && names_cap > 0) {
        size_t m = std::min<size_t>(nm.size(), names_cap - 1);
        std::memcpy(names, nm.data(), m);
        names[m] = 0;
    }
    return 0;
}

int oracle_parse_params(const char* path, float* R, float* thr, uint32_t* filter_flag) {
    std::ifstream ifs(path);
    if (!ifs.is_open()) return 1;
    float r = 0, t = 0;
    unsigned f = 0;
    ifs >> r;
    ifs >> t;
    ifs >> f;
    if (ifs.fail() && !ifs.eof()) return 2;
    *R = r;
    *thr = t;
    *filter_flag = f;
    return 0;
}

}  // extern "C"

/* ------------------------------------------------------------------------- */
/* Cost model: the network of the CUDA kernels (gpu-colocationmininig_gb300/  */
/* csrc/colo_mlp.cu) restated per row, to check their outputs and gradients. */
/* With bf16 = 1 the same values are rounded to BF16 (round to nearest even) */
/* before they enter a product: inputs, weights, H1, H2, dZ2, dZ1; sums are   */
/* taken in double.  With bf16 = 0 nothing is rounded, so the gradient can   */
/* be checked against finite differences.                                    */
/* ------------------------------------------------------------------------- */
static float bf16_rne(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

namespace {
constexpr int MI = 24, MIP = 32, MH = 64;
constexpr int M_W1 = 0, M_B1 = MIP * MH, M_W2 = M_B1 + MH, M_B2 = M_W2 + MH * MH, M_W3 = M_B2 + MH, M_B3 = M_W3 + MH;

struct MlpRow {
    double xb[MIP], z1[MH], h1[MH], z2[MH], h2[MH], y;
};

void mlp_row(const float* P, const float* x, int bf16, MlpRow& r) {
    auto q = [&](double v) { return bf16 ? (double)bf16_rne((float)v) : v; };
    for (int i = 0; i < MIP; ++i) r.xb[i] = i < MI ? q(x[i]) : 0.0;
    for (int o = 0; o < MH; ++o) {
        double a = P[M_B1 + o];
        for (int i = 0; i < MIP; ++i) a += r.xb[i] * q(P[M_W1 + i * MH + o]);
        r.z1[o] = a;
        r.h1[o] = q(a > 0 ? a : 0.0);
    }
    for (int o = 0; o < MH; ++o) {
        double a = P[M_B2 + o];
        for (int i = 0; i < MH; ++i) a += r.h1[i] * q(P[M_W2 + i * MH + o]);
        r.z2[o] = a;
        r.h2[o] = q(a > 0 ? a : 0.0);
    }
    double y = P[M_B3];
    for (int o = 0; o < MH; ++o) y += r.h2[o] * q(P[M_W3 + o]);
    r.y = y;
}
}  // namespace

extern "C" {

void oracle_mlp_forward(const float* P, const float* X, uint64_t n, int bf16, double* Y) {
    MlpRow r;
    for (uint64_t i = 0; i < n; ++i) {
        mlp_row(P, X + i * MI, bf16, r);
        Y[i] = r.y;
    }
}

void oracle_mlp_grad(const float* P, const float* X, const float* T, uint64_t n, int bf16, double* G, double* loss) {
    auto q = [&](double v) { return bf16 ? (double)bf16_rne((float)v) : v; };
    const int NP = M_B3 + 1;
    for (int i = 0; i < NP; ++i) G[i] = 0;
    double L = 0;
    MlpRow r;
    double dz2[MH], dz2b[MH], dz1b[MH];
    for (uint64_t s = 0; s < n; ++s) {
        mlp_row(P, X + s * MI, bf16, r);
        const double d = (r.y - T[s]) / (double)n;
        L += 0.5 * (r.y - T[s]) * (r.y - T[s]) / (double)n;
        G[M_B3] += d;
        for (int o = 0; o < MH; ++o) {
            G[M_W3 + o] += r.h2[o] * d;
            dz2[o] = r.z2[o] > 0 ? d * q(P[M_W3 + o]) : 0.0;
            G[M_B2 + o] += dz2[o];
            dz2b[o] = q(dz2[o]);
        }
        for (int i = 0; i < MH; ++i) {
            double a = 0;
            for (int o = 0; o < MH; ++o) a += dz2b[o] * q(P[M_W2 + i * MH + o]);
            const double dz1 = r.z1[i] > 0 ? a : 0.0;
            G[M_B1 + i] += dz1;
            dz1b[i] = q(dz1);
        }
        for (int i = 0; i < MH; ++i)
            for (int o = 0; o < MH; ++o) G[M_W2 + i * MH + o] += r.h1[i] * dz2b[o];
        for (int i = 0; i < MI; ++i)
            for (int o = 0; o < MH; ++o) G[M_W1 + i * MH + o] += r.xb[i] * dz1b[o];
    }
    if (loss) *loss = L;
}

}  // extern "C"

/* ======================================================================== */
/* Scaled mining: oracle_mine_fast                                          */
/*                                                                          */
/* The same results as oracle_mine -- every level's candidates, filter      */
/* bounds and verdicts, row counts, participation numerators, PI bits and   */
/* instance tables in the reference's row order -- organised so that        */
/* 10^7-10^8 points finish in seconds on a multicore host.  It is the timed */
/* CPU baseline at full workload sizes and the source of the full-size      */
/* parity fixtures; tests/test_cpu_oracle.py checks it against oracle_mine  */
/* (the literal restatement) and against the reference's golden vectors.    */
/*                                                                          */
/* What changes is the order of work, not the rules:                        */
/*  - bucketing sorts (cell, id) pairs in parallel and keeps occupied cells  */
/*    only, with each cell's reference-neighbour cells (the visit order of   */
/*    DeviceProcess_Kernel.h:24-32) and its geometric 3x3 cells precomputed; */
/*  - the neighbour relation N+(a) = {b : feat(b) > feat(a), refadj(a->b),  */
/*    sq(a,b) <= R^2} is evaluated once, each list ordered by (feature,     */
/*    visit order, id): the slice of one feature is exactly the sequence    */
/*    degree2TableSlotCounter_Kernel (Kernel.h:12-55) and the level-k       */
/*    kernels (Kernel.h:255-385) walk for an anchor;                        */
/*  - the quad filter (Kernel.h:469-509) tests 2x2 quads with per-cell      */
/*    feature bitsets; pairs are bounded cell by cell (a cell Z is in U_c   */
/*    when one of its quads holds both members; the member in Z is in all   */
/*    of them), larger candidates from the quads of their rarest member's   */
/*    cells, each cell of U_c counted once;                                 */
/*  - participation numerators are counted from per-member bitsets with the  */
/*    window rule of getParticipationIndex (DeviceProcess.cu:108-132):       */
/*    k = 2: num0 = |P0 & [0, L0-1]|, num1 = |P1 \ {0}| + [0 in P1 or L0 in  */
/*    P0]; k >= 3: num0 = |P0 & [0, L0-1]|, num_j = [L_{j-1} in P_{j-1}] +   */
/*    |P_j & [0, L_j-1]| (L_j = n_j - 1);                                   */
/*  - Apriori checks subsets in a hash set instead of a linear scan          */
/*    (colocationFinder.cpp:618-634), with the same breaks.                 */
/* ======================================================================== */

namespace {

struct FastData {
    uint64_t n = 0;
    uint32_t F = 0;
    const float* x = nullptr;
    const float* y = nullptr;
    const uint32_t* feat = nullptr;
    std::vector<uint32_t> fstart, fcount;
    oracle_grid g{};
    float R2 = 0.0f, thr = 0.0f;
    std::vector<uint64_t> cellOf;     /* per point */
    std::vector<uint32_t> order;      /* point ids sorted by (cell, id) */
    std::vector<uint64_t> ckey;       /* occupied cells, ascending */
    std::vector<uint64_t> crun;       /* M + 1: first run of each cell */
    std::vector<uint32_t> rfeat, rcnt;
    std::vector<uint64_t> rstart;     /* first position in `order` */
    std::vector<int32_t> nb9;         /* 9 per cell: reference neighbour cells in visit order, -1 none */
    std::vector<int32_t> g9;          /* 9 per cell: geometric 3x3 (dy major), -1 none */
    uint32_t W = 0;                   /* 64-bit words per feature bitset */
    std::vector<uint64_t> cbits;      /* M * W */
    std::vector<uint64_t> fcell_off;  /* F + 1 */
    std::vector<uint32_t> fcell;      /* occupied cells holding each feature */
    std::vector<uint64_t> nboff;      /* n + 1: N+(a) */
    std::vector<uint32_t> nbv;
    std::vector<uint64_t> act_off;    /* F + 1: anchors with a non-empty N+, by feature */
    std::vector<uint32_t> act;
    const uint64_t* res_keys = nullptr;
    const uint8_t* res_le = nullptr;
    uint64_t nres = 0;
    mutable std::atomic<uint64_t> unresolved{0};

    bool near(uint32_t a, uint32_t b) const {   /* Data::near */
        SqDecision dc = sq_decide(x[a], y[a], x[b], y[b], R2);
        if (!dc.ambiguous) return dc.le;
        uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
        const uint64_t* it = std::lower_bound(res_keys, res_keys + nres, key);
        if (it != res_keys + nres && *it == key) return res_le[it - res_keys] != 0;
        unresolved.fetch_add(1, std::memory_order_relaxed);
        return dc.le;
    }
    int64_t cell_index(uint64_t cell) const {
        auto it = std::lower_bound(ckey.begin(), ckey.end(), cell);
        return (it != ckey.end() && *it == cell) ? (int64_t)(it - ckey.begin()) : -1;
    }
    uint32_t count(uint32_t ci, uint32_t f) const {
        const uint32_t* b = rfeat.data() + crun[ci];
        const uint32_t* e = rfeat.data() + crun[ci + 1];
        const uint32_t* it = std::lower_bound(b, e, f);
        return (it != e && *it == f) ? rcnt[it - rfeat.data()] : 0u;
    }
    /* [lo, hi) of the entries of feature f in N+(a) */
    void slice(uint32_t a, uint32_t f, uint64_t* lo, uint64_t* hi) const {
        const uint32_t* b = nbv.data() + nboff[a];
        const uint32_t* e = nbv.data() + nboff[a + 1];
        const uint32_t* l = std::lower_bound(b, e, f, [&](uint32_t id, uint32_t v) { return feat[id] < v; });
        const uint32_t* h = std::upper_bound(l, e, f, [&](uint32_t v, uint32_t id) { return v < feat[id]; });
        *lo = (uint64_t)(l - nbv.data());
        *hi = (uint64_t)(h - nbv.data());
    }
};

int build_fast(FastData& d, const float* x, const float* y, const uint32_t* feat, uint64_t n, uint32_t F,
               const float bounds[4], float R, float thr) {
    d.n = n;
    d.F = F;
    d.x = x;
    d.y = y;
    d.feat = feat;
    d.thr = thr;
    d.R2 = R * R;                        /* colocationFinder.cpp:73 */
    if (make_grid(bounds[0], bounds[1], bounds[2], bounds[3], R, &d.g)) return 2;
    d.fstart.assign(F, 0);
    d.fcount.assign(F, 0);
    for (uint64_t i = 0; i < n; ++i) {   /* colocationFinder.cpp:168-229 */
        if (feat[i] >= F) return 3;
        if (i > 0 && feat[i] < feat[i - 1]) return 3;
        if (d.fcount[feat[i]] == 0) d.fstart[feat[i]] = (uint32_t)i;
        d.fcount[feat[i]]++;
    }
    for (uint32_t f = 0; f < F; ++f)
        if (d.fcount[f] == 0) return 3;
    const oracle_grid& g = d.g;
    d.cellOf.resize(n);
    std::atomic<int> bad{0};
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        if (!std::isfinite(x[i]) || !std::isfinite(y[i])) {
            bad.store(4);
            continue;
        }
        d.cellOf[i] = cell_of(g, x[i], y[i]);
        if (d.cellOf[i] >= g.total_cells) bad.store(4);
    }
    if (bad.load()) return bad.load();
    /* the stable sort by cell of DeviceProcess.cu:342 = sort by (cell, id) */
    struct Key {
        uint64_t cell;
        uint32_t id, f;
    };
    std::vector<Key> keys(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) keys[i] = {d.cellOf[i], (uint32_t)i, feat[i]};
    auto by_cell = [](const Key& a, const Key& b) { return a.cell < b.cell || (a.cell == b.cell && a.id < b.id); };
#ifdef _OPENMP
    __gnu_parallel::sort(keys.begin(), keys.end(), by_cell);
#else
    std::sort(keys.begin(), keys.end(), by_cell);
#endif
    d.order.resize(n);
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)n; ++p) d.order[p] = keys[p].id;
    /* occupied cells and (cell, feature) runs: ids ascend within a cell, so
     * features do too and each run is contiguous */
    for (uint64_t p = 0; p < n; ++p) {
        const uint64_t cell = keys[p].cell;
        const bool new_cell = p == 0 || keys[p - 1].cell != cell;
        if (new_cell) {
            d.ckey.push_back(cell);
            d.crun.push_back(d.rfeat.size());
        }
        if (new_cell || keys[p - 1].f != keys[p].f) {
            d.rfeat.push_back(keys[p].f);
            d.rstart.push_back(p);
            d.rcnt.push_back(0);
        }
        d.rcnt.back()++;
    }
    d.crun.push_back(d.rfeat.size());
    std::vector<Key>().swap(keys);
    const uint64_t M = d.ckey.size();
    if (M >= (1ull << 31)) return 6;
    d.nb9.assign(M * 9, -1);
    d.g9.assign(M * 9, -1);
    /* geometric 3x3 by walking the grid rows: cells of one row ascend in x,
     * so each neighbouring row is scanned once per row */
    std::vector<uint64_t> rowy, rowb;   /* occupied rows: y and first cell */
    {
        std::vector<uint64_t> cy(M);
#pragma omp parallel for schedule(static)
        for (int64_t ci = 0; ci < (int64_t)M; ++ci) cy[ci] = d.ckey[ci] / g.gx;
        for (uint64_t ci = 0; ci < M; ++ci)
            if (ci == 0 || cy[ci] != cy[ci - 1]) {
                rowy.push_back(cy[ci]);
                rowb.push_back(ci);
            }
        rowb.push_back(M);
    }
    const int64_t NR = (int64_t)rowy.size();
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t ri = 0; ri < NR; ++ri) {
        const uint64_t y = rowy[ri];
        int64_t nbr[2] = {ri > 0 && rowy[ri - 1] + 1 == y ? ri - 1 : -1, ri + 1 < NR && rowy[ri + 1] == y + 1 ? ri + 1 : -1};
        uint64_t ptr[2] = {nbr[0] >= 0 ? rowb[nbr[0]] : 0, nbr[1] >= 0 ? rowb[nbr[1]] : 0};
        for (uint64_t ci = rowb[ri]; ci < rowb[ri + 1]; ++ci) {
            const uint64_t x = d.ckey[ci] % g.gx;
            int32_t* o = &d.g9[ci * 9];
            if (ci > rowb[ri] && d.ckey[ci - 1] + 1 == d.ckey[ci]) o[3] = (int32_t)(ci - 1);
            if (ci + 1 < rowb[ri + 1] && d.ckey[ci + 1] == d.ckey[ci] + 1) o[5] = (int32_t)(ci + 1);
            o[4] = (int32_t)ci;
            for (int side = 0; side < 2; ++side) {
                if (nbr[side] < 0) continue;
                const uint64_t e = rowb[nbr[side] + 1];
                uint64_t& p = ptr[side];
                while (p < e && d.ckey[p] % g.gx + 1 < x) ++p;     /* first cell with x' >= x - 1 */
                for (uint64_t q = p; q < e && d.ckey[q] % g.gx <= x + 1; ++q)
                    o[(side ? 6 : 0) + (int)(d.ckey[q] % g.gx + 1 - x)] = (int32_t)q;
            }
        }
    }
    /* the reference's neighbour cells in visit order: the geometric entry
     * when the visited id is one, a search otherwise (the column-wrap cases) */
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t ci = 0; ci < (int64_t)M; ++ci) {
        int s = 0;
        const int64_t cx = (int64_t)(d.ckey[ci] % g.gx), cy = (int64_t)(d.ckey[ci] / g.gx);
        for_neighbor_cells(g, d.ckey[ci], [&](uint64_t nc) {
            const int64_t dx = (int64_t)(nc % g.gx) - cx, dy = (int64_t)(nc / g.gx) - cy;
            d.nb9[ci * 9 + s++] = (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1) ? d.g9[ci * 9 + (dy + 1) * 3 + (dx + 1)]
                                                                              : (int32_t)d.cell_index(nc);
        });
    }
    d.W = (F + 63) / 64;
    d.cbits.assign(M * d.W, 0);
    d.fcell_off.assign(F + 1, 0);
    for (uint64_t ci = 0; ci < M; ++ci)
        for (uint64_t r = d.crun[ci]; r < d.crun[ci + 1]; ++r) {
            d.cbits[ci * d.W + d.rfeat[r] / 64] |= 1ull << (d.rfeat[r] % 64);
            d.fcell_off[d.rfeat[r] + 1]++;
        }
    for (uint32_t f = 0; f < F; ++f) d.fcell_off[f + 1] += d.fcell_off[f];
    d.fcell.resize(d.fcell_off[F]);
    {
        std::vector<uint64_t> cur(d.fcell_off.begin(), d.fcell_off.end() - 1);
        for (uint64_t ci = 0; ci < M; ++ci)
            for (uint64_t r = d.crun[ci]; r < d.crun[ci + 1]; ++r) d.fcell[cur[d.rfeat[r]]++] = (uint32_t)ci;
    }
    return 0;
}

/* N+(a) for every point (the neighbour tests of Kernel.h:12-55 / 255-316,
 * evaluated once).  Count pass, offsets, fill pass; each list is then ordered
 * by feature, keeping the visit order within a feature. */
void join_fast(FastData& d) {
    const uint64_t n = d.n, M = d.ckey.size();
    std::vector<uint32_t> cnt(n, 0);
    auto walk = [&](uint64_t ci, uint32_t a, uint32_t fa, auto&& emit) {
        for (int s = 0; s < 9; ++s) {
            const int32_t nc = d.nb9[ci * 9 + s];
            if (nc < 0) continue;
            const uint32_t* fb = d.rfeat.data() + d.crun[nc];
            const uint32_t* fe = d.rfeat.data() + d.crun[nc + 1];
            for (const uint32_t* it = std::upper_bound(fb, fe, fa); it != fe; ++it) {
                const uint64_t r = (uint64_t)(it - d.rfeat.data());
                for (uint64_t p = d.rstart[r]; p < d.rstart[r] + d.rcnt[r]; ++p) {
                    const uint32_t b = d.order[p];
                    if (d.near(a, b)) emit(b);
                }
            }
        }
    };
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t ci = 0; ci < (int64_t)M; ++ci)
        for (uint64_t r = d.crun[ci]; r < d.crun[ci + 1]; ++r)
            for (uint64_t p = d.rstart[r]; p < d.rstart[r] + d.rcnt[r]; ++p) {
                const uint32_t a = d.order[p];
                uint32_t c = 0;
                walk((uint64_t)ci, a, d.rfeat[r], [&](uint32_t) { ++c; });
                cnt[a] = c;
            }
    d.nboff.assign(n + 1, 0);
    for (uint64_t a = 0; a < n; ++a) d.nboff[a + 1] = d.nboff[a] + cnt[a];
    d.nbv.resize(d.nboff[n]);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t ci = 0; ci < (int64_t)M; ++ci)
        for (uint64_t r = d.crun[ci]; r < d.crun[ci + 1]; ++r)
            for (uint64_t p = d.rstart[r]; p < d.rstart[r] + d.rcnt[r]; ++p) {
                const uint32_t a = d.order[p];
                if (!cnt[a]) continue;
                uint32_t* out = d.nbv.data() + d.nboff[a];
                uint32_t w = 0;
                walk((uint64_t)ci, a, d.rfeat[r], [&](uint32_t b) { out[w++] = b; });
                std::stable_sort(out, out + w, [&](uint32_t u, uint32_t v) { return d.feat[u] < d.feat[v]; });
            }
    d.act_off.assign(d.F + 1, 0);
    for (uint64_t a = 0; a < n; ++a)
        if (cnt[a]) {
            d.act.push_back((uint32_t)a);
            d.act_off[d.feat[a] + 1]++;
        }
    for (uint32_t f = 0; f < d.F; ++f) d.act_off[f + 1] += d.act_off[f];
}

inline uint64_t popc_prefix(const std::vector<uint64_t>& bits, uint64_t nbits) {   /* bits [0, nbits) */
    uint64_t s = 0, w = nbits / 64;
    for (uint64_t i = 0; i < w; ++i) s += (uint64_t)__builtin_popcountll(bits[i]);
    if (nbits % 64) s += (uint64_t)__builtin_popcountll(bits[w] & ((1ull << (nbits % 64)) - 1));
    return s;
}
inline bool bit_of(const std::vector<uint64_t>& bits, uint64_t i) { return (bits[i / 64] >> (i % 64)) & 1u; }
inline void set_bit_atomic(std::vector<uint64_t>& bits, uint64_t i) {
    __atomic_fetch_or(&bits[i / 64], 1ull << (i % 64), __ATOMIC_RELAXED);
}

/* The window sums of getParticipationIndex (DeviceProcess.cu:108-132) from
 * per-member participation bitsets (see the section comment), then the
 * float ratio and strict-< minimum starting at 1.0f. */
void numerators_fast(const FastData& d, const uint32_t* c, uint32_t k, const std::vector<std::vector<uint64_t>>& P,
                     uint64_t* num, float* pi_out, uint32_t* argmin_out) {
    for (uint32_t j = 0; j < k; ++j) {
        const uint64_t nj = d.fcount[c[j]];
        const uint64_t within = popc_prefix(P[j], nj - 1);   /* P_j & [0, L_j - 1] */
        if (j == 0) {
            num[j] = within;
        } else if (k == 2) {
            const uint64_t all = popc_prefix(P[1], nj);
            const bool zero = bit_of(P[1], 0);
            num[j] = (all - (zero ? 1 : 0)) + ((zero || bit_of(P[0], d.fcount[c[0]] - 1)) ? 1 : 0);
        } else {
            num[j] = (bit_of(P[j - 1], d.fcount[c[j - 1]] - 1) ? 1 : 0) + within;
        }
    }
    float PI = 1.0f;
    uint32_t am = 0;
    for (uint32_t j = 0; j < k; ++j) {
        float pr = (float)num[j] / (float)d.fcount[c[j]];
        if (pr < PI) {
            PI = pr;
            am = j;
        }
    }
    *pi_out = PI;
    *argmin_out = am;
}

/* threshold_Kernel (Kernel.h:545-573), as threshold_pass */
bool threshold_fast(const FastData& d, const uint32_t* c, uint32_t k, const uint64_t* ub) {
    float pi0 = 1.0f;
    for (uint32_t j = 0; j < k; ++j) {
        float pr = (float)((double)ub[j] / (double)(float)d.fcount[c[j]]);
        if (j == 0) pi0 = pr;
        else if (pi0 > pr) pi0 = pr;
    }
    return pi0 >= d.thr;
}

/* Valid quads of cell ci (bx in [0, gx-2], by in [0, gy-2]) as the four
 * positions of its geometric 3x3 they cover; fn(cells[4]) per quad. */
template <class Fn>
inline void for_quads(const FastData& d, uint64_t ci, Fn&& fn) {
    const oracle_grid& g = d.g;
    const int64_t cx = (int64_t)(d.ckey[ci] % g.gx), cy = (int64_t)(d.ckey[ci] / g.gx);
    for (int oy = -1; oy <= 0; ++oy)
        for (int ox = -1; ox <= 0; ++ox) {
            const int64_t bx = cx + ox, by = cy + oy;
            if (bx < 0 || by < 0 || bx > (int64_t)g.gx - 2 || by > (int64_t)g.gy - 2) continue;
            int32_t q[4];
            for (int yy = 0; yy < 2; ++yy)
                for (int xx = 0; xx < 2; ++xx) q[yy * 2 + xx] = d.g9[ci * 9 + (oy + yy + 1) * 3 + (ox + xx + 1)];
            fn(q);
        }
}

/* Degree-2 bounds for all pairs i < j (generation order of
 * colocationFinder.cpp:75-82), cell by cell. */
void filter_pairs_fast(const FastData& d, std::vector<uint64_t>& ub) {
    const uint32_t F = d.F, W = d.W;
    const uint64_t C = (uint64_t)F * (F - 1) / 2;
    auto idx = [F](uint64_t i, uint64_t j) { return i * (2ull * F - i - 1) / 2 + (j - i - 1); };
    ub.assign(C * 2, 0);
    const uint64_t M = d.ckey.size();
#pragma omp parallel
    {
        std::vector<uint64_t> loc(C * 2, 0);
        std::vector<uint64_t> Q(W);
#pragma omp for schedule(dynamic, 4096)
        for (int64_t ci = 0; ci < (int64_t)M; ++ci) {
            std::fill(Q.begin(), Q.end(), 0);
            bool any = false;
            for_quads(d, (uint64_t)ci, [&](const int32_t* q) {
                any = true;
                for (int t = 0; t < 4; ++t)
                    if (q[t] >= 0)
                        for (uint32_t w = 0; w < W; ++w) Q[w] |= d.cbits[(uint64_t)q[t] * W + w];
            });
            if (!any) continue;
            for (uint64_t r = d.crun[ci]; r < d.crun[ci + 1]; ++r) {
                const uint32_t i = d.rfeat[r];
                const uint64_t c = d.rcnt[r];
                for (uint32_t w = 0; w < W; ++w)
                    for (uint64_t m = Q[w]; m; m &= m - 1) {
                        const uint32_t j = w * 64 + (uint32_t)__builtin_ctzll(m);
                        if (j == i) continue;
                        if (i < j) loc[idx(i, j) * 2 + 0] += c;
                        else loc[idx(j, i) * 2 + 1] += c;
                    }
            }
        }
#pragma omp critical
        for (uint64_t t = 0; t < C * 2; ++t) ub[t] += loc[t];
    }
}

/* Degree >= 3 bound of one candidate (filter_sparse's rule), from the quads
 * of the cells of its member with the fewest cells.  stamp: per-thread cell
 * marks, gen: a value not yet used in it. */
void filter_cand_fast(const FastData& d, const uint32_t* c, uint32_t k, uint64_t* ub, std::vector<uint32_t>& stamp,
                      uint32_t gen) {
    const uint32_t m = k < 8 ? k : 8, W = d.W;
    for (uint32_t j = 0; j < k; ++j) ub[j] = 0;
    std::vector<uint64_t> mb(W, 0);
    uint32_t drv = c[0];
    for (uint32_t j = 0; j < m; ++j) {
        mb[c[j] / 64] |= 1ull << (c[j] % 64);
        if (d.fcell_off[c[j] + 1] - d.fcell_off[c[j]] < d.fcell_off[drv + 1] - d.fcell_off[drv]) drv = c[j];
    }
    for (uint64_t t = d.fcell_off[drv]; t < d.fcell_off[drv + 1]; ++t)
        for_quads(d, d.fcell[t], [&](const int32_t* q) {
            for (uint32_t w = 0; w < W; ++w) {
                uint64_t v = 0;
                for (int s = 0; s < 4; ++s)
                    if (q[s] >= 0) v |= d.cbits[(uint64_t)q[s] * W + w];
                if ((v & mb[w]) != mb[w]) return;
            }
            for (int s = 0; s < 4; ++s) {
                if (q[s] < 0 || stamp[q[s]] == gen) continue;
                stamp[q[s]] = gen;
                for (uint32_t j = 0; j < m; ++j) ub[j] += d.count((uint32_t)q[s], c[j]);
            }
        });
}

struct FastRef {
    uint64_t rows = 0;
    std::vector<uint32_t> slots;   /* per anchor (k = 2, active anchors of c[0]) or parent row */
};

/* Degree-2 count (degree2TableSlotCounter_Kernel, Kernel.h:12-55) and PI. */
FastRef refine2_fast(const FastData& d, const uint32_t* c, uint64_t* num, float* pi, uint32_t* am) {
    FastRef out;
    const uint32_t f0 = c[0], f1 = c[1];
    std::vector<std::vector<uint64_t>> P(2);
    P[0].assign(d.fcount[f0] / 64 + 1, 0);
    P[1].assign(d.fcount[f1] / 64 + 1, 0);
    const uint64_t a0 = d.act_off[f0], a1 = d.act_off[f0 + 1];
    out.slots.assign(a1 - a0, 0);
    for (uint64_t t = a0; t < a1; ++t) {
        const uint32_t a = d.act[t];
        uint64_t lo, hi;
        d.slice(a, f1, &lo, &hi);
        if (lo == hi) continue;
        out.slots[t - a0] = (uint32_t)(hi - lo);
        out.rows += hi - lo;
        P[0][(a - d.fstart[f0]) / 64] |= 1ull << ((a - d.fstart[f0]) % 64);
        for (uint64_t e = lo; e < hi; ++e) {
            const uint32_t b = d.nbv[e] - d.fstart[f1];
            P[1][b / 64] |= 1ull << (b % 64);
        }
    }
    numerators_fast(d, c, 2, P, num, pi, am);
    return out;
}

/* degree2TableGenerator_Kernel (Kernel.h:56-100): rows (a, b) by anchor, then slice order. */
std::vector<uint32_t> fill2_fast(const FastData& d, const uint32_t* c, const FastRef& ref) {
    std::vector<uint32_t> tab;
    tab.reserve(ref.rows * 2);
    const uint64_t a0 = d.act_off[c[0]];
    for (uint64_t t = 0; t < ref.slots.size(); ++t) {
        if (!ref.slots[t]) continue;
        const uint32_t a = d.act[a0 + t];
        uint64_t lo, hi;
        d.slice(a, c[1], &lo, &hi);
        for (uint64_t e = lo; e < hi; ++e) {
            tab.push_back(a);
            tab.push_back(d.nbv[e]);
        }
    }
    return tab;
}

/* Level k >= 3 count (generalInstanceTableSlotCounter_Kernel, Kernel.h:255-316)
 * over the prefix table, and PI.  par: split the parent rows over threads. */
FastRef refinek_fast(const FastData& d, const uint32_t* c, uint32_t k, const std::vector<uint32_t>& parent, bool par,
                     uint64_t* num, float* pi, uint32_t* am) {
    FastRef out;
    const uint32_t km1 = k - 1, last = c[k - 1];
    const uint64_t prow = parent.size() / km1;
    std::vector<std::vector<uint64_t>> P(k);
    for (uint32_t j = 0; j < k; ++j) P[j].assign(d.fcount[c[j]] / 64 + 1, 0);
    out.slots.assign(prow, 0);
    uint64_t rows = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : rows) if (par)
    for (int64_t t = 0; t < (int64_t)prow; ++t) {
        const uint32_t* r = &parent[(size_t)t * km1];
        uint64_t lo, hi;
        d.slice(r[0], last, &lo, &hi);
        uint32_t cnt = 0;
        for (uint64_t e = lo; e < hi; ++e) {
            const uint32_t b = d.nbv[e];
            bool ok = true;
            for (uint32_t i = 1; i < km1 && ok; ++i)
                if (!d.near(r[i], b)) ok = false;
            if (!ok) continue;
            ++cnt;
            set_bit_atomic(P[km1], b - d.fstart[last]);
        }
        if (cnt)
            for (uint32_t i = 0; i < km1; ++i) set_bit_atomic(P[i], r[i] - d.fstart[c[i]]);
        out.slots[t] = cnt;
        rows += cnt;
    }
    out.rows = rows;
    numerators_fast(d, c, k, P, num, pi, am);
    return out;
}

/* generateInstanceTableGeneral_Kernel (Kernel.h:318-385): parent row order, then slice order. */
std::vector<uint32_t> fillk_fast(const FastData& d, const uint32_t* c, uint32_t k, const std::vector<uint32_t>& parent,
                                 const FastRef& ref, bool par) {
    const uint32_t km1 = k - 1, last = c[k - 1];
    const uint64_t prow = parent.size() / km1;
    std::vector<uint64_t> off(prow + 1, 0);
    for (uint64_t t = 0; t < prow; ++t) off[t + 1] = off[t] + ref.slots[t];
    std::vector<uint32_t> tab(off[prow] * k);
#pragma omp parallel for schedule(dynamic, 1024) if (par)
    for (int64_t t = 0; t < (int64_t)prow; ++t) {
        if (!ref.slots[t]) continue;
        const uint32_t* r = &parent[(size_t)t * km1];
        uint64_t lo, hi, o = off[t] * k;
        d.slice(r[0], last, &lo, &hi);
        for (uint64_t e = lo; e < hi; ++e) {
            const uint32_t b = d.nbv[e];
            bool ok = true;
            for (uint32_t i = 1; i < km1 && ok; ++i)
                if (!d.near(r[i], b)) ok = false;
            if (!ok) continue;
            for (uint32_t i = 0; i < km1; ++i) tab[o++] = r[i];
            tab[o++] = b;
        }
    }
    return tab;
}

struct PatHash {
    size_t operator()(const std::vector<uint32_t>& v) const {
        uint64_t h = 1469598103934665603ull;
        for (uint32_t x : v) h = (h ^ x) * 1099511628211ull;
        return (size_t)h;
    }
};
using PatMap = std::unordered_map<std::vector<uint32_t>, int64_t, PatHash>;

PatMap pattern_index(const std::vector<uint32_t>& list, size_t cnt, uint32_t deg) {
    PatMap m;
    m.reserve(cnt * 2);
    for (size_t i = 0; i < cnt; ++i) {
        std::vector<uint32_t> p(list.begin() + i * deg, list.begin() + (i + 1) * deg);
        m.emplace(std::move(p), (int64_t)i);   /* first occurrence, as getIndex's linear search */
    }
    return m;
}

/* candidateColocationGeneral (colocationFinder.cpp:517-557) with the same
 * breaks as apriori(); subsets are looked up in a hash set. */
std::vector<uint32_t> apriori_fast(const std::vector<uint32_t>& prev, size_t nprev, uint32_t degree) {
    std::vector<uint32_t> cand;
    const uint32_t lastIndex = degree - 2, w = degree - 1;
    PatMap have = pattern_index(prev, nprev, w);
    std::vector<std::vector<uint32_t>> subs;
    for (size_t i = 0; i < nprev; ++i) {
        bool flag = true;
        for (size_t j = i + 1; j < nprev; ++j) {
            for (size_t t = 0; t < lastIndex; ++t)
                if (prev[i * w + t] != prev[j * w + t]) {
                    flag = false;
                    break;
                }
            if (flag && prev[i * w + lastIndex] < prev[j * w + lastIndex]) {
                std::vector<uint32_t> inter(prev.begin() + i * w, prev.begin() + (i + 1) * w);
                inter.push_back(prev[j * w + lastIndex]);
                subsets_lex(inter, subs);
                flag = true;
                for (size_t s = 2; s < degree; ++s) {
                    flag = have.count(subs[s]) > 0;
                    if (!flag) break;
                }
                if (!flag) break;
                cand.insert(cand.end(), inter.begin(), inter.end());
            } else {
                break;
            }
        }
    }
    return cand;
}

}  // namespace

extern "C" {

int oracle_mine_fast(const float* x, const float* y, const uint32_t* feat, uint64_t n, uint32_t nfeat,
                     const float bounds[4], float R, float thr, uint32_t max_k, int threads, int keep_tables,
                     const uint64_t* res_keys, const uint8_t* res_le, uint64_t nres, oracle_result** out) {
    oracle_result* res = new oracle_result();
    *out = res;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    if (n == 0 || nfeat < 2) return res->status = 0;
    using clk = std::chrono::steady_clock;
    auto t0 = clk::now();
    auto lap = [&](int ph) {
        auto t1 = clk::now();
        res->phase_ms[ph] += std::chrono::duration<double, std::milli>(t1 - t0).count();
        t0 = t1;
    };
    FastData d;
    int st = build_fast(d, x, y, feat, n, nfeat, bounds, R, thr);
    if (st) return res->status = st;
    lap(0);
    d.res_keys = res_keys;
    d.res_le = res_le;
    d.nres = res_keys ? nres : 0;
    struct Tally {
        oracle_result* r;
        const FastData& d;
        ~Tally() { r->unresolved = d.unresolved.load(); }
    } tally{res, d};
    join_fast(d);
    lap(1);
    const uint64_t M = d.ckey.size();
    const uint64_t kParRows = 1u << 16;   /* tables at least this long split their rows over threads */

    std::vector<uint32_t> cands;
    for (uint32_t i = 0; i + 1 < nfeat; ++i)       /* colocationFinder.cpp:75-82 */
        for (uint32_t j = i + 1; j < nfeat; ++j) {
            cands.push_back(i);
            cands.push_back(j);
        }
    uint32_t k = 2;
    std::vector<uint32_t> prev, parentList;
    std::vector<size_t> prevIdx;
    std::vector<std::vector<uint32_t>> parentTables;
    while (true) {
        const size_t C = cands.size() / k;
        OLevel L;
        L.k = k;
        L.cand = cands;
        L.ub.assign(C * k, 0);
        L.num.assign(C * k, 0);
        L.rows.assign(C, 0);
        L.pass.assign(C, 0);
        L.prevalent.assign(C, 0);
        L.pi.assign(C, -1.0f);
        L.argmin.assign(C, 0);
        /* filter */
        if (k == 2) {
            filter_pairs_fast(d, L.ub);
        } else {
#pragma omp parallel
            {
                std::vector<uint32_t> stamp(M, 0);
                uint32_t gen = 0;
#pragma omp for schedule(dynamic, 1)
                for (int64_t c = 0; c < (int64_t)C; ++c) filter_cand_fast(d, &cands[c * k], k, &L.ub[c * k], stamp, ++gen);
            }
        }
        for (size_t c = 0; c < C; ++c) L.pass[c] = threshold_fast(d, &cands[c * k], k, &L.ub[c * k]) ? 1 : 0;
        lap(2);
        /* refinement of the candidates that pass */
        std::vector<FastRef> refs(C);
        std::vector<int64_t> parent_of(C, -1);
        PatMap parentIdx;
        if (k > 2) parentIdx = pattern_index(parentList, parentList.size() / (k - 1), k - 1);
        std::vector<size_t> todo;
        for (size_t c = 0; c < C; ++c) {
            if (!L.pass[c]) continue;
            if (k > 2) {
                std::vector<uint32_t> p(cands.begin() + c * k, cands.begin() + c * k + (k - 1));
                auto it = parentIdx.find(p);
                if (it == parentIdx.end()) return res->status = 5;
                parent_of[c] = it->second;
            }
            todo.push_back(c);
        }
        auto refine_one = [&](size_t c, bool par) {
            const uint32_t* cc = &cands[c * k];
            if (k == 2)
                refs[c] = refine2_fast(d, cc, &L.num[c * k], &L.pi[c], &L.argmin[c]);
            else
                refs[c] = refinek_fast(d, cc, k, parentTables[parent_of[c]], par, &L.num[c * k], &L.pi[c],
                                       &L.argmin[c]);
            L.rows[c] = refs[c].rows;
        };
        auto big = [&](size_t c) { return k > 2 && parentTables[parent_of[c]].size() / (k - 1) >= kParRows; };
        for (size_t c : todo)
            if (big(c)) refine_one(c, true);
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t t = 0; t < (int64_t)todo.size(); ++t)
            if (!big(todo[t])) refine_one(todo[t], false);
        lap(3);
        prev.clear();
        prevIdx.clear();
        for (size_t c : todo)
            if (!(L.pi[c] < thr)) {                      /* cpp:335, cpp:827 */
                L.prevalent[c] = 1;
                prev.insert(prev.end(), &cands[c * k], &cands[c * k] + k);
                prevIdx.push_back(c);
            }
        const size_t P = prevIdx.size();
        std::vector<uint32_t> next;
        if (P > 0 && (max_k == 0 || k + 1 <= max_k) && k + 1 <= nfeat) next = apriori_fast(prev, P, k + 1);
        const size_t Cn = next.size() / (k + 1);
        lap(5);
        /* tables of the prevalent patterns that prefix a next candidate */
        std::vector<uint8_t> need(P, 0);
        {
            PatMap pidx = pattern_index(prev, P, k);
            for (size_t i = 0; i < Cn; ++i) {
                std::vector<uint32_t> p(next.begin() + i * (k + 1), next.begin() + i * (k + 1) + k);
                auto it = pidx.find(p);
                if (it != pidx.end()) need[it->second] = 1;
            }
        }
        std::vector<std::vector<uint32_t>> newTables(P);
        L.tables.assign(keep_tables ? C : 0, {});
        L.has_table.assign(C, 0);
        auto fill_one = [&](size_t p, bool par) {
            const size_t c = prevIdx[p];
            const uint32_t* cc = &cands[c * k];
            newTables[p] = k == 2 ? fill2_fast(d, cc, refs[c]) : fillk_fast(d, cc, k, parentTables[parent_of[c]], refs[c], par);
        };
        for (size_t p = 0; p < P; ++p)
            if (need[p] && big(prevIdx[p])) fill_one(p, true);
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t p = 0; p < (int64_t)P; ++p)
            if (need[p] && !big(prevIdx[p])) fill_one((size_t)p, false);
        for (size_t p = 0; p < P; ++p) {
            if (!need[p]) continue;
            const size_t c = prevIdx[p];
            L.has_table[c] = 1;
            if (keep_tables) L.tables[c] = newTables[p];
        }
        lap(4);
        res->levels.push_back(std::move(L));
        if (Cn == 0) break;
        parentTables.swap(newTables);
        parentList = prev;
        cands = next;
        k++;
    }
    return res->status = 0;
}

}  // extern "C"
