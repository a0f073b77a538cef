// colo_batch.h -- device state of one mining batch and the stage launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "colo_internal.h"

namespace colo {

// Host description of one job inside a batch.
struct JobHost {
    JobGrid grid;
    uint64_t p0 = 0, np = 0;     // point range
};

struct Batch {
    cudaStream_t s = 0;
    int sms = 148;
    // sizes
    uint64_t N = 0;              // points
    uint32_t F = 0;              // features (global)
    uint32_t J = 0;              // jobs
    uint32_t W = 1;              // mask words per cell (max local feature count / 32)
    uint32_t Fmax_local = 0;
    uint64_t M = 0;              // occupied cells
    uint64_t Rn = 0;             // (cell, feature) runs
    uint64_t key_bits = 1;
    // host copies of small arrays
    std::vector<JobHost> jobs;
    std::vector<uint32_t> h_fstart, h_fcount, h_fjob;
    std::vector<uint32_t> h_frun_off;   // prefix of the number of runs (occupied cells) per feature
    // points (by id)
    const float* x = nullptr;    // borrowed (dataset device copy)
    const float* y = nullptr;
    DevBuf<uint32_t> fstart, fcount, fjob;
    DevBuf<JobGrid> grids;
    DevBuf<DevFlags> flags;
    // bucketed (sorted by cell key, then id)
    DevBuf<float2> xy;           // coordinates by id, packed (built by the cell-key pass)
    DevBuf<uint32_t> sid, sfeat, scell;   // scell (cell of each sorted point) only when keep_scell
    bool keep_scell = false;              // colo_stage_cells reports each point's cell
    DevBuf<float2> sxy;          // coordinates in cell-sorted order
    // cells
    DevBuf<uint64_t> ckey;
    DevBuf<uint32_t> cstart, crun, cjob;
    uint64_t h2d_points = 0;     // bytes of point data copied to the device for this batch
    uint64_t rows = 0;           // grid rows of all jobs (row table size - 1)
    DevBuf<uint32_t> rowstart;   // per grid row: first occupied cell at or after the row (empty when too large)
    DevBuf<int32_t> nb9;
    DevBuf<uint32_t> cmask;
    DevBuf<uint32_t> nbmask;     // per cell: feature mask of its geometric 3x3 block
    DevBuf<uint32_t> listq, nlistq;   // cells whose 3x3 block has a feature above their lowest own one
    DevBuf<uint32_t> qmask;      // per cell: masks of the 4 quads containing it ([M][4][W])
    // driver lists: for global feature f, the cells whose 3x3 block holds f
    // (nbmask bit), dlist[doff[f] .. doff[f+1]), in no particular order; the
    // level filters test exactly these cells for the candidates f drives
    DevBuf<uint32_t> dlist;
    DevBuf<uint64_t> doff;
    std::vector<uint64_t> h_dcnt;    // cells per feature's list (every feature)
    std::vector<uint64_t> h_doff;    // offsets of the lists filled (features in dlist_have; others empty)
    std::vector<uint8_t> dlist_have; // features whose lists are filled (by the level filters, on demand)
    DevBuf<uint8_t> qfirst;      // per cell: bit q set when it is the first occupied cell of its quad q
    // runs
    DevBuf<uint32_t> rfeat, rstart, rcnt, rcell;
    // neighbourhood run lists: for cell c, the runs of its adjacent cells
    // ordered by (feature, cell), entries above the cell's lowest own feature:
    // nrl_ent[nrl_off[c] .. nrl_off[c+1]), each the run's (first sorted
    // position, point count)
    DevBuf<uint64_t> nrl_off;
    DevBuf<uint2> nrl_ent;
    uint64_t nrl_total = 0;
    // per run: first entry of its cell's list with a higher feature (absolute
    // index), the entries from there to the list's end (run_qn), and the
    // number of target points in them; run_sfx and run_qn are set where run_L > 0
    DevBuf<uint64_t> run_sfx;
    DevBuf<uint32_t> run_qn;
    DevBuf<uint32_t> run_L;
    // neighbour lists N+(a) = nb[nb_beg[a] .. nb_beg[a] + nb_cnt[a]), each in
    // (feature, neighbour cell, id) order; nb_beg[a] is set only where nb_cnt[a] > 0
    DevBuf<uint64_t> nb_beg;
    DevBuf<uint32_t> nb_cnt, nb;
    uint64_t E = 0;              // neighbour entries (UINT64_MAX: still on the device in dE)
    DevBuf<unsigned long long> dE;
    uint64_t nb_cap = 0;         // allocated entries (upper bound in single-pass mode)
    uint64_t join_pairs = 0;     // pair distance evaluations
    uint64_t active_anchors = 0; // anchors whose cell has higher-feature neighbours
    bool join_single = true;     // single pass into per-run upper-bound regions
    int join_group = 8;          // lanes per anchor in the join (autotuned)
    int filter_unit = 32;        // candidates per warp unit in the level filter (autotuned: 8, 16, 32)
    int level_block = 256;       // threads per block of the level kernels (autotuned: 64, 128, 256)
    int level_queue = 0;         // 1: level count/fill kernels as a persistent work queue (autotuned)
    uint32_t test_spin = 0;      // tests only: the sort's look-back gives up after this many polls
    uint64_t filter_items = 0;   // (driver cell, candidate) items of the level filters
};

// colo_bucket.cu
void bucket_points(Batch& b);            // cells, runs, masks, nb9, runs per feature
void build_neighborhoods(Batch& b);      // NRL / NPL
// colo_join.cu
void join_neighbors(Batch& b);           // neighbour CSR
uint64_t neighbor_entries(Batch& b);     // E (waits for the device sum once)
// Level-k candidates of every job from its prevalent (k-1)-patterns (km1
// features each, lexicographic), with each candidate's prefix pattern index;
// a null entry is a job with no next level.  colo_apriori.cu.
void apriori_device(cudaStream_t s, const std::vector<const std::vector<uint32_t>*>& prev, uint32_t km1,
                    std::vector<std::vector<uint32_t>>& out, std::vector<std::vector<uint32_t>>& parent);
// colo_filter.cu
// Driver lists: their sizes are counted by the quad masks' kernel; the lists
// themselves are filled by the level filters for the drivers of their
// candidates (a level whose drivers are not all filled yet fills the union of
// the old and new ones).
// Level-2 upper bounds of every pair of every job: ub2[job_off[j] + lf*Fj + lg] is the
// bound of feature lf's side of pair {lf, lg}.  job_off has J+1 entries.
// Runs on stream s (no wait at the end).
void filter_pairs(Batch& b, DevBuf<uint32_t>& ub2, std::vector<uint64_t>& job_off, cudaStream_t s);
// Level-k upper bounds for host candidates cand[c*k + j] (global features) of
// jobs job[c]: d_ub[c*k + j] (zeroed by the caller).  d_stats (optional,
// zeroed, 2 per candidate): full quads and cells of U_c.
// d_cand (optional): the same candidates already on the device.
void filter_level(Batch& b, const uint32_t* h_cand, const uint32_t* h_job, uint64_t ncand, uint32_t k,
                  uint32_t* d_ub, unsigned long long* d_stats, const uint32_t* d_cand = nullptr);

// colo_level.cu --------------------------------------------------------------
// One candidate's view for the level kernels.
struct CandDesc {
    const uint32_t* parent;      // column-major parent table (k-1 columns); nullptr: implicit (k=2)
    uint64_t prow;               // parent rows (k=2: anchors of member 0)
    uint64_t pstride;            // parent column stride (>= prow)
    uint32_t m[kMaxK];           // member features
    uint32_t* slots;             // per parent row counts (count pass output)
    const uint64_t* offs;        // per parent row output offsets (fill pass input)
    uint32_t* out;               // column-major output table (k columns, rows = total)
    uint64_t out_rows;           // rows of the output table (column stride)
    uint64_t out_cap;            // capacity (single-pass mode; also its column stride)
    unsigned long long* rows;    // count pass: rows of this candidate (atomic sum)
    uint32_t* bitmap;            // member bitmaps: member j's words start at bm_base plus
    uint64_t bm_base;            // the sum over i < j of ceil(fcount[m[i]] / 32)
    uint32_t job;
    uint32_t k;
};

struct LevelWork {
    const CandDesc* cands;       // device array
    const uint64_t* chunk_off;   // device: prefix of 32-row chunks per candidate (ncand+1)
    uint64_t ncand;
    uint64_t nchunks;
    unsigned long long* items;   // optional: sum of candidate-slice lengths examined
    unsigned long long* chunk_status = nullptr;   // single pass: nchunks words, zeroed
    unsigned long long* ticket = nullptr;         // single pass: chunk ticket counter, zeroed
};

// count pass: slots + bitmaps; fill pass: rows; single pass: slots +
// bitmaps + rows at their count-and-fill positions (overflow recorded per
// candidate; a look-back that waits too long sets the batch's timeout flag).
void level_count(Batch& b, const LevelWork& w, uint32_t k);
void level_fill(Batch& b, const LevelWork& w, uint32_t k);
void level_single(Batch& b, const LevelWork& w, uint32_t k, uint32_t* d_overflow);
// Participation statistics per candidate and member: [A, last, first, full]
// (A = set bits in [0, n-2]), added into d_stats, which must be zero.
void level_pi(Batch& b, const CandDesc* d_cands, uint64_t ncand, uint32_t k, uint64_t* d_stats);

// Squared-distance evaluation of the reference expression for n pairs; with
// `within`, also the kernels' decision ref_within(...) for threshold R2.
void eval_sqdist(const float* x1, const float* y1, const float* x2, const float* y2, uint64_t n,
                 float* out, cudaStream_t s, float R2 = 0.0f, uint8_t* within = nullptr);

}  // namespace colo
