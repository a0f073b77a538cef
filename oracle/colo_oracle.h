/*
 * colo_oracle.h -- CPU oracle for the colocation-mining hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain C++ restatement of the
 * reference implementation's semantics (GPU-ColocationMininig, Codes/).  It
 * exists to check the CUDA product path and to serve as the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py (its
 * cpu_baseline leg and its --impl reference arm) may load it.  The product
 * library never links, loads or calls it.
 *
 * Every function in colo_oracle.cpp names the reference file:line whose
 * behaviour it restates.
 */
#ifndef COLO_ORACLE_H
#define COLO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_result oracle_result;

/* Grid exactly as setGrid (colocationFinder.cpp:102-126) derives it. */
typedef struct {
    float min_x, min_y, max_x, max_y_ext, cell_width;
    uint32_t gx, gy;
    uint64_t total_cells;
    int32_t compat32;     /* 1: the reference's 32-bit cell arithmetic is exact */
} oracle_grid;

/* Derive the grid; returns 0 on success, nonzero for a grid the reference
 * cannot represent (R<=0, empty extent, >2^32 columns). */
int oracle_make_grid(float min_x, float min_y, float max_x, float max_y, float R,
                     oracle_grid* g);

/* Per-point cell ids (Codes/DeviceProcess_Kernel.h:615-625).  Returns the
 * number of points whose cell falls outside [0, total_cells). */
uint64_t oracle_cell_ids(const oracle_grid* g, const float* x, const float* y,
                         uint64_t n, uint64_t* cell_out);

/* Squared distance of Codes/Utility_Inline.h:25-33 as the device computes it
 * away from float rounding midpoints: the correctly rounded float of the
 * exact dx^2 + dy^2. */
float oracle_sqdist(float x1, float y1, float x2, float y2);
/* The comparison sq <= R2 as the device makes it; *ambiguous = 1 when the
 * exact sum lies so close to a float rounding midpoint that the device's
 * rounding could flip it (then the return is the round-to-even guess). */
int oracle_sq_decide(float x1, float y1, float x2, float y2, float R2, int* ambiguous);
/* The same for n pairs; value[i] = correctly rounded squared distance,
 * near_mid[i] = 1 when the exact sum is within the midpoint window. */
void oracle_sq_decide_batch(const float* x1, const float* y1, const float* x2, const float* y2, uint64_t n,
                            float R2, uint8_t* le, uint8_t* ambiguous, float* value, uint8_t* near_mid);
/* Keys (i << 32 | j, i < j, different features) of every ambiguous pair;
 * returns the count, copies up to cap keys (sorted). */
uint64_t oracle_ambiguous_pairs(const float* x, const float* y, const uint32_t* feat, uint64_t n,
                                float R, uint64_t* keys, uint64_t cap);

/* Reference neighbour-cell rule: 1 if cell `nb` is visited from cell `c`
 * (Codes/Utility_Inline.h:35-53 with the stencil loops, e.g.
 * Codes/DeviceProcess_Kernel.h:24-32). */
int oracle_cell_adjacent(const oracle_grid* g, uint64_t c, uint64_t nb);

/* Full mining run.  feat[i] is the 0-based feature index of point i; it must
 * be non-decreasing (the reference requires feature-grouped input,
 * colocationFinder.cpp:168-184).  max_k = 0 means no size cap (the
 * reference has none).  threads <= 0 means all OpenMP threads.
 * keep_tables != 0 keeps every instance table built (small inputs only). */
int oracle_mine(const float* x, const float* y, const uint32_t* feat, uint64_t n,
                uint32_t nfeat, const float bounds[4], float R, float thr,
                uint32_t max_k, int threads, int keep_tables,
                const uint64_t* res_keys, const uint8_t* res_le, uint64_t nres,
                oracle_result** out);

/* The same results as oracle_mine (every level's candidates, bounds,
 * verdicts, rows, numerators, PI bits and tables in the same order),
 * organised for 10^7-10^8 points: parallel bucketing, the neighbour lists
 * evaluated once, bitset quad tests and hashed Apriori subset checks. */
int oracle_mine_fast(const float* x, const float* y, const uint32_t* feat, uint64_t n,
                     uint32_t nfeat, const float bounds[4], float R, float thr,
                     uint32_t max_k, int threads, int keep_tables,
                     const uint64_t* res_keys, const uint8_t* res_le, uint64_t nres,
                     oracle_result** out);

void     oracle_free(oracle_result* r);
/* Wall-clock milliseconds of oracle_mine_fast's phases: bucketing, join,
 * filter, refine, fill, Apriori (zeros for oracle_mine). */
void     oracle_phase_ms(const oracle_result* r, double* ms6);
int      oracle_status(const oracle_result* r);
/* Ambiguous comparisons met without a device outcome in res_keys/res_le
 * (sorted keys as from oracle_ambiguous_pairs; res_le = device sq <= R2). */
uint64_t oracle_unresolved(const oracle_result* r);
uint32_t oracle_num_levels(const oracle_result* r);
uint32_t oracle_level_k(const oracle_result* r, uint32_t li);
uint64_t oracle_level_ncand(const oracle_result* r, uint32_t li);
/* Copies one level's trace.  Arrays are sized ncand*k (cand, ub, num) or
 * ncand (pass, rows, pi, prevalent, argmin).  Any pointer may be NULL. */
void oracle_level_get(const oracle_result* r, uint32_t li, uint32_t* cand,
                      uint64_t* ub, uint8_t* pass, uint64_t* rows, uint64_t* num,
                      float* pi, uint8_t* prevalent, uint32_t* argmin);
/* Instance table of level li, candidate ci (kept only with keep_tables and
 * only for tables the level loop built).  Returns the row count, or
 * UINT64_MAX when absent; copies rows*k u32 row-major into out if non-NULL. */
uint64_t oracle_table(const oracle_result* r, uint32_t li, uint64_t ci, uint32_t* out);

/* Neighbour lists N+(a) = {b : feat(b) > feat(a), cells adjacent, sq <= R^2}
 * in the reference's visiting order (feature, neighbour cell, b).  offs has
 * n+1 entries; returns total entries; fills nbr if non-NULL. */
uint64_t oracle_neighbors(const float* x, const float* y, const uint32_t* feat,
                          uint64_t n, uint32_t nfeat, const float bounds[4], float R,
                          const uint64_t* res_keys, const uint8_t* res_le, uint64_t nres,
                          uint64_t* offs, uint32_t* nbr, uint64_t* n_unresolved);

/* Literal dense-grid filter (Codes/DeviceProcess_Kernel.h:469-509) for small
 * grids: ub[c*k + j] and pass[c].  Used to cross-check the sparse filter. */
int oracle_filter_dense(const float* x, const float* y, const uint32_t* feat, uint64_t n,
                        uint32_t nfeat, const float bounds[4], float R, float thr,
                        const uint32_t* cand, uint64_t ncand, uint32_t k,
                        uint64_t* ub, uint8_t* pass);

/* Apriori candidate generation of level k from the ordered prevalent
 * (k-1)-patterns (colocationFinder.cpp:517-557 with 598-634, 669-679).
 * Returns the number of candidates; out (if non-NULL) receives them. */
uint64_t oracle_apriori(const uint32_t* prev, uint64_t nprev, uint32_t k,
                        uint32_t* out, uint64_t out_cap);

/* Parsing, populateData (colocationFinder.cpp:139-254) and LoadParameter
 * (colocationFinder.cpp:57-74).  oracle_parse_csv returns 0 on success and
 * fills n / nfeat; call again with arrays of that size to copy the data.
 * names receives the feature names joined by '\n' (cap bytes). */
int oracle_parse_csv(const char* path, uint64_t* n, uint32_t* nfeat, float* x, float* y,
                     uint32_t* feat, float bounds[4], char* names, uint64_t names_cap);
int oracle_parse_params(const char* path, float* R, float* thr, uint32_t* filter_flag);

/* Cost model (the CUDA kernels' network): predictions and the gradient of
 * mean 0.5*(y - t)^2 (6337 parameters); bf16 = 1 rounds to BF16 where the
 * kernels do, bf16 = 0 computes exactly in double. */
void oracle_mlp_forward(const float* P, const float* X, uint64_t n, int bf16, double* Y);
void oracle_mlp_grad(const float* P, const float* X, const float* T, uint64_t n, int bf16, double* G,
                     double* loss);

#ifdef __cplusplus
}
#endif
#endif
