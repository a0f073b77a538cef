/*
 * colo.h -- C ABI of the GB300 colocation-mining library (libcolo.so).
 *
 * The library replaces the GPU path of GPU-ColocationMininig (Codes/): grid
 * bucketing, the cell-pair spatial join, the cell-aggregate upper-bound
 * filter, level-wise instance tables and the participation index.  Every
 * entry point takes plain pointers and sizes, returns a colo_status, never
 * prints and never exits.  A context owns one CUDA stream on one device and
 * all device memory it allocates; use one context per host thread.
 *
 * Each declaration names the reference interface it replaces (paths inside
 * the reference project).
 */
#ifndef COLO_H
#define COLO_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    COLO_OK = 0,
    COLO_ERR_ARG = 1,        /* bad argument (NULL, size, out of range) */
    COLO_ERR_IO = 2,         /* file cannot be opened / written */
    COLO_ERR_PARSE = 3,      /* malformed config, parameter or CSV file */
    COLO_ERR_INPUT = 4,      /* data the reference cannot represent (point outside the grid, non-finite) */
    COLO_ERR_CUDA = 5,       /* CUDA runtime error (message in colo_last_error) */
    COLO_ERR_NOMEM = 6,      /* device or host allocation failed */
    COLO_ERR_TIMEOUT = 7,    /* a bounded device wait gave up */
    COLO_ERR_CAPACITY = 8,   /* a fixed-size buffer is too small for the request */
    COLO_ERR_NO_DEVICE = 9,  /* no CUDA device / library not usable */
    COLO_ERR_INTERNAL = 10
} colo_status;

/* Execution form of the level loop. */
typedef enum {
    COLO_MODE_PLAIN = 0,     /* per-candidate count -> PI -> fill launches (two-pass) */
    COLO_MODE_BATCHED = 1,   /* one persistent work-queue launch per level phase, CUDA graph */
    COLO_MODE_LEARNED = 2    /* batched + cost-model presized single-pass fill with exact fallback */
} colo_mode;

typedef struct colo_ctx colo_ctx;
typedef struct colo_dataset colo_dataset;
typedef struct colo_result colo_result;

/* Mining parameters.  distance / pi_threshold / filter_flag are the three
 * values of the reference's parameter file (colocationFinder.cpp:57-74);
 * filter_flag is read and ignored as in the reference. */
typedef struct {
    float distance;          /* R; neighbours satisfy squared distance <= R*R (float) */
    float pi_threshold;      /* prevalent iff !(PI < pi_threshold) */
    uint32_t filter_flag;
    uint32_t max_size;       /* 0 = no cap (the reference has none) */
    int32_t mode;            /* colo_mode */
    int32_t keep_tables;     /* 1: keep every instance table in the result (tests) */
    int32_t reserved[6];     /* reserved[0] bit 0: time every kernel with CUDA events;
                                bit 1: record cost-model features of every candidate;
                                bit 2: generate candidates on the device at every level
                                (otherwise only for levels with 4096+ prevalent patterns);
                                bit 3: keep instance tables in pinned host memory mapped
                                into the device (otherwise only tables whose device
                                allocation fails go there);
                                bit 4 (COLO_MODE_LEARNED): write every refined
                                candidate's table in the counting pass (otherwise only
                                tables presized at 2^20 rows or more);
                                reserved[1] > 0, tests of the timeout path only: the
                                bucketing sort's look-back gives up after that many
                                polls and its first tile withholds its counts, so the
                                mine fails with COLO_ERR_TIMEOUT (no wait is unbounded;
                                the context stays usable) */
} colo_params;

const char* colo_status_string(colo_status s);

/* ---- context ---------------------------------------------------------- */
/* Replaces the colocationFinder constructor (colocationFinder.cpp:21-42):
 * no fixed-size buffers are allocated up front. */
colo_status colo_create(colo_ctx** out, int device);
colo_status colo_destroy(colo_ctx* ctx);
/* Last error message of this context ("" if none). */
const char* colo_last_error(const colo_ctx* ctx);
void colo_params_default(colo_params* p);

/* ---- input ------------------------------------------------------------ */
/* LoadParameter (colocationFinder.cpp:57-74): "R thr flag" whitespace separated. */
colo_status colo_read_params(const char* path, colo_params* out);
/* Begin's config file (colocationFinder.cpp:1077-1092): five lines --
 * location, parameter file, dataset, output location, output file.  Each
 * out buffer receives a NUL-terminated line (cap bytes each). */
colo_status colo_read_config(const char* path, char* location, char* param_file, char* dataset,
                             char* out_location, char* out_file, size_t cap);
/* populateData (colocationFinder.cpp:139-254): count line, "fid,x,y" lines
 * grouped by feature until an empty line, then "minX,minY,maxX,maxY". */
colo_status colo_dataset_from_csv(colo_ctx* ctx, const char* path, colo_dataset** out);
/* Same data from host arrays: raw feature ids grouped as in populateData
 * (a change of id starts a new feature, colocationFinder.cpp:168-184). */
colo_status colo_dataset_from_host(colo_ctx* ctx, const float* x, const float* y,
                                   const int32_t* fid, uint64_t n, const float bounds[4],
                                   colo_dataset** out);
/* Write a dataset in the reference's CSV format (for the CLI and tests). */
colo_status colo_dataset_write_csv(const colo_dataset* ds, const char* path);
/* colo_dataset_from_csv with a chosen number of parser threads (0: one per
 * hardware thread, fewer for small files).  The text is cut into runs of
 * whole lines parsed in parallel; points, features, names and the line named
 * by an error are those of the serial reading.  No counterpart in the
 * reference (its populateData reads serially). */
colo_status colo_dataset_from_csv_threads(colo_ctx* ctx, const char* path, uint32_t threads,
                                          colo_dataset** out);
/* populateData's CSV parsed on the device: the text is copied to the device
 * once, line ends are found and every line is parsed by its own thread with
 * the host reader's rules; coordinates whose exact conversion cannot be
 * proved on the device (and lines with quotes or escapes) are parsed on the
 * host.  Same result and errors as colo_dataset_from_csv; the dataset's
 * coordinates are resident on the device afterwards.  No counterpart in the
 * reference. */
colo_status colo_dataset_from_csv_device(colo_ctx* ctx, const char* path, colo_dataset** out);
/* Binary point file: the points (x, y f32), raw ids (i32), feature names and
 * bounds of a dataset, loaded without parsing.  Little-endian; a 64-byte
 * header ("COLOPTS1", version 1, header bytes, n, features, name bytes,
 * bounds[4]), then x[n], y[n], id[n], name_len[features] u32, the names.
 * No counterpart in the reference. */
colo_status colo_dataset_write_binary(const colo_dataset* ds, const char* path);
colo_status colo_dataset_from_binary(colo_ctx* ctx, const char* path, colo_dataset** out);
/* Host only (needs no device): parse a CSV dataset (threads as above) and
 * write it as a binary point file.  err receives a failure's message
 * (err_cap bytes, NUL-terminated; may be NULL). */
colo_status colo_csv_to_binary(const char* csv_path, const char* bin_path, uint32_t threads, char* err,
                               size_t err_cap);
/* Copy the points to the device now and keep them there for later mines
 * (initializeDeviceMemory, colocationFinder.cpp:443-464).  Otherwise a mine of
 * one dataset page-locks and maps the host arrays and its cell-key pass reads
 * them over the host link (no device copy is kept); a batch of several
 * datasets copies them. */
colo_status colo_dataset_upload(colo_dataset* ds);
/* Drop the device copy (the next mine reads the host arrays again). */
colo_status colo_dataset_evict(colo_dataset* ds);
uint64_t colo_dataset_num_points(const colo_dataset* ds);
uint32_t colo_dataset_num_features(const colo_dataset* ds);
/* Number of instances of feature f (0 if f is out of range). */
uint64_t colo_dataset_feature_count(const colo_dataset* ds, uint32_t f);
/* Name (as written in the CSV) of feature f. */
const char* colo_dataset_feature_name(const colo_dataset* ds, uint32_t f);
void colo_dataset_free(colo_dataset* ds);

/* ---- mining ----------------------------------------------------------- */
/* The level loop of Begin (colocationFinder.cpp:1068-1147): degree2Processing
 * (256-425), then generatePrevalentPatternsGeneral (736-854) and
 * generateInstanceTableGeneral (856-909) per level, candidateColocationGeneral
 * (517-557) between levels. */
colo_status colo_mine(colo_ctx* ctx, colo_dataset* ds, const colo_params* p, colo_result** out);
/* Many independent jobs; in COLO_MODE_BATCHED/LEARNED every job's level-k
 * candidates share one launch per level. */
colo_status colo_mine_batch(colo_ctx* ctx, colo_dataset* const* ds, const colo_params* p,
                            uint32_t njobs, colo_result** out);

/* ---- results ---------------------------------------------------------- */
uint32_t colo_result_num_levels(const colo_result* r);
uint32_t colo_result_level_size(const colo_result* r, uint32_t li);       /* k of level li */
uint64_t colo_result_level_candidates(const colo_result* r, uint32_t li); /* |C_k| */
/* Per-candidate trace of one level; arrays sized ncand*k (cand, ub, num) or
 * ncand (pass, rows, pi, prevalent, argmin); any pointer may be NULL.
 * ub: filter upper-bound counts; pass: filter verdict; rows: instance-table
 * rows (0 when not refined); num: participation numerators; pi: float PI
 * (-1 when not refined); argmin: member giving the minimum. */
colo_status colo_result_level(const colo_result* r, uint32_t li, uint32_t* cand, uint64_t* ub,
                              uint8_t* pass, uint64_t* rows, uint64_t* num, float* pi,
                              uint8_t* prevalent, uint32_t* argmin);
/* Instance table of candidate ci of level li (kept with keep_tables):
 * returns rows, copies rows*k point ids row-major into out if non-NULL;
 * UINT64_MAX if the table was not built. */
uint64_t colo_result_table(const colo_result* r, uint32_t li, uint64_t ci, uint32_t* out);
/* savetoFileGen format (colocationFinder.cpp:979-997):
 * <location>ColocationDegree_<k>.txt with lines "( a | b | c )". */
colo_status colo_result_write_patterns(const colo_result* r, const colo_dataset* ds,
                                       const char* location);
/* Timing of the last mine, milliseconds: [0] total, [1] upload, [2] bucketing,
 * [3] join, [4] filter, [5] refine, [6] fill, [7] host Apriori. */
colo_status colo_result_times(const colo_result* r, double* ms8);
/* Work counters (n entries): [0] kernel launches, [1] join anchors with
 * higher-feature neighbour cells, [2] neighbour entries E, [3] table rows
 * written, [4] pair distance evaluations in the join, [5] points, [6] occupied cells, [7] runs, [8] slice entries
 * examined by count passes, [9] parent words read by count passes,
 * [10] table words written, [11] bitmap words, [12] host-to-device bytes
 * of point coordinates (0 when the points were resident),
 * [13] device-to-host bytes, [14] neighbourhood-run entries, [15] refined
 * candidates, [16] (driver cell, candidate) items of the level filters,
 * [17] candidates filled in one presized pass, [18] of those, overflowed and
 * refilled by the two-pass fallback, [19] (cell of U_c, member) run lookups
 * of the level filters, [20] full quads found by the level filters, [21]
 * cells of U_c summed over candidates, [22] microseconds of the pairs'
 * cost-model step on the host, [23] microseconds from the level filters'
 * launches to their readback, [24] bytes of instance tables placed in pinned
 * host memory. */
colo_status colo_result_counters(const colo_result* r, uint64_t* c, uint32_t n);
/* Per-kernel CUDA-event timing of the mine (with reserved[0] bit 0 set).  Besides the kernel
 * families, entries named "gap X" give the stream time between the previous timed kernel and
 * family X (the GPU waiting for the host), and "host X" the host time from the last wait on
 * the stream to X's launch. */
uint32_t colo_result_num_kernels(const colo_result* r);
colo_status colo_result_kernel(const colo_result* r, uint32_t i, char* name, size_t cap, uint64_t* launches,
                               double* ms);
/* The context's CUDA stream (cudaStream_t), for callers that time or order
 * their own work against the library's. */
void* colo_ctx_stream(const colo_ctx* ctx);
void colo_result_free(colo_result* r);

/* ---- stage entry points (mirror the reference's inner extern "C" API) ---- */
/* CountCellFeatures (DeviceProcess.cu:312-369): per-point cell ids and the
 * (cell, feature) runs of the bucketed dataset.  cell_of[n]; run arrays
 * sized by *nruns (call with NULL arrays first to get the count). */
colo_status colo_stage_cells(colo_ctx* ctx, colo_dataset* ds, float R, uint64_t* cell_of,
                             uint64_t* run_cell, uint32_t* run_feat, uint32_t* run_count,
                             uint64_t* nruns);
/* The neighbour relation that degree2TableSlotCounter_Kernel and the level-k
 * kernels evaluate (DeviceProcess_Kernel.h:12-55, 255-316) as a CSR:
 * N+(a) = {b : feat(b) > feat(a), cells adjacent, sq(a,b) <= R^2}, each list
 * ordered by (feature, neighbour cell, b).  offs[n+1], nbr[*total]. */
colo_status colo_stage_neighbors(colo_ctx* ctx, colo_dataset* ds, float R, uint64_t* offs,
                                 uint32_t* nbr, uint64_t* total);
/* filter2 / threshold_Kernel (DeviceProcess.cu:219-235): upper bounds and
 * verdicts for ncand candidates of size k (global feature indices). */
colo_status colo_stage_filter(colo_ctx* ctx, colo_dataset* ds, float R, float thr,
                              const uint32_t* cand, uint64_t ncand, uint32_t k, uint64_t* ub,
                              uint8_t* pass);
/* Reference squared-distance expression (Utility_Inline.h:25-33) evaluated
 * on the device for n point pairs: out[i] = sq(x1,y1,x2,y2) bits. */
colo_status colo_stage_sqdist(colo_ctx* ctx, const float* x1, const float* y1, const float* x2,
                              const float* y2, uint64_t n, float* out);
/* The same plus, in within[i], the decision the join and level kernels take
 * for sq <= R2 (their fast FMA test with the reference expression as the
 * fallback near the boundary); either output may be NULL. */
colo_status colo_stage_within(colo_ctx* ctx, const float* x1, const float* y1, const float* x2,
                              const float* y2, uint64_t n, float R2, float* out, uint8_t* within);

/* The device-wide exclusive scan the mining kernels use for their offsets
 * (replacing thrust::exclusive_scan, DeviceProcess.cu:342-344), on n host
 * values: out[i] = in[0] + ... + in[i-1], *total = the sum of all n.  wide = 0:
 * in is uint32_t, out uint64_t; wide = 1: in and out are uint64_t. */
colo_status colo_stage_scan(colo_ctx* ctx, const void* in, uint64_t n, int wide, uint64_t* out, uint64_t* total);

/* candidateColocationGeneral (colocationFinder.cpp:517-557) on the device:
 * the level-k candidates of the nprev prevalent (k-1)-patterns in prev
 * (row-major, lexicographic order), with the reference's breaks.  Writes up
 * to cap candidates (k features each) to out and each one's prefix pattern
 * index to parent; *n_out receives the number of candidates.  The mining
 * loop takes this path when a level has many prevalent patterns. */
colo_status colo_stage_apriori(colo_ctx* ctx, const uint32_t* prev, uint64_t nprev, uint32_t k, uint32_t* out,
                               uint32_t* parent, uint64_t cap, uint64_t* n_out);

/* ---- autotuning ------------------------------------------------------- */
/* Times the cell-pair join of this dataset at 1, 2, 4, 8, 16 and 32 lanes
 * per anchor (CUDA events, after a warm-up) and keeps the fastest for later
 * mines on this context.  The join writes the same lists at every width.
 * join_group (optional) receives the choice, ms (optional,
 * COLO_JOIN_WIDTHS doubles, in that order) the times.  The cell size is not tuned: it is R, as the reference's neighbour
 * rule is defined on that grid.  No counterpart in the reference. */
#define COLO_JOIN_WIDTHS 6
colo_status colo_autotune(colo_ctx* ctx, colo_dataset* ds, const colo_params* p, int32_t* join_group,
                          double* ms);
/* Sets the join's lanes per anchor for later mines on this context without
 * timing (1, 2, 4, 8, 16 or 32; 0 restores the default).  COLO_ERR_ARG for any
 * other width. */
colo_status colo_set_join_group(colo_ctx* ctx, int32_t join_group);

/* Launch shapes tuned per dataset (no counterpart in the reference): lanes
 * per anchor in the cell-pair join (1, 2, 4, 8, 16, 32), candidates per warp
 * unit in the level filter (8, 16, 32), threads per block of the level
 * kernels (64, 128, 256; 0 keeps the defaults 8, 32, 256) and the level
 * queue (0: one warp per 32-row chunk; 1: a persistent grid whose warps take
 * chunks by ticket, largest candidates first in COLO_MODE_LEARNED).  Every
 * setting gives the same results. */
typedef struct {
    int32_t join_group;
    int32_t filter_unit;
    int32_t level_block;
    int32_t level_queue;
    int32_t from_cache;      /* colo_autotune_all: 1 when the shapes came from the cache file */
} colo_tuning;
/* Tunes all four for this dataset and parameters and keeps them for later
 * mines on this context: the join as colo_autotune does, then the filter unit,
 * the level block size and the level queue from the CUDA-event time of their
 * own kernels in whole mines.  cache_path (optional) is a text file of tuned shapes keyed by
 * (points, features, occupied cells, R, SM count): a key found there is
 * applied without timing; a new key is appended.  out (optional) receives
 * the shapes. */
colo_status colo_autotune_all(colo_ctx* ctx, colo_dataset* ds, const colo_params* p, const char* cache_path,
                              colo_tuning* out);
/* Sets / reads the context's launch shapes (COLO_ERR_ARG for other values). */
colo_status colo_set_tuning(colo_ctx* ctx, const colo_tuning* t);
colo_status colo_get_tuning(const colo_ctx* ctx, colo_tuning* t);

/* ---- learned cost model ----------------------------------------------- */
/* A 24 -> 64 -> 64 -> 1 ReLU MLP (BF16 weights and activations, FP32
 * accumulation, hand-written tensor-core kernels) that predicts
 * log1p(instance-table rows) of a candidate that passed the filter.  In
 * COLO_MODE_LEARNED it presizes the single-pass table buffers and orders the
 * level queue; a candidate whose table overflows is refilled by the exact
 * two-pass fill, so results never depend on it.  No counterpart in the
 * reference.  Parameters (COLO_MODEL_PARAMS floats): W1[32][64] (input rows
 * 24..31 zero), b1[64], W2[64][64], b2[64], W3[64], b3. */
#define COLO_MODEL_FEATURES 24
#define COLO_MODEL_PARAMS (32 * 64 + 64 + 64 * 64 + 64 + 64 + 1)
/* y[i] = model(x[i*24 .. i*24+23]) for n rows (host arrays). */
colo_status colo_model_forward(colo_ctx* ctx, const float* params, const float* x, uint64_t n, float* y);
/* Gradient of mean_i 0.5*(y_i - t_i)^2 with respect to the parameters. */
colo_status colo_model_grad(colo_ctx* ctx, const float* params, const float* x, const float* t, uint64_t n,
                            float* grad, float* loss);
/* Adam (lr, beta 0.9/0.999) on the GPU over shuffled minibatches; params is
 * updated in place; epoch_loss[e] (optional) = mean minibatch loss. */
colo_status colo_model_train(colo_ctx* ctx, float* params, const float* x, const float* t, uint64_t n,
                             uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float* epoch_loss);
/* Install a model for COLO_MODE_LEARNED mines on this context (NULL: none;
 * without a model LEARNED mines run the BATCHED schedule). */
colo_status colo_ctx_set_model(colo_ctx* ctx, const float* params);
/* The model's 24 input features of every candidate of level li (ncand*24
 * floats): [0] k/8, [1..8] log1p(n_j), [9..16] log1p(ub_j) (members j < 8,
 * else 0), [17] log1p(parent rows), [18] log1p(cells of U_c), [19]
 * log1p(full quads), [20] log1p(min n_j), [21] log1p(min ub_j), [22]
 * log1p(parent rows) - log1p(n_last), [23] log1p(ub_last) - log1p(n_last).
 * Quad statistics are 0 for pairs.  Recorded for every candidate when the
 * mine's colo_params.reserved[0] has bit 1 set (training data); zeros
 * otherwise.  (A COLO_MODE_LEARNED mine computes them for its predictions
 * without keeping them: on the device right after the level filter for
 * k >= 3, on the host for pairs.) */
colo_status colo_result_features(const colo_result* r, uint32_t li, float* x);

/* ---- allocation-free entry point -------------------------------------- */
/* No counterpart in the reference (the reference allocates its participation
 * bitmaps with cudaMalloc per candidate).  For callers that cannot call
 * cudaMalloc: hosts whose own pool holds the GPU's memory (an allocation
 * behind the pool's back fails or breaks its accounting) and latency-bound
 * services that cannot accept cudaFree's device-wide synchronisation.
 *
 * Participation numerators and PI of one size-k candidate (2 <= k <= 32)
 * from its instance table, as colo_mine computes them:
 *   table  device, rows*k point ids, row-major (colo_result_table's layout)
 *   fstart, fcount  host, k entries: first point id and instance count of
 *          each member feature; ids outside [fstart, fstart+fcount) are not
 *          counted, and then num[] = UINT64_MAX and *pi = NaN
 *   num    device, k numerators;  pi  device, 1 float (may be NULL)
 *   stream cudaStream_t on the calling thread's current device (NULL: the
 *          legacy default stream); the call only enqueues work.
 * Allocates nothing: the bitmaps live in a fixed device array of
 * COLO_TABLE_PI_STATIC_WORDS 32-bit words (4 MiB, plus 2 KiB of control
 * words), held by every GPU where the library is loaded until exit.
 * COLO_ERR_CAPACITY when the sum over members of ceil(fcount/32) exceeds it.
 * The first call on a device looks up the array's device address (once per
 * device) and caches it; make that first call before any stream capture.  A
 * cudaDeviceReset of a device after its first call is not supported: the
 * cached address would no longer be valid.  All calls share
 * the array and each clears what it uses: calls that overlap on the GPU race
 * and give wrong results. */
#define COLO_TABLE_PI_STATIC_WORDS (1u << 20)
colo_status colo_table_pi_static(const uint32_t* table, uint64_t rows, uint32_t k,
                                 const uint32_t* fstart, const uint32_t* fcount, uint64_t* num,
                                 float* pi, void* stream);

#ifdef __cplusplus
}
#endif
#endif
