/*
 * libtch — exact cgMLST Hamming distance matrix on the NVIDIA GB300 (sm_103a).
 *
 *   H = P Pt - (O Ot + R)
 *
 *   P  n x L presence bits (allele called at a locus)
 *   O  n x D one-hot bits of the frequent alleles (seen >= tau times)
 *   R  equal pairs of the rare alleles, as CSR by row (partners j > i)
 *
 * H[i][j] is the number of loci where profiles i and j are both called and
 * differ.  Every value is an exact integer (u16, at most L <= 65535).
 *
 * The first block is the reference project's C ABI, kept bit-compatible so
 * that its Rust host (tensorcore/rs/src/main.rs:84-93) links against this
 * library unchanged.  Everything after it is an extension with no counterpart
 * in the reference.  No declaration uses CUDA or PyTorch types: device
 * pointers and streams are passed as plain pointers.
 *
 * Return convention of every int function (reference tch.cu:52-53, 155-169):
 * 0 on success; non-zero on failure, with a NUL-terminated message written to
 * err[errlen] when err is not NULL.
 */
#ifndef TCH_H
#define TCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------------------
 * Reference ABI (tensorcore/rs/cuda/tch.cu:68-86)
 * ------------------------------------------------------------------------- */

/* Stripe callback (tch.cu:79).  Called once per stripe, in increasing r0
 * order, on the thread that called tch_run, after the stripe's copy to host
 * memory completed.  `stripe` is rows x w u16, row-major, w = n - r0; column c
 * holds H[r0 + r][r0 + c].  Only c > r is meaningful (the callers read the
 * strict upper triangle, main.rs:204-211).  The pointer is valid only during
 * the call. */
typedef void (*tch_cb)(void* ctx, int r0, int rows, size_t w, const uint16_t* stripe);

/* Number of CUDA devices; 0 on error.  Replaces tch.cu:68-71. */
int tch_device_count(void);

/* Free device memory in bytes after making `device` current; 0 on error.
 * Replaces tch.cu:73-77. */
size_t tch_free_vram(int device);

/* The whole distance matrix, upper triangle, in stripes of S rows.
 * Replaces tch.cu:81-170 (declared on the Rust side at main.rs:88-92).
 *
 *   O      n_pad x K1 bits, row-major, bit k of a row at byte k>>3, bit k&7
 *          (LSB first).  K1 a multiple of 1024, n_pad of 256, padding zero.
 *   P      n_pad x K2 bits, same layout.
 *   start  n+1 offsets into js; js[start[i] .. start[i+1]) are the partners
 *          j > i of row i (any order, repeats allowed: one entry per locus
 *          where i and j share a rare allele).  n_rare = start[n].
 *   S      rows per stripe (a multiple of 8 in the reference's host).
 *   gpu_secs     (may be NULL) device time of the whole pipeline.
 *   rare_on_gpu  1 if the rare pairs were applied on the GPU, 0 if on the
 *                host because they did not fit in device memory (tch.cu:105).
 */
int tch_run(int device, int n, size_t n_pad, const uint8_t* O, size_t K1, const uint8_t* P, size_t K2,
            const uint32_t* start, const uint32_t* js, size_t n_rare, int S, tch_cb cb, void* ctx,
            double* gpu_secs, int* rare_on_gpu, char* err, int errlen);

/* ----------------------------------------------------------------------------
 * Extensions (no counterpart in the reference)
 * ------------------------------------------------------------------------- */

#define TCH_VERSION 1

/* Contraction kernels.  AUTO picks the fastest one measured on GB300 that is
 * exact for the problem's size.  Compiled into this library: POPC and TC_F4;
 * the others name paths measured by the peak probe and not built (the b1 and
 * s8 warp MMAs issue at ~150 TOPS on GB300, kind::i8 does not exist on
 * sm_103a, the fp8 kind runs at half the fp4 rate). */
enum tch_kernel {
    TCH_KERNEL_AUTO = 0,
    TCH_KERNEL_POPC = 1, /* CUDA cores: LOP3 AND + popcount on the bit-packed rows */
    TCH_KERNEL_MMA_B1 = 2, /* legacy warp MMA: mma.sync m16n8k256 b1 AND+popc   */
    TCH_KERNEL_TC_F8 = 3, /* tcgen05.mma kind::f8f6f4, e4m3 0/+-1, TMEM fp32     */
    TCH_KERNEL_TC_I8 = 4, /* tcgen05.mma kind::i8, s8 0/+-1, TMEM s32           */
    TCH_KERNEL_TC_F16 = 5, /* tcgen05.mma kind::f16, bf16 0/+-1, TMEM fp32       */
    TCH_KERNEL_TC_F4 = 6, /* tcgen05.mma kind::mxf4 (scales 1.0), e2m1 0/+-1, TMEM fp32 */
    TCH_KERNEL_COUNT = 7
};

int tch_version(void);
/* Name of a kernel id ("popc", "tc_f4", ...), or "?" */
const char* tch_kernel_name(int kernel);
/* 1 if `kernel` was compiled into this library. */
int tch_kernel_available(int kernel);
/* Process-wide default kernel used by tch_run (TCH_KERNEL_AUTO initially;
 * the TCH_KERNEL environment variable, a kernel name, overrides it at load). */
int tch_set_kernel(int kernel);
int tch_get_kernel(void);

/* Sizes and choices of a solver, filled by tch_solver_info. */
typedef struct tch_info {
    int n;             /* profiles */
    int L;             /* loci (0 when built from bit-packed operands) */
    int tau;           /* frequency threshold (0 when unknown) */
    int kernel;        /* enum tch_kernel actually used */
    size_t n_pad;      /* padded row count of the device operands */
    size_t k_presence; /* presence columns of the device operand rows */
    size_t k_onehot;   /* the rest of a row's columns: one-hot and padding */
    size_t d_onehot;   /* frequent one-hot columns before padding (0 if unknown) */
    size_t n_rare;     /* rare equal pairs */
    int rare_sorted;   /* 1 if every row's partner list is ascending */
    size_t device_bytes; /* device memory held by the solver */
    int k_chunks;        /* separate allocations the operand rows are split into along K */
    int rare_dense;      /* 1 if the rare term is counted per stripe from rare groups */
    int sub_rows;        /* rows per rare-count + tile-pass pair inside a stripe (0 = the whole stripe) */
    int tile_group;      /* row blocks per raster group of the tile pass (0 = the library default) */
} tch_info;

/* Largest single device allocation of a solver's operand rows, in bytes
 * (0 = no limit, the default; also TCH_MAX_CHUNK_BYTES).  Above it the rows
 * are split along K into up to 8 allocations that the contraction kernel
 * streams in turn, so the one-hot matrix never has to fit in one buffer.
 * Applies to solvers created afterwards. */
int tch_set_max_chunk_bytes(size_t bytes);

/* A solver holds one profile set on one device: the operands of the two
 * contractions and the rare-pair CSR, resident in device memory. */
typedef struct tch_solver tch_solver;

/* Build a solver from the reference's bit-packed host buffers (same meaning
 * as tch_run's arguments).  `kernel` = enum tch_kernel. */
int tch_solver_from_bits(int device, int n, size_t n_pad, const uint8_t* O, size_t K1, const uint8_t* P,
                         size_t K2, const uint32_t* start, const uint32_t* js, size_t n_rare, int kernel,
                         tch_solver** out, char* err, int errlen);

/* Build a solver straight from allele calls (host buffer, n x L u64 row-major,
 * 0 = missing; any other value is an allele id compared for equality only).
 * The encoding the reference's host does (main.rs:134-165, 366-444: dense
 * ranks, frequent one-hot columns, presence, rare equal pairs) runs on the
 * device.  tau <= 0 picks tau with the analytic GB300 cost model.  The rare
 * term is kept as groups of rows per rare allele and counted per stripe into
 * a dense u16 block (tch_set_rare_term(1), the default), or built as the
 * reference's pair lists (tch_set_rare_term(0)).  Fails like the reference
 * when a locus has more than 65535 distinct ids or L > 65535; pair lists also
 * fail when the rare pairs reach 2^32, dense counts when the rare cells do. */
int tch_solver_from_calls(int device, int n, int L, const uint64_t* calls, int tau, int kernel, tch_solver** out,
                          char* err, int errlen);

/* The same from dense per-locus ranks (u16, 0 = missing; equal ranks are equal
 * alleles), the payload of the reference prototype's ranks file
 * (tensorcore/to_ranks.py: int32 n, int32 L, then n x L u16 row-major). */
int tch_solver_from_ranks(int device, int n, int L, const uint16_t* ranks, int tau, int kernel, tch_solver** out,
                          char* err, int errlen);

/* tch_run's stripe/callback contract on allele calls: device encoding, then
 * the whole upper triangle through the callback.  *tau_used (may be NULL)
 * receives the tau that was used.  TCH_VERBOSE=1 prints the tau table. */
int tch_run_calls(int device, int n, int L, const uint64_t* calls, int tau, int S, tch_cb cb, void* ctx,
                  double* gpu_secs, int* tau_used, char* err, int errlen);

/* Rates of the analytic tau model (pair x column MACs per second of the
 * stripe kernel, rare pairs per second); defaults are GB300 measurements. */
int tch_set_tau_model(double gemm_rate, double rare_rate);

/* Rare pairs per second of the dense rare-count build (tau model of
 * solvers with dense rare counts). */
int tch_set_dense_rare_rate(double rate);

/* How solvers built from allele calls hold the rare term, for solvers
 * created afterwards: 1 = rare groups on the device, counted per stripe into
 * a dense block subtracted in the tile epilogue (default); 0 = per-row
 * ascending pair lists walked in the epilogue.  Also TCH_RARE=lists|dense.
 * No reference counterpart (the reference always builds pair lists). */
int tch_set_rare_term(int dense);

/* ---- learned tau and schedule (no reference counterpart) ------------------
 * A small MLP predicts ln(ms) of one whole-triangle solve for each candidate
 * (tau, sub-stripe rows, raster group) from TCH_TAU_FEATURES features; a
 * solver built from calls with tau <= 0 takes the candidate with the smallest
 * prediction when a model is set (tch_set_tau_mlp) and the set has at most
 * 65 536 profiles (the shapes the shipped model was trained on): its tau and
 * its schedule (tch_solver_set_schedule).  Otherwise: the analytic model's tau
 * and the default schedule.  Feature row of a candidate: ln n, ln L, quantiles
 * 0.25 / 0.5 / 0.9 of ln(1 + distinct alleles per locus), missing fraction,
 * ln tau, ln(1 + frequent one-hot columns), ln(1 + rare pairs), ln(1 + rare
 * cells), ln(pairs x operand columns), ln(analytic estimate in seconds),
 * ln(sub-stripe rows / n) (0 for the whole stripe), ln(raster group).
 * Network: F -> 32 -> 32 -> 1, ReLU, fp32, parameters W1[F][32] | b1[32] |
 * W2[32][32] | b2[32] | w3[32] | b3. */
#define TCH_TAU_FEATURES 14
#define TCH_MLP_HIDDEN 32
#define TCH_MLP_PARAMS                                                                             \
    (TCH_TAU_FEATURES * TCH_MLP_HIDDEN + TCH_MLP_HIDDEN + TCH_MLP_HIDDEN * TCH_MLP_HIDDEN + \
     TCH_MLP_HIDDEN + TCH_MLP_HIDDEN + 1)

/* Candidates of a profile set (device encoder's counts; taus whose encoding
 * fits in free device memory, each with every schedule) and their feature
 * rows: taus[r], sub_rows[r], groups[r] (0 = whole stripe),
 * feats[r * TCH_TAU_FEATURES + f] for r < *rows <= max_rows.  est_s[r] (may be
 * NULL) receives the analytic model's estimate of the candidate's tau. */
int tch_tau_features(int device, int n, int L, const uint64_t* calls, int max_rows, int* taus, int* sub_rows,
                     int* groups, float* feats, double* est_s, int* rows, char* err, int errlen);

/* He-normal initial parameters from a seed (host). */
int tch_mlp_init(float* w, uint64_t seed);
/* Full-batch Adam on the GPU (the project's forward/backward kernels, one
 * step captured as a CUDA graph): w updated in place, *loss = final MSE. */
int tch_mlp_train(int device, float* w, const float* X, const float* y, int n, int steps, float lr, float* loss,
                  char* err, int errlen);
/* y[i] = f(X[i]) on the GPU. */
int tch_mlp_predict(int device, const float* w, const float* X, int n, float* y, char* err, int errlen);
/* Mean squared error of f(X) against y and its gradient (TCH_MLP_PARAMS floats). */
int tch_mlp_loss_grad(int device, const float* w, const float* X, const float* y, int n, float* loss, float* grad,
                      char* err, int errlen);
/* Model used by tau <= 0 (copied; NULL = analytic model only). */
int tch_set_tau_mlp(const float* w);

/* ---- serving (no reference counterpart) ----------------------------------------
 * A profile database resident on the device and batches of new profiles
 * against it.  tch_db_query(db, m, q, qdb, qq, stream): q = m x L allele calls
 * (host, u64, 0 = missing) in the database's locus order; writes (host,
 * either may be NULL)
 *   qdb[r * n + j] = distance of new profile r to database row j   (m x n)
 *   qq[a * m + b]  = distance of new profiles a < b                 (m x m,
 *                    upper triangle; other cells untouched)
 * with the reference's semantics (ids compared for equality, 0 missing).  Runs
 * on `stream` (NULL = legacy default) from a stream-ordered pool of the
 * database and returns when the results are in host memory. */
typedef struct tch_db tch_db;
int tch_db_create(int device, int n, int L, const uint64_t* calls, int tau, tch_db** out, char* err, int errlen);
void tch_db_destroy(tch_db* db);
int tch_db_info(const tch_db* db, int* n, int* L, int* tau, size_t* d_onehot, size_t* device_bytes, int* k_chunks);
/* Device bytes a query batch of m profiles takes while it runs. */
size_t tch_db_query_bytes(const tch_db* db, int m);
int tch_db_query(tch_db* db, int m, const uint64_t* qcalls, uint16_t* qdb, uint16_t* qq, void* stream, char* err,
                 int errlen);

/* Page-locked host memory (results copied into it reach the host at the
 * link's speed; pageable buffers go through a staging copy). */
void* tch_host_alloc(size_t bytes);
void tch_host_free(void* p);

/* Continuous batching: `slots` worker threads, one stream each; a FIFO of
 * requests, admitted when tch_db_query_bytes(m) fits in `budget` bytes next to
 * the requests running (0 = half the free device memory; a request larger than
 * the budget runs alone).  Host buffers of a request stay the caller's and
 * must live until tch_server_wait returns for it. */
typedef struct tch_server tch_server;
int tch_server_create(tch_db* db, int slots, size_t budget, tch_server** out, char* err, int errlen);
/* Returns a request id (> 0), or -1 on bad arguments. */
int64_t tch_server_submit(tch_server* sv, int m, const uint64_t* qcalls, uint16_t* qdb, uint16_t* qq);
/* Blocks until the request is done; *queued_s = submit -> start, *latency_s =
 * submit -> results in host memory.  Each id is waited for once: a second
 * wait on it (or one that starts after the first) fails as unknown.
 * tch_server_destroy finishes the queued requests; call it after every
 * wait has returned. */
int tch_server_wait(tch_server* sv, int64_t id, double* queued_s, double* latency_s, char* err, int errlen);
void tch_server_destroy(tch_server* sv);

/* ---- batched solves (no reference counterpart) -----------------------------------
 * `count` independent profile sets (set s: n[s] x L[s] allele calls, host u64,
 * 0 = missing; tau[s] <= 0 or tau == NULL: chosen per set) encoded on the
 * device once.  tch_batch_run writes every set's whole upper triangle into one
 * device buffer: set s at d_out + offsets[s], row stride ld[s] u16
 * (tch_batch_layout; offsets[count] = total u16 elements), cell (i, j), i < j,
 * at (i * ld[s] + j).  A schedule is captured once as a CUDA graph (per
 * output buffer) and replayed on every later run:
 *   branches >= 1  every set's rare counts + tile pass, the sets spread over
 *                  `branches` parallel streams (default 8);
 *   branches == 0  persistent: two launches for the whole batch, the rare
 *                  counts of every row of every set, then one tile pass over
 *                  every set's tiles (dense rare counts, sets of at most
 *                  65 536 rows, at most 8 GiB of rare counts in all; otherwise
 *                  tch_batch_set_schedule(b, 0) returns 1 and the tuner skips it).
 * tch_batch_tune times every schedule and keeps the fastest (*best_branches,
 * 0 = persistent).  Errors found on the device are reported by tch_batch_check. */
typedef struct tch_batch tch_batch;
int tch_batch_create(int device, int count, const int* n, const int* L, const uint64_t* const* calls, const int* tau,
                     tch_batch** out, char* err, int errlen);
/* Add one more set (encoded now); invalidates the captured graph. */
int tch_batch_add(tch_batch* b, int n, int L, const uint64_t* calls, int tau, char* err, int errlen);
int tch_batch_layout(const tch_batch* b, size_t* offsets, size_t* ld);
int tch_batch_run(tch_batch* b, uint16_t* d_out, void* stream, char* err, int errlen);
int tch_batch_check(tch_batch* b, char* err, int errlen);
int tch_batch_tune(tch_batch* b, uint16_t* d_out, void* stream, int reps, double* best_ms, int* best_branches,
                   char* err, int errlen);
int tch_batch_set_schedule(tch_batch* b, int branches);
int tch_batch_info(const tch_batch* b, int* count, int* taus, int* branches);
void tch_batch_destroy(tch_batch* b);

/* ---- the allele table parsed on the GPU (main.rs:286-348) -------------------------
 * tch_tsv_parse copies text[0, len) (the whole input, UTF-8 already checked by
 * the caller) to the device and parses it there as the reference's load does:
 * its lines as str::lines gives them, line 0 the header (L = its field count -
 * 1), every later non-empty line a sample: the id up to the first `sep`, then
 * its cells by parse_allele (main.rs:95-113: Unicode trim, one leading "INF-"
 * dropped unless skip_repl, `missing` (at most 64 bytes) or empty -> 0, all
 * ASCII digits -> the u64 value, anything else -> 0; cells past L dropped,
 * missing ones 0).  A value above 2^64 - 1 fails with "sample <id>: allele
 * '<cell>' too large".  The calls stay in device memory: tch_solver_from_tsv
 * builds a solver from them without a host copy. */
typedef struct tch_tsv tch_tsv;
int tch_tsv_parse(int device, const char* text, size_t len, char sep, int skip_repl, const char* missing,
                  tch_tsv** out, char* err, int errlen);
int tch_tsv_shape(const tch_tsv* t, int* n, int* L);
/* Sample id of row i: text[begin[i], end[i]) of the parsed text. */
int tch_tsv_ids(const tch_tsv* t, size_t* begin, size_t* end);
/* Completeness filters (main.rs:313-348) on the device: loci whose share of
 * non-missing calls x 100 >= locus_pct, then samples whose share >= sample_pct
 * (a negative threshold: no filter). */
int tch_tsv_filter(tch_tsv* t, double locus_pct, double sample_pct, char* err, int errlen);
/* The calls (n x L u64) copied to host memory. */
int tch_tsv_calls(const tch_tsv* t, uint64_t* calls);
/* A solver from the parsed calls (device encoder; tau <= 0: chosen by the
 * models), as tch_solver_from_calls. */
int tch_solver_from_tsv(const tch_tsv* t, int tau, tch_solver** out, char* err, int errlen);
void tch_tsv_free(tch_tsv* t);

/* Fill *info. */
int tch_solver_info(const tch_solver* s, tch_info* info);
/* Schedule of the solver's stripes: every stripe runs as sub-stripes of
 * sub_rows rows (0 = the whole stripe at once; rounded up to a multiple of
 * 128), each its rare counts then its tile pass (a smaller rare-count block,
 * more launches), and the tile pass visits its tiles in raster groups of
 * `tile_group` 128-row blocks (0 = the library default).  A solver built by
 * tch_solver_from_calls / _from_ranks with tau <= 0 and a learned model set
 * (tch_set_tau_mlp) starts with the model's pick.  Every schedule gives the
 * same distances. */
int tch_solver_set_schedule(tch_solver* s, int sub_rows, int tile_group);

/* One stripe into caller-owned DEVICE memory, asynchronously on `stream`
 * (a cudaStream_t, NULL = the legacy default stream):
 *   d_out[(i - r0) * ldo + (j - r0)] = H[i][j]   for r0 <= i < r0 + rows,
 *                                                  max(i, r0) <= j < n
 * Cells with j <= i are unspecified.  ldo >= n - r0.  Errors detected on the
 * device (an invalid rare pair) are reported by the next tch_solver_check. */
int tch_solver_stripe(tch_solver* s, int r0, int rows, uint16_t* d_out, size_t ldo, void* stream, char* err,
                      int errlen);

/* The two passes of tch_solver_stripe for a solver with dense rare counts
 * (tch_info.rare_dense = 1), for callers that schedule them apart (e.g. the
 * counts of the next stripe on a second stream):
 *   tch_solver_rare_counts: d_R[(i - r0) * ldr + (j - r0)] = rare loci shared
 *     by i and j, for r0 <= i < r0 + rows and i < j < n; 0 in the row's other
 *     columns from r0 + ((i - r0) & ~255) to r0 + up(n - r0, 256).
 *   tch_solver_stripe_counts: the stripe of tch_solver_stripe with the rare
 *     term taken from d_R.
 * d_R 16-byte aligned, ldr >= up(n - r0, 256) and a multiple of 8.  No
 * reference counterpart. */
int tch_solver_rare_counts(tch_solver* s, int r0, int rows, uint16_t* d_R, size_t ldr, void* stream, char* err,
                           int errlen);
int tch_solver_stripe_counts(tch_solver* s, int r0, int rows, uint16_t* d_out, size_t ldo, const uint16_t* d_R,
                             size_t ldr, void* stream, char* err, int errlen);

/* The whole matrix as the reference's TSV (tensorcore/rs/src/main.rs:224-265:
 * header `index_name{osep id}*`, then per sample `id{osep value}*`, newline;
 * layout 0 full, 1 lower-tri, 2 upper-tri (masked cells print 0, the diagonal
 * 0), then cap > 0 caps every value), formatted on the GPU: the upper triangle
 * is computed into device memory, mirrored, and formatted in blocks of
 * block_rows rows (0 = 2048); cb receives the header, then every block's text,
 * in order, on the calling thread.  No reference counterpart as an entry
 * point (the reference formats on the CPU). */
typedef void (*tch_text_cb)(void* ctx, const char* text, size_t len);
int tch_solver_write_tsv(tch_solver* s, const char* const* ids, const char* osep, const char* index_name, int layout,
                         int cap, int block_rows, tch_text_cb cb, void* ctx, char* err, int errlen);

/* Synchronise the device and report any error recorded by earlier stripes. */
int tch_solver_check(tch_solver* s, char* err, int errlen);

/* The whole upper triangle through host memory, with tch_run's stripe and
 * callback contract (double-buffered: stripe s+1 is computed while the
 * callback consumes stripe s). */
int tch_solver_run(tch_solver* s, int S, tch_cb cb, void* ctx, double* gpu_secs, char* err, int errlen);

void tch_solver_destroy(tch_solver* s);

/* ---- consumers of the matrix: MST, single-linkage clusters, nearest neighbours ----
 * The uses the reference's documentation names for the matrix (outbreak
 * clustering, minimum spanning trees, nearest-neighbour searches;
 * docs/index.html, "The problem"); the reference itself stops at the matrix.
 * Computed on the device from the full matrix in device memory; only the
 * result comes back.
 *
 * Edges of the complete graph are ordered by (distance, smaller index, larger
 * index).  That order is strict, so the minimum spanning tree is unique. */

/* The minimum spanning tree of the profiles: n - 1 edges (u[e] < v[e], w[e]
 * their distance) in the order above, and *total = the sum of w (any output
 * may be NULL).  The solver's full matrix is computed into device memory
 * (n * up(n, 8) * 2 bytes) for the call.  n < 2 gives no edges. */
int tch_solver_mst(tch_solver* s, uint32_t* u, uint32_t* v, uint16_t* w, uint64_t* total, char* err, int errlen);

/* Single-linkage clusters at each of nt thresholds: profiles i and j share a
 * cluster at threshold t when a chain of profiles joins them with every step
 * at distance <= t.  labels[k * n + i] = the smallest profile index in i's
 * cluster at thresholds[k].  (From the minimum spanning tree: the clusters at
 * t are its components after removing the edges heavier than t.) */
int tch_solver_clusters(tch_solver* s, const uint32_t* thresholds, int nt, uint32_t* labels, char* err,
                        int errlen);

/* The k nearest profiles of every profile, 1 <= k <= 32 and k < n, in the
 * order (distance, index): idx[i * k + r] and dist[i * k + r] for rank r. */
int tch_solver_neighbors(tch_solver* s, int k, uint32_t* idx, uint16_t* dist, char* err, int errlen);

/* The same on a full symmetric n x n u16 matrix already in device memory
 * (row stride ld, a multiple of 8; d_H 16-byte aligned; the values on the
 * diagonal and in columns n to ld - 1 are ignored, and columns from up(n, 8)
 * on are not loaded), on `stream` (NULL: a stream of the call); outputs in
 * host memory; the call synchronises before it returns.  n < 2^21. */
int tch_mst_device(const uint16_t* d_H, size_t ld, int n, void* stream, uint32_t* u, uint32_t* v, uint16_t* w,
                   uint64_t* total, char* err, int errlen);
int tch_neighbors_device(const uint16_t* d_H, size_t ld, int n, int k, void* stream, uint32_t* idx, uint16_t* dist,
                         char* err, int errlen);

/* Host only: single-linkage cluster labels at nt thresholds from a minimum
 * spanning tree's m edges (any order; u, v < n), as tch_solver_clusters
 * labels them. */
int tch_mst_clusters(int n, const uint32_t* u, const uint32_t* v, const uint16_t* w, size_t m,
                     const uint32_t* thresholds, int nt, uint32_t* labels, char* err, int errlen);

/* ----------------------------------------------------------------------------
 * Stripe without any device allocation.  No counterpart in the reference: it
 * exists for callers that may not call cudaMalloc (a service with a fixed
 * device-memory budget that it hands out itself, a framework whose allocator
 * must own every byte), which therefore cannot use tch_run or tch_solver_*.
 * ------------------------------------------------------------------------- */

/* Size of the library's file-scope device scratch array (64 MiB). */
#define TCH_NOALLOC_SCRATCH_BYTES (64u << 20)

/* One stripe, like tch_solver_stripe, with every input already in the
 * caller's DEVICE memory and no allocation by the library:
 *
 *   d_O     n x K1 bits, d_P n x K2 bits (tch_run's row layout; rows beyond
 *           n are not read), K1 and K2 multiples of 1024
 *   d_start n + 1 offsets, d_js n_rare partners (any order within a row)
 *   d_out   receives H[i][j] at (i - r0) * ldo + (j - r0) for the stripe's
 *           rows i and columns max(i, r0) <= j < n; ldo even, d_out 16-byte
 *           aligned
 *
 * The two packed fp4 copies of the operand rows of all n profiles and the
 * device error word live in one static device array of
 * TCH_NOALLOC_SCRATCH_BYTES bytes, so the call fails with a clear message when
 * 256 + up(n, 256) * (K2 + K1) bytes exceed it (one byte per bit column; e.g.
 * n = 2 048 with K2 + K1 up to 32 768).
 * The first call on a device takes the array's address (cudaGetSymbolAddress)
 * and must come before any stream capture.  Every call reuses the array, so
 * calls that overlap on the GPU race; the call synchronises `stream` before it
 * returns, on success and on every failure after it has queued work.  The
 * caller's current device is the same after the call as before it.  A device
 * that has loaded the array keeps it until process exit. */
int tch_stripe_noalloc(int device, int n, const uint8_t* d_O, size_t K1, const uint8_t* d_P, size_t K2,
                       const uint32_t* d_start, const uint32_t* d_js, size_t n_rare, int r0, int rows,
                       uint16_t* d_out, size_t ldo, void* stream, char* err, int errlen);

/* ----------------------------------------------------------------------------
 * Host encoder (restates the reference host, main.rs:134-198 and 366-444).
 * Multi-threaded C++; `threads` <= 0 uses every hardware thread.
 * tch_choose_tau and tch_encode_host take ranks and distinct counts as
 * tch_dense_ranks gives them and fail when a count exceeds 65535 or a rank
 * exceeds its locus's count.
 * ------------------------------------------------------------------------- */

/* Dense per-locus ranks (main.rs:134-165): for each locus, the sorted unique
 * non-zero ids get ranks 1..k (0 stays missing).  calls and x are n x L
 * row-major; n_distinct[L] receives k per locus.  Fails when a locus has
 * more than 65535 distinct ids. */
int tch_dense_ranks(const uint64_t* calls, int n, int L, uint16_t* x, uint32_t* n_distinct, int threads,
                    char* err, int errlen);

/* Analytic tau (main.rs:167-198): tau in {2, 4, ..., 4096} minimising
 * n^2/2 * K1 / gemm_rate + R / rare_rate such that the one-hot bits, the
 * rare CSR and the stripe buffers fit in free_bytes and R < 4e9.  With
 * gemm_rate = 5.9e14 and rare_rate = 3.5e9 this is the reference's choice.
 * verbose != 0 prints the reference's per-tau table on stderr. */
int tch_choose_tau(const uint16_t* x, const uint32_t* n_distinct, int n, int L, int stripe, size_t free_bytes,
                   double gemm_rate, double rare_rate, int verbose, int* tau, char* err, int errlen);

/* The reference's operands for a given tau (main.rs:366-444): O, P bit-packed
 * in tch_run's layout, and the rare-pair CSR with each row's partners in
 * ascending order (the reference's order is unspecified). */
typedef struct tch_host_encoding {
    int n, L, tau;
    size_t D;     /* frequent one-hot columns */
    size_t n_pad, K1, K2;
    size_t n_rare;
    uint8_t* O;   /* n_pad * K1 / 8 bytes */
    uint8_t* P;   /* n_pad * K2 / 8 bytes */
    uint32_t* start; /* n + 1 */
    uint32_t* js;    /* n_rare */
} tch_host_encoding;

int tch_encode_host(const uint16_t* x, const uint32_t* n_distinct, int n, int L, int tau, int threads,
                    tch_host_encoding* out, char* err, int errlen);
void tch_host_encoding_free(tch_host_encoding* e);

#ifdef __cplusplus
}
#endif

#endif /* TCH_H */
