// Internal declarations shared by the translation units of libtch.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "tch.h"

namespace tch {

// Error-recording helpers: every public entry point returns 0 / non-zero and
// writes a message into the caller's buffer.
struct Err {
    char* buf;
    int len;
    int set(const char* fmt, ...) __attribute__((format(printf, 2, 3)));
};

#define TCH_CK(e, x)                                                                        \
    do {                                                                                   \
        cudaError_t ck_ = (x);                                                             \
        if (ck_ != cudaSuccess) {                                                          \
            (e).set("%s: %s (%s:%d)", #x, cudaGetErrorString(ck_), __FILE__, __LINE__);    \
            goto fail;                                                                     \
        }                                                                                  \
    } while (0)

inline size_t up(size_t x, size_t m) { return (x + m - 1) / m * m; }

// Per-device one-time set-up flags (kernel attributes are set per device).
constexpr int kMaxDevices = 64;
inline int current_device() {
    int d = 0;
    cudaGetDevice(&d);
    return d >= 0 && d < kMaxDevices ? d : 0;
}

// Bits reported through the device error word.
enum DevErr : int {
    DEVERR_RARE_PAIR = 1,  // a rare partner j outside (i, n)
    DEVERR_OVERFLOW = 2,   // a distance outside [0, 65535]
    DEVERR_TIMEOUT = 4,    // a bounded wait gave up
    DEVERR_TOO_MANY_ALLELES = 8,  // a locus has more distinct ids than the encoder's table holds
};

// Rare-pair CSR on the device.
struct RareCSR {
    const uint32_t* start = nullptr;  // n + 1
    const uint32_t* js = nullptr;     // n_rare
    size_t n_rare = 0;
    bool sorted = false;              // every row ascending -> fused subtraction
    // Optional device flag set by a check of this stripe's rows that ran
    // earlier on the same stream: 0 = ascending (fused subtraction), non-zero =
    // not (the separate atomic pass).  Lets the host launch both without
    // waiting for the check.
    const int* unsorted_flag = nullptr;
    // Dense alternative: the stripe's rare counts as a u16 block laid out
    // like the output (row stride ldr, column j at j - r0); subtracted in the
    // tile epilogue.  Takes precedence over the pair list.
    const uint16_t* dense = nullptr;
    size_t ldr = 0;
};

// Bit-packed operands in the reference layout, u32 words, LSB first.
struct BitOperands {
    const uint32_t* P = nullptr;  // n_pad x wP words
    const uint32_t* O = nullptr;  // n_pad x wO words
    int wP = 0, wO = 0;
};

// The operand rows can be split along K into up to kMaxKChunks separate
// allocations: chunk c holds columns [c * width, c * width + width_c) of every
// row (width a multiple of 128 bytes; the last chunk may be narrower).  The
// one-hot part then never has to fit in one allocation.
constexpr int kMaxKChunks = 8;
struct KChunks {
    uint8_t* p[kMaxKChunks] = {};
    int n = 0;      // chunks in use
    int width = 0;  // bytes of K per chunk row
    int kb = 0;     // bytes per full row
    __host__ __device__ int width_of(int c) const { return c < n - 1 ? width : kb - width * (n - 1); }
    __host__ __device__ uint8_t* at(size_t row, int col) const {
        const int c = col / width;
        return p[c] + row * (size_t)width_of(c) + (col - c * width);
    }
};

// Packed e2m1 operand rows of the tensor-core tile pass.  A row is
// [presence (kp columns) | frequent one-hot (ko columns) | zeros], K columns
// in all, a multiple of 256 (one 128-byte swizzle row of K per pipeline
// stage), two 4-bit elements per byte: column c is the low nibble of byte c/2
// when c is even, the high nibble when odd; kb = K / 2 bytes per row.  In
// `pos` every element is 0 or +1.0 (0x2); in `neg` the one-hot columns hold
// -1.0 (0xA) instead, so that pos_i . neg_j = P_i . P_j - O_i . O_j.  The
// tile pass reads A rows from pos and B rows from neg.  Both copies are split
// along K alike (KChunks); either may be absent (p[] null) where a role is
// never used (a query batch needs only pos, a database only neg).
constexpr uint32_t kFp4One = 0x2, kFp4MinusOne = 0xA;
struct Fp4Operands {
    KChunks pos, neg;
    size_t n_rows = 0;  // multiple of 256
    int kb = 0;         // bytes per row (K / 2)
};

// 8 bits -> 8 nibbles: bit k of x becomes bit 4k of the result.
__host__ __device__ __forceinline__ uint32_t spread_nibbles(uint32_t x) {
    x &= 0xFFu;
    x = (x | (x << 12)) & 0x000F000Fu;
    x = (x | (x << 6)) & 0x03030303u;
    x = (x | (x << 3)) & 0x11111111u;
    return x;
}

// Columns K of the packed rows for kp presence and ko one-hot columns.
inline size_t fp4_columns(size_t kp, size_t ko) { return std::max<size_t>(up(kp + ko, 256), 256); }

// Splits kb bytes of K into chunks of at most max_bytes per chunk for `rows`
// rows (0 = one chunk); returns the chunk width, or 0 if more than
// kMaxKChunks chunks would be needed.
inline int chunk_width_for(int kb, size_t rows, size_t max_bytes) {
    if (!max_bytes || (size_t)kb * rows <= max_bytes) return kb;
    size_t w = max_bytes / std::max<size_t>(rows, 1) / 128 * 128;
    if (w < 128) w = 128;
    const size_t n = ((size_t)kb + w - 1) / w;
    return n > (size_t)kMaxKChunks ? 0 : (int)w;
}

// Upper triangle: rows [r0, r0 + rows) against columns [r0, n) of the same
// set, out[(i - r0) * ldo + (j - r0)].  Rectangle (rect): rows [r0, r0 + rows)
// of one set against columns [0, n) of another, out[(i - r0) * ldo + j].
struct StripeArgs {
    int n = 0, r0 = 0, rows = 0;
    uint16_t* out = nullptr;
    size_t ldo = 0;
    int* err = nullptr;
    bool rect = false;
    int group = 0;  // row blocks per raster group of the tile pass (0 = the library default)
};

// ---- k_popc.cu --------------------------------------------------------------------
cudaError_t launch_popc_stripe(const BitOperands& ops, const RareCSR& rare, const StripeArgs& a,
                               cudaStream_t st);
// Unsorted CSR: separate pass with 32-bit atomics on the u16 stripe.
cudaError_t launch_rare_atomic(const RareCSR& rare, const StripeArgs& a, cudaStream_t st);
// ORs into *d_flag: 1 if a row in [r_begin, r_end) is not ascending, 2 if a
// partner is outside (i, n).  r_end < 0 means n.
cudaError_t launch_rare_check_sorted(const RareCSR& rare, int n, int* d_flag, cudaStream_t st, int r_begin = 0,
                                     int r_end = -1);

// ---- k_expand.cu ------------------------------------------------------------------
// Bit rows (tch_run's layout) -> packed e2m1 operand rows: the first wp words
// of each P row (presence, kp = 32 wp columns) then the first wo words of each
// O row (one-hot, 32 wo columns), zeros after; rows n .. n_rows - 1 all zero.
// X.pos / X.neg as allocated by the caller (n_rows x kb bytes each, chunked).
cudaError_t launch_expand_bits(const BitOperands& bits, int n, int wp, int wo, const Fp4Operands& X,
                               cudaStream_t st);
// Words of the P and O rows that hold a set bit in any row (the rest are
// zero padding): *wp, *wo.
cudaError_t used_bit_words(const BitOperands& bits, size_t n_pad, int* wp, int* wo, cudaStream_t st);
// neg from pos: every non-zero element at column >= kp made -1.0.
cudaError_t launch_negate_onehot(const Fp4Operands& X, int kp, cudaStream_t st);
// Allocates the pos and/or neg copies (n_rows x kb bytes each, split along K
// into chunks of at most max_chunk bytes, 0 = one allocation; their chunk
// layout is set either way); adds the bytes to *bytes.
cudaError_t alloc_fp4(Fp4Operands* X, size_t n_rows, int kb, size_t max_chunk, bool pos, bool neg, size_t* bytes);
void free_fp4(Fp4Operands* X);

// ---- k_tc.cu ----------------------------------------------------------------------
// The tile pass: rows [r0, r0 + rows) of ops (its pos copy) against the
// columns of bops (its neg copy; nullptr = ops, the upper triangle; required
// for a rectangle, with the same K layout and chunking), minus the dense rare
// counts R (row stride ldr, column j at j - c0; nullptr = no rare term).
cudaError_t launch_tc_stripe(const Fp4Operands& ops, const Fp4Operands* bops, const uint16_t* R, size_t ldr,
                             const StripeArgs& a, int num_sms, cudaStream_t st);
// Many whole triangles in one persistent launch (batched solves): item k's
// upper triangle of its own operand into its own output, minus its own rare
// counts (R, ldr as for launch_tc_stripe; may be null).  tc_batch_prepare
// writes the job descriptors, tensor maps and tile -> job table to device
// memory (the plan owns them); launch_tc_batch runs them (capturable).
struct TcBatchItem {
    const Fp4Operands* ops = nullptr;
    int n = 0;
    const uint16_t* R = nullptr;
    size_t ldr = 0;
    uint16_t* out = nullptr;
    size_t ldo = 0;
};
struct TcBatchPlan {
    void* d_jobs = nullptr;
    void* d_maps = nullptr;
    void* d_tile_job = nullptr;  // the job of every tile
    int njobs = 0, num_tiles = 0;
    int grid = 0;  // CTAs of the launch (at most num_sms), each on every grid-th tile
    int* err = nullptr;
};
cudaError_t tc_batch_prepare(const std::vector<TcBatchItem>& items, int num_sms, TcBatchPlan* plan, int* err);
cudaError_t launch_tc_batch(const TcBatchPlan& plan, cudaStream_t st);
void tc_batch_release(TcBatchPlan* plan);

// ---- k_encode.cu ------------------------------------------------------------------
// Rates of the analytic tau model on this GPU.
struct TauModel {
    // pair x column MACs per second of the fp4 tile pass (63 005 x 1 142
    // long-tail profiles: 3.0e15 at tau 1 024, 2.85e15 at 2 048)
    double gemm_rate = 2.9e15;
    double rare_rate = 1.0e12;  // rare pairs per second of the pair-list counts (pair lists)
    // rare pairs per second of the dense rare-count build, at the margin (its
    // fixed part, the u16 block written per stripe, does not depend on tau)
    double dense_rate = 1.5e12;
};

// The rare alleles as groups of rows, kept on the device: the dense rare
// counts of any stripe are built from them on demand.
struct RareGroups {
    const uint16_t* x = nullptr;        // n x L ranks
    const uint64_t* cnt_off = nullptr;  // L + 1: slot of (locus k, rank a) is cnt_off[k] + a
    const uint64_t* goff = nullptr;     // slots + 1: a rare group's rows are members[goff[q] .. goff[q+1])
    const uint32_t* members = nullptr;  // rows of every rare group (count >= 2), ascending per group
    const uint32_t* mpos = nullptr;     // n x L: index in members of row i's own entry, kNoGroup outside groups
    int n = 0, L = 0;
    // Row runs (optional; null: found per locus from the arrays above): row i's
    // partners are runs roff[i] .. roff[i + 1] - 1, in locus order; run q is
    // members[rlo[q] ..) and its items start at rpre[q] within the row (an
    // exclusive prefix), the row's last run ending at rtot[i].
    const uint64_t* roff = nullptr;
    const uint32_t* rlo = nullptr;
    const uint32_t* rpre = nullptr;
    const uint32_t* rtot = nullptr;
};

// R[(i - r0) * ldr + (j - r0)] = number of loci where rows i and j share a
// rare allele, for r0 <= i < r0 + rows and i < j < n; written as 0 for the
// other columns from the start of row i's diagonal tile, r0 + ((i - r0) &
// ~255), up to r0 + up(n - r0, 256); columns before that are left as they
// are.  ldr >= up(n - r0, 256) and a multiple of 8; R 16-byte aligned.
constexpr int kRareDenseAlign = 256;
// Rank of an id that a profile set has never seen (new-profile encoding).
constexpr uint32_t kNovelRank = 0xFFFFFFFFu;
// mpos of a cell whose allele is in no rare group (frequent, missing, or seen once).
constexpr uint32_t kNoGroup = 0xFFFFFFFFu;
// R[r * ldr + j] = loci where new profile r (ranks xq, m x L u32 in the set's
// numbering) and row j of the set share an allele that is rare in the set
// (groups must include single-row groups), for j < n; 0 up to up(n, 256).
cudaError_t launch_rare_query(const RareGroups& g, const uint32_t* xq, int m, uint16_t* R, size_t ldr, int sms,
                              cudaStream_t st);
cudaError_t launch_rare_dense(const RareGroups& g, int r0, int rows, uint16_t* R, size_t ldr, int sms,
                              cudaStream_t st);
// Every set's whole-triangle rare counts in one launch (batched solves):
// item k's counts into its own block R (ldr >= up(n, 256); row i's columns
// from its diagonal tile on, as launch_rare_dense with r0 = 0, rows = n).
// Sets wider than one counter pass (65 536 columns) are rejected.
struct RareBatchItem {
    RareGroups g;
    uint16_t* R = nullptr;
    size_t ldr = 0;
};
struct RareBatchPlan {
    void* d_jobs = nullptr;
    void* d_row_job = nullptr;  // the job of every row
    int njobs = 0, total_rows = 0, cwords = 0;
};
cudaError_t rare_batch_prepare(const std::vector<RareBatchItem>& items, RareBatchPlan* plan);
cudaError_t launch_rare_batch(const RareBatchPlan& plan, int sms, cudaStream_t st);
void rare_batch_release(RareBatchPlan* plan);
// The same block from pair lists (partners of row i: js[start[i] .. start[i +
// 1]), in any order, repeated once per shared rare allele); a partner outside
// (i, n) sets DEVERR_RARE_PAIR in *err and is skipped.
cudaError_t launch_rare_from_lists(const uint32_t* start, const uint32_t* js, int n, int r0, int rows, uint16_t* R,
                                   size_t ldr, int* err, int sms, cudaStream_t st);

// Operands built on the device from allele calls; device memory owned here.
struct DeviceEncoding {
    int n = 0, L = 0, tau = 0;
    size_t D = 0;             // frequent one-hot columns
    uint16_t* x = nullptr;    // n x L ranks
    Fp4Operands X;            // x_rows packed e2m1 rows [presence (L) | one-hot (D)], split along K
    size_t x_rows = 0;
    int kb = 0;               // bytes per row
    int sub_rows = 0, tile_group = 0;  // schedule of the learned model's pick (0 = defaults)
    uint32_t* start = nullptr;  // n + 1 (CSR mode)
    uint32_t* js = nullptr;     // n_rare, ascending per row (CSR mode)
    size_t n_rare = 0;
    // dense mode: the rare groups stay on the device instead of a pair list
    bool dense = false;
    uint64_t* cnt_off = nullptr;
    uint64_t* goff = nullptr;
    uint32_t* members = nullptr;
    uint32_t* mpos = nullptr;
    // every row's partner runs (RareGroups::roff ..), built for triangle solves
    uint64_t* roff = nullptr;
    uint32_t* rlo = nullptr;
    uint32_t* rpre = nullptr;
    uint32_t* rtot = nullptr;
    // query maps (ENC_QUERY): ids in rank order per locus (slot cnt_off[k] + rank,
    // ascending), frequent column of each slot (-1 = rare), per-locus column base
    uint64_t* slot_ids = nullptr;
    int32_t* col = nullptr;
    uint32_t* base = nullptr;
    size_t bytes = 0;
};

// encode_on_device flags: ENC_DENSE keeps the rare groups (dense rare counts)
// instead of building pair lists; ENC_QUERY (implies dense) also keeps
// single-row groups and the maps that encode new profiles like these.
enum EncodeFlags : int { ENC_DENSE = 1, ENC_QUERY = 2 };

// Candidates (tau x schedule) of an encoding and their learned-model feature rows.
struct TauTable {
    std::vector<int> taus;
    std::vector<int> subs;      // sub-stripe rows (0 = the whole stripe)
    std::vector<int> groups;    // raster group (row blocks)
    std::vector<float> feats;   // taus.size() x TCH_TAU_FEATURES
    std::vector<double> est_s;  // analytic estimate per candidate
};
// Schedule values the candidates take.
// Sub-stripes of 2 048 rows were the fastest schedule for 1 of 384 training
// profile sets of the GB300 sweep (and at most 2 % faster there): not offered.
constexpr int kSchedSubs[2] = {0, 8192};
constexpr int kSchedGroups[3] = {4, 8, 16};

// With table != nullptr the encoder stops after the counts and fills it.
int encode_on_device(int device, int n, int L, const uint64_t* d_calls, int tau_req, const TauModel& model,
                     bool verbose, size_t max_chunk_bytes, int flags, DeviceEncoding* out, Err& e,
                     TauTable* table = nullptr);
void free_device_encoding(DeviceEncoding* d);

// ---- tch_solver.cu (used by the batch runner and the database) ------------------------
// Largest single allocation of operand rows (tch_set_max_chunk_bytes; 0 = one).
size_t max_chunk_bytes();
int solver_from_calls(int device, int n, int L, const uint64_t* calls, int tau, int kernel, bool verbose,
                      tch_solver** out, Err& e);
// lists_uploaded: called by the stripe pipeline after the stripe's partner
// lists reached the device (solvers that upload them stripe by stripe).
int solver_stripe(tch_solver* s, int r0, int rows, uint16_t* d_out, size_t ldo, cudaStream_t st, Err& e,
                  bool lists_uploaded = false);
// The same from allele calls already in device memory (n x L u64, L >= 1; read only).
int solver_from_device_calls(int device, int n, int L, const uint64_t* d_calls, int tau, bool verbose,
                             tch_solver** out, Err& e);
int solver_check(tch_solver* s, Err& e);
void solver_free(tch_solver* s);
int solver_stripe_counts(tch_solver* s, int r0, int rows, uint16_t* d_out, size_t ldo, uint16_t* R, size_t ldr,
                         cudaStream_t st, Err& e);
double solver_work(const tch_solver* s);
int solver_size(const tch_solver* s);
// The packed fp4 operand of a tensor-core solver (nullptr for the others).
const Fp4Operands* solver_operands(const tch_solver* s);
// The rare groups of a dense-rare solver (false: it holds pair lists).
bool solver_rare_groups(const tch_solver* s, RareGroups* g);

// ---- format.cu ----------------------------------------------------------------------
// H[i][j] = H[j][i] for j < i < n: the lower half of an n x n matrix (row
// stride ld) from its upper half.
cudaError_t launch_mirror(uint16_t* H, size_t ld, int n, cudaStream_t st);

// ---- k_mlp.cu ----------------------------------------------------------------------
constexpr int kMlpIn = TCH_TAU_FEATURES, kMlpHidden = TCH_MLP_HIDDEN, kMlpParams = TCH_MLP_PARAMS;
// pred / loss / grad optional; y required for loss and grad.
int mlp_run(int device, const float* w, const float* X, const float* y, int n, float* pred, float* loss,
            float* grad, Err& e);
int mlp_train(int device, float* w, const float* X, const float* y, int n, int steps, float lr, float* loss_out,
              Err& e);
// The model set by tch_set_tau_mlp, if any.
bool tau_mlp_weights(float* out);

}  // namespace tch
