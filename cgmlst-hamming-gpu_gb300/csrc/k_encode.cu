// Device encoder: allele calls (u64, 0 = missing) -> the tensor-core operand X
// and the rare-pair CSR, without leaving the GPU except for small tables.
//
// It produces what the reference's host computes in main.rs:134-165 (dense
// per-locus ranks), 366-403 (frequent one-hot columns, presence) and 404-444
// (rare equal pairs), as device kernels:
//
//   1. insert_kernel      per-locus open-addressing hash tables (u64 keys,
//                         atomicCAS) with a count per distinct id
//   2. rank_kernel        one CTA per locus: compacts the distinct ids and
//                         ranks each by counting the smaller ids (the
//                         reference's sorted-unique rank, 1..k), and writes
//                         the count of every rank
//   3. cell_rank_kernel   every cell -> its rank (u16 matrix x, n x L)
//      (host)             tau from the counts (analytic model), frequent
//                         column map and per-locus offsets
//   4. pack_x_kernel      x -> X rows [presence | one-hot] as packed e2m1
//                         nibbles (+1.0), the pos copy; negate_onehot_kernel
//                         derives the neg copy (one-hot part -1.0)
//   5. group_fill_kernel  rows of each rare (locus, rank) group of size >= 2
//      group_sort_kernel  ... sorted ascending inside the group
//   6. rare_rows_kernel   one CTA per row: u16 counters over the columns
//                         j > i (shared memory, 64 Ki columns per chunk), one
//                         increment per shared rare group, then a block scan
//                         emits the partners in ascending order with their
//                         multiplicity.  Run twice: counts, then the CSR.
//
// The CSR rows come out ascending; the tensor-core path counts them into the
// dense rare-count block that the tile epilogue subtracts.  All ids are compared for equality only; any 64-bit values
// work (hashed ids included).

#include <chrono>
#include <vector>

#include <math.h>

#include "tch_internal.cuh"

namespace tch {
namespace {

constexpr uint32_t kMaxDistinct = 65535;
constexpr int kJC = 65536;  // columns per counter chunk (u16 counters: 128 KB)

__device__ __forceinline__ uint32_t hash_slot(uint64_t v, int logC) {
    return (uint32_t)((v * 0x9E3779B97F4A7C15ull) >> (64 - logC));
}

__global__ void insert_kernel(const uint64_t* __restrict__ calls, int n, int L, int k0, int nk,
                              unsigned long long* keys, uint32_t* cnts, int logC, uint32_t* nd, int* err) {
    const size_t C = (size_t)1 << logC, total = (size_t)n * nk;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = t / nk;
        const int kk = (int)(t % nk);
        const unsigned long long v = calls[i * L + k0 + kk];
        if (!v) continue;
        unsigned long long* kt = keys + kk * C;
        uint32_t s = hash_slot(v, logC);
        bool placed = false;
        for (size_t probe = 0; probe < C; probe++, s = (s + 1) & (uint32_t)(C - 1)) {
            unsigned long long cur = kt[s];
            if (cur == 0) cur = atomicCAS(kt + s, 0ull, v);
            if (cur == 0) {  // new distinct id
                atomicAdd(nd + k0 + kk, 1u);
                atomicAdd(cnts + kk * C + s, 1u);
                placed = true;
                break;
            }
            if (cur == v) {
                atomicAdd(cnts + kk * C + s, 1u);
                placed = true;
                break;
            }
        }
        if (!placed) atomicOr(err, DEVERR_TOO_MANY_ALLELES);
    }
}

// One CTA per locus of the batch.  rank = 1 + #(distinct ids smaller than it).
__global__ void rank_kernel(int k0, const unsigned long long* keys, const uint32_t* cnts, int logC,
                            const uint32_t* nd, const uint64_t* cnt_off, uint32_t* cnt_flat, uint16_t* rank_slot,
                            unsigned long long* list_keys, uint32_t* list_slots, unsigned long long* slot_ids,
                            uint32_t lcap, int* err) {
    const int kk = blockIdx.x;
    const size_t C = (size_t)1 << logC;
    const unsigned long long* kt = keys + kk * C;
    // a locus has at most min(n, kMaxDistinct) distinct ids: lcap entries per list
    unsigned long long* lk = list_keys + (size_t)kk * lcap;
    uint32_t* ls = list_slots + (size_t)kk * lcap;
    __shared__ uint32_t m;
    __shared__ unsigned long long tile[2048];
    if (threadIdx.x == 0) m = 0;
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < C; s += blockDim.x) {
        const unsigned long long v = kt[s];
        if (v) {
            const uint32_t idx = atomicAdd(&m, 1u);
            if (idx < lcap) {
                lk[idx] = v;
                ls[idx] = s;
            }
        }
    }
    __syncthreads();
    const uint32_t mm = m;
    if (mm > lcap || mm != nd[k0 + kk]) {
        if (threadIdx.x == 0) atomicOr(err, DEVERR_TOO_MANY_ALLELES);
        return;
    }
    const uint64_t off = cnt_off[k0 + kk];
    // each thread ranks up to 8 ids per sweep of the id list through shared memory
    for (uint32_t e0 = 0; e0 < mm; e0 += 8 * blockDim.x) {
        unsigned long long mine[8];
        uint32_t r[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const uint32_t e = e0 + q * blockDim.x + threadIdx.x;
            mine[q] = e < mm ? lk[e] : ~0ull;
            r[q] = 0;
        }
        for (uint32_t f0 = 0; f0 < mm; f0 += 2048) {
            const uint32_t cntf = min(2048u, mm - f0);
            __syncthreads();
            for (uint32_t f = threadIdx.x; f < cntf; f += blockDim.x) tile[f] = lk[f0 + f];
            __syncthreads();
            for (uint32_t f = 0; f < cntf; f++) {
                const unsigned long long w = tile[f];
#pragma unroll
                for (int q = 0; q < 8; q++) r[q] += w < mine[q];
            }
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const uint32_t e = e0 + q * blockDim.x + threadIdx.x;
            if (e < mm) {
                const uint32_t slot = ls[e];
                rank_slot[kk * C + slot] = (uint16_t)(r[q] + 1);
                cnt_flat[off + r[q] + 1] = cnts[kk * C + slot];
                if (slot_ids) slot_ids[off + r[q] + 1] = mine[q];  // ids in rank order
            }
        }
    }
}

__global__ void cell_rank_kernel(const uint64_t* __restrict__ calls, int n, int L, int k0, int nk,
                                 const unsigned long long* keys, const uint16_t* rank_slot, int logC,
                                 uint16_t* x, int* err) {
    const size_t C = (size_t)1 << logC, total = (size_t)n * nk;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = t / nk;
        const int kk = (int)(t % nk);
        const unsigned long long v = calls[i * L + k0 + kk];
        uint16_t rk = 0;
        if (v) {
            const unsigned long long* kt = keys + kk * C;
            uint32_t s = hash_slot(v, logC);
            bool found = false;
            for (size_t probe = 0; probe < C; probe++, s = (s + 1) & (uint32_t)(C - 1)) {
                const unsigned long long cur = kt[s];
                if (cur == v) {
                    rk = rank_slot[kk * C + s];
                    found = true;
                    break;
                }
                if (cur == 0) break;
            }
            if (!found) atomicOr(err, DEVERR_TOO_MANY_ALLELES);
        }
        x[i * L + k0 + kk] = rk;
    }
}

// +1.0 at column col of row `row` of a packed e2m1 operand (zeroed before):
// the 32-bit word holding columns 8w .. 8w + 7 gets the nibble by an atomic
// OR, as two columns of one byte belong to different cells.
__device__ __forceinline__ void set_fp4_one(const KChunks& X, size_t row, size_t col) {
    uint32_t* w = reinterpret_cast<uint32_t*>(X.at(row, (int)((col >> 1) & ~(size_t)3)));
    atomicOr(w, kFp4One << (4 * (col & 7)));
}

__global__ void pack_x_kernel(const uint16_t* __restrict__ x, int n, int L, const uint64_t* __restrict__ cnt_off,
                              const int32_t* __restrict__ col_flat, const uint32_t* __restrict__ base, KChunks X) {
    const size_t total = (size_t)n * L;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = t / L;
        const int k = (int)(t % L);
        const int a = x[t];
        if (!a) continue;
        set_fp4_one(X, i, (size_t)k);
        const int32_t c = col_flat[cnt_off[k] + a];
        if (c >= 0) set_fp4_one(X, i, (size_t)L + base[k] + (size_t)c);
    }
}

__global__ void group_fill_kernel(const uint16_t* __restrict__ x, int n, int L, const uint64_t* __restrict__ cnt_off,
                                  const uint64_t* __restrict__ goff, uint32_t* gfill, uint32_t* members) {
    const size_t total = (size_t)n * L;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int a = x[t];
        if (!a) continue;
        const size_t i = t / L;
        const int k = (int)(t % L);
        const uint64_t q = cnt_off[k] + a;
        const uint64_t g0 = goff[q], g1 = goff[q + 1];
        if (g1 > g0) members[g0 + atomicAdd(gfill + q, 1u)] = (uint32_t)i;
    }
}

// One CTA per rare group: rows are distinct, so a row's place is the number
// of smaller rows in the group.  groups holds (first, end, locus) triples;
// mpos (optional, n x L) receives every row's own index in `sorted`.
__global__ void group_sort_kernel(const uint64_t* __restrict__ groups, const uint32_t* __restrict__ members,
                                  uint32_t* sorted, uint32_t* mpos, int L) {
    const uint64_t g0 = groups[3 * blockIdx.x], g1 = groups[3 * blockIdx.x + 1];
    const int locus = (int)groups[3 * blockIdx.x + 2];
    const uint32_t g = (uint32_t)(g1 - g0);
    __shared__ uint32_t tile[4096];
    for (uint32_t e0 = 0; e0 < g; e0 += 4 * blockDim.x) {
        uint32_t mine[4], r[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t e = e0 + q * blockDim.x + threadIdx.x;
            mine[q] = e < g ? members[g0 + e] : 0xFFFFFFFFu;
            r[q] = 0;
        }
        for (uint32_t f0 = 0; f0 < g; f0 += 4096) {
            const uint32_t cntf = min(4096u, g - f0);
            __syncthreads();
            for (uint32_t f = threadIdx.x; f < cntf; f += blockDim.x) tile[f] = members[g0 + f0 + f];
            __syncthreads();
            for (uint32_t f = 0; f < cntf; f++) {
                const uint32_t w = tile[f];
#pragma unroll
                for (int q = 0; q < 4; q++) r[q] += w < mine[q];
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t e = e0 + q * blockDim.x + threadIdx.x;
            if (e < g) {
                sorted[g0 + r[q]] = mine[q];
                if (mpos) mpos[(size_t)mine[q] * L + locus] = (uint32_t)(g0 + r[q]);
            }
        }
    }
}

// Partner runs of every row (one warp per row, loci in order): the members
// after the row's own entry in each of its rare groups, when there are any.
// Pass 0 writes each row's run count; pass 1 the runs' first members, their
// exclusive item prefix within the row, and the row's item total.
__global__ void row_runs_kernel(const uint16_t* __restrict__ x, int n, int L, const uint64_t* __restrict__ cnt_off,
                                const uint64_t* __restrict__ goff, const uint32_t* __restrict__ mpos, int pass,
                                uint32_t* count, const uint64_t* __restrict__ roff, uint32_t* rlo, uint32_t* rpre,
                                uint32_t* rtot) {
    const int lane = threadIdx.x & 31;
    const int warps = (int)(gridDim.x * blockDim.x / 32);
    for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32); i < n; i += warps) {
        uint32_t nrun = 0, items = 0;
        const uint64_t base = pass ? roff[i] : 0;
        for (int k0 = 0; k0 < L; k0 += 32) {
            const int k = k0 + lane;
            uint32_t lo = 0, len = 0;
            if (k < L) {
                const uint32_t mp = mpos[(size_t)i * L + k];
                if (mp != kNoGroup) {
                    const uint64_t g1 = goff[cnt_off[k] + x[(size_t)i * L + k] + 1];
                    if ((uint64_t)mp + 1 < g1) lo = mp + 1, len = (uint32_t)(g1 - mp - 1);
                }
            }
            const unsigned has = __ballot_sync(0xFFFFFFFFu, len > 0);
            if (pass) {
                uint32_t inc = len;  // inclusive warp scan of the run lengths
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, d);
                    if (lane >= d) inc += t;
                }
                if (len) {
                    const uint64_t q = base + nrun + __popc(has & ((1u << lane) - 1u));
                    rlo[q] = lo;
                    rpre[q] = items + inc - len;
                }
                items += __shfl_sync(0xFFFFFFFFu, inc, 31);
            }
            nrun += __popc(has);
        }
        if (lane == 0) {
            if (pass) rtot[i] = items;
            else count[i] = nrun;
        }
    }
}

__device__ __forceinline__ uint64_t lower_bound_rows(const uint32_t* __restrict__ a, uint64_t lo, uint64_t hi,
                                                     uint32_t key) {
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo) / 2;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

constexpr int RR_THREADS = 512;

// Rare partners of each row, ascending with multiplicity.  emit == 0: writes
// the row's partner count to row_count[i]; emit == 1: writes the partners to
// js[start[i] ...].
__global__ void __launch_bounds__(RR_THREADS)
rare_rows_kernel(const uint16_t* __restrict__ x, int n, int L, const uint64_t* __restrict__ cnt_off,
                 const uint64_t* __restrict__ goff, const uint32_t* __restrict__ members, int emit,
                 uint32_t* row_count, const uint64_t* __restrict__ start, uint32_t* js) {
    extern __shared__ uint32_t cw[];  // kJC u16 counters as kJC / 2 words
    __shared__ uint32_t warp_tot[RR_THREADS / 32];
    __shared__ uint64_t chunk_base;
    constexpr int PER = kJC / RR_THREADS;  // counters owned by a thread in the scan
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        if (threadIdx.x == 0) chunk_base = emit ? start[i] : 0;
        uint64_t total = 0;
        for (int c0 = i + 1; c0 < n; c0 += kJC) {
            const int c1 = min(n, c0 + kJC);
            for (int w = threadIdx.x; w < kJC / 2; w += RR_THREADS) cw[w] = 0;
            __syncthreads();
            for (int k = threadIdx.x; k < L; k += RR_THREADS) {
                const int a = x[(size_t)i * L + k];
                if (!a) continue;
                const uint64_t q = cnt_off[k] + a;
                const uint64_t g0 = goff[q], g1 = goff[q + 1];
                if (g1 <= g0) continue;
                // members in batches of 16 independent loads (a dependent load per
                // member leaves the walk latency-bound)
                uint64_t p = lower_bound_rows(members, g0, g1, (uint32_t)c0);
                while (p < g1) {
                    const int m = g1 - p < 16 ? (int)(g1 - p) : 16;
                    uint32_t buf[16];
#pragma unroll
                    for (int q = 0; q < 16; q++) buf[q] = q < m ? members[p + q] : 0xFFFFFFFFu;
                    bool stop = false;
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        if (q < m && !stop) {
                            if (buf[q] >= (uint32_t)c1) {
                                stop = true;
                            } else {
                                const uint32_t o = buf[q] - (uint32_t)c0;
                                atomicAdd(cw + (o >> 1), 1u << (16 * (o & 1)));
                            }
                        }
                    }
                    if (stop) break;
                    p += (uint64_t)m;
                }
            }
            __syncthreads();
            // exclusive scan of the counters in column order
            const uint16_t* cc = reinterpret_cast<const uint16_t*>(cw);
            uint32_t mine = 0;
            const int b = threadIdx.x * PER;
            for (int e = 0; e < PER; e++) mine += cc[b + e];
            uint32_t incl = mine;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += y;
            }
            if (lane == 31) warp_tot[warp] = incl;
            __syncthreads();
            uint32_t before = 0, all = 0;
            for (int w = 0; w < RR_THREADS / 32; w++) {
                if (w < warp) before += warp_tot[w];
                all += warp_tot[w];
            }
            if (emit) {
                uint64_t pos = chunk_base + before + (incl - mine);
                for (int e = 0; e < PER; e++) {
                    const uint32_t c = cc[b + e];
                    for (uint32_t r = 0; r < c; r++) js[pos++] = (uint32_t)(c0 + b + e);
                }
            }
            total += all;
            __syncthreads();
            if (threadIdx.x == 0) chunk_base += all;
            __syncthreads();
        }
        if (!emit && threadIdx.x == 0) row_count[i] = (uint32_t)(total < 0xFFFFFFFFull ? total : 0xFFFFFFFFull);
        __syncthreads();
    }
}

template <class T>
cudaError_t dalloc(T** p, size_t count, size_t* bytes) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess && bytes) *bytes += count * sizeof(T);
    return e;
}

int grid_for(size_t total, int sms) { return (int)std::min<size_t>((total + 255) / 256, (size_t)sms * 32); }

}  // namespace

// One candidate tau: its encoding sizes, device memory and analytic time.
struct TauRow {
    int tau = 0;
    size_t d = 0;             // frequent one-hot columns
    double r = 0, cells = 0;  // rare pairs, cells in rare groups
    double sq = 0;            // sum of squared counts of the alleles that are not frequent
    double kb = 0, mem = 0, t = 0;
    bool fits = false;
};

// Analytic cost of tau on GB300: tensor-core time for the one-hot columns plus
// the rare term (fused pair-list walk, or the dense rare-count build), subject
// to device memory.
std::vector<TauRow> tau_rows(const std::vector<uint32_t>& cnt_flat, const std::vector<uint64_t>& off, int n, int L,
                             size_t free_bytes, const TauModel& m, bool dense) {
    // the candidates are powers of two, so an allele is frequent at tau = 2^t
    // exactly when floor(log2(count)) >= t: one pass bins the counts by that,
    // and every candidate sums whole bins (the sums are integers far below 2^53,
    // exact in double whatever their order)
    constexpr int kBins = 33;
    double bn[kBins] = {}, bsq[kBins] = {}, br[kBins] = {}, bcells[kBins] = {};
    for (int k = 0; k < L; k++)
        for (uint64_t q = off[k] + 1; q < off[k + 1]; q++) {
            const uint32_t c = cnt_flat[q];
            if (!c) continue;
            const int b = 31 - __builtin_clz(c);
            const double v = (double)c;
            bn[b] += 1.0;
            bsq[b] += v * v;
            if (c >= 2) {
                br[b] += v * (v - 1.0) / 2.0;
                bcells[b] += v;
            }
        }
    const double pairs = (double)n * (double)(n - 1) / 2.0;
    const size_t rows = up((size_t)std::max(n, 1), 256);
    const double nl = (double)n * (double)L;
    std::vector<TauRow> out;
    for (int t = 1; (1 << t) <= (dense ? 65536 : 4096); t++) {
        TauRow w;
        w.tau = 1 << t;
        double d = 0;
        for (int b = 0; b < kBins; b++) {
            if (b >= t) {
                d += bn[b];
            } else {
                w.sq += bsq[b];
                w.r += br[b];
                w.cells += bcells[b];
            }
        }
        w.d = (size_t)d;
        w.kb = (double)fp4_columns(L, w.d);  // K: MACs per pair; the two operand copies take K bytes per row
        if (dense) {  // ranks, own positions, group members, row runs (a stripe's counts come later)
            w.mem = (double)rows * w.kb + nl * 6.0 + 12.0 * w.cells + 12.0 * n;
            w.t = pairs * w.kb / m.gemm_rate + w.r / m.dense_rate;
            w.fits = w.mem <= (double)free_bytes && w.cells < 4.0e9;
        } else {
            w.mem = (double)rows * w.kb + 4.0 * (w.r + n + 1.0) + 2.0 * (double)n * (double)up((size_t)n, 8) / 4;
            w.t = pairs * w.kb / m.gemm_rate + w.r / m.rare_rate;
            w.fits = w.mem <= (double)free_bytes && w.r < 4.0e9;
        }
        out.push_back(w);
    }
    return out;
}

int choose_tau_analytic(const std::vector<TauRow>& rows) {
    int best = 0;
    double best_t = 1e300;
    for (const TauRow& w : rows)
        if (w.fits && w.t < best_t) {
            best = w.tau;
            best_t = w.t;
        }
    return best;
}

// Feature rows of the candidates that fit (the layout tch.h documents).
void tau_features(const std::vector<TauRow>& rows, const std::vector<uint32_t>& cnt_flat,
                  const std::vector<uint64_t>& off, int n, int L, TauTable* t) {
    std::vector<double> lnd((size_t)L);
    double present = 0;
    for (int k = 0; k < L; k++) {
        lnd[k] = log1p((double)(off[k + 1] - off[k] - 1));
        for (uint64_t q = off[k] + 1; q < off[k + 1]; q++) present += cnt_flat[q];
    }
    std::sort(lnd.begin(), lnd.end());
    auto quant = [&](double f) { return L ? lnd[(size_t)std::min<double>(L - 1, f * (L - 1) + 0.5)] : 0.0; };
    const double nl = std::max(1.0, (double)n * (double)L);
    const double pairs = std::max(1.0, (double)n * (double)(n - 1) / 2.0);
    const float base[6] = {(float)log((double)std::max(n, 1)), (float)log((double)std::max(L, 1)), (float)quant(0.25),
                           (float)quant(0.5), (float)quant(0.9), (float)(1.0 - present / nl)};
    t->taus.clear();
    t->subs.clear();
    t->groups.clear();
    t->feats.clear();
    t->est_s.clear();
    for (const TauRow& w : rows) {
        if (!w.fits) continue;
        for (int sub : kSchedSubs) {
            if (sub && sub >= n) continue;  // the same as the whole stripe
            for (int grp : kSchedGroups) {
                t->taus.push_back(w.tau);
                t->subs.push_back(sub);
                t->groups.push_back(grp);
                t->est_s.push_back(w.t);
                for (float b : base) t->feats.push_back(b);
                t->feats.push_back((float)log((double)w.tau));
                t->feats.push_back((float)log1p((double)w.d));
                t->feats.push_back((float)log1p(w.r));
                t->feats.push_back((float)log1p(w.cells));
                t->feats.push_back((float)log(pairs * w.kb));
                t->feats.push_back((float)log(std::max(w.t, 1e-9)));
                t->feats.push_back((float)(sub ? log((double)sub / std::max(n, 1)) : 0.0));
                t->feats.push_back((float)log((double)grp));
            }
        }
    }
}

// A database that serves new profiles (ENC_QUERY): tau minimising the time of
// one new profile against all n rows -- the contraction over n rows of kb
// bytes, plus the rare counts, sum over its loci of the group size it hits
// (expected sum of c^2 / n over the alleles that are not frequent).
int choose_tau_query(const std::vector<TauRow>& rows, int n, const TauModel& m, bool verbose) {
    int best = 0;
    double best_t = 1e300;
    for (const TauRow& w : rows) {
        const double t = (double)n * w.kb / m.gemm_rate + w.sq / std::max(n, 1) / m.dense_rate;
        if (verbose)
            fprintf(stderr, "  tau=%5d  one-hot=%8zu  rare items per query %.0f  est %.3f us per query%s\n", w.tau, w.d,
                    w.sq / std::max(n, 1), t * 1e6, w.fits ? "" : "  (does not fit)");
        if (w.fits && t < best_t) {
            best = w.tau;
            best_t = t;
        }
    }
    return best;
}

// tau <= 0: the learned model's pick (tau and schedule) when one is set and
// the set is within the shapes it was trained on, else the analytic tau with
// the default schedule.  *sub / *group receive the schedule (0 = defaults).
// The model's sweep timed sets of up to 63 005 rows, every row counted in one
// rare-count pass; sets wider than a pass (65 536 columns) count their rare
// term in several and take the analytic pick (on 200 000 x 3 000 Zipf profiles
// the learned pick ran 440 ms against the analytic 356 ms).
constexpr int kLearnedMaxRows = 65536;
int choose_tau_gb300(int device, const std::vector<uint32_t>& cnt_flat, const std::vector<uint64_t>& off, int n,
                     int L, size_t free_bytes, const TauModel& m, bool dense, bool verbose, int* sub, int* group) {
    const std::vector<TauRow> rows = tau_rows(cnt_flat, off, n, L, free_bytes, m, dense);
    const int analytic = choose_tau_analytic(rows);
    int learned = 0, lsub = 0, lgroup = 0;
    std::vector<float> pred;
    TauTable t;
    float w[kMlpParams];
    if (n <= kLearnedMaxRows && tau_mlp_weights(w)) {
        tau_features(rows, cnt_flat, off, n, L, &t);
        pred.resize(t.taus.size());
        Err quiet{nullptr, 0};
        if (!t.taus.empty() && !mlp_run(device, w, t.feats.data(), nullptr, (int)t.taus.size(), pred.data(), nullptr,
                                        nullptr, quiet)) {
            float best = INFINITY;
            for (size_t q = 0; q < t.taus.size(); q++)
                if (pred[q] < best) best = pred[q], learned = t.taus[q], lsub = t.subs[q], lgroup = t.groups[q];
        }
    }
    if (verbose) {
        for (const TauRow& r : rows)
            fprintf(stderr, "  tau=%5d  one-hot=%8zu  rare=%14.0f  est %.4fs  vram %.2f GB%s\n", r.tau, r.d, r.r, r.t,
                    r.mem / 1e9, r.fits ? "" : "  (does not fit)");
        fprintf(stderr, "  tau: analytic %d, learned %d (sub-stripes %d rows, raster group %d)\n", analytic, learned,
                lsub, lgroup);
    }
    // the learned pick is taken as it is: the held-out evaluation of the model
    // (tau_learn.py) measures it against the analytic pick on real timings
    *sub = learned ? lsub : 0;
    *group = learned ? lgroup : 0;
    return learned ? learned : analytic;
}

int encode_on_device(int device, int n, int L, const uint64_t* d_calls, int tau_req, const TauModel& model,
                     bool verbose, size_t max_chunk_bytes, int flags, DeviceEncoding* out, Err& e,
                     TauTable* table) {
    const bool dense_rare = (flags & (ENC_DENSE | ENC_QUERY)) != 0;
    const bool query_maps = (flags & ENC_QUERY) != 0;
    int sms = 0, hflag = 0;
    size_t freeb = 0, totb = 0, tmp_bytes = 0;
    int logC = 10;
    while (((size_t)1 << logC) < 2 * (size_t)std::min<int>(std::max(n, 1), (int)kMaxDistinct)) logC++;
    const size_t C = (size_t)1 << logC;
    // loci per batch: hash tables + id lists within ~2 GB
    const uint32_t lcap = (uint32_t)std::min<int>(std::max(n, 1), (int)kMaxDistinct);
    const size_t per_locus = C * (8 + 4 + 2) + (size_t)lcap * 12;
    const int nk_max = (int)std::max<size_t>(1, std::min<size_t>((size_t)L, ((size_t)2 << 30) / per_locus));
    unsigned long long* keys = nullptr;
    uint32_t *cnts = nullptr, *nd = nullptr, *list_slots = nullptr, *cnt_flat = nullptr, *gfill = nullptr;
    uint32_t *members = nullptr, *sorted = nullptr, *row_count = nullptr, *base_d = nullptr, *mpos = nullptr;
    uint16_t* rank_slot = nullptr;
    unsigned long long* list_keys = nullptr;
    uint64_t *cnt_off_d = nullptr, *goff_d = nullptr, *groups_d = nullptr, *start64 = nullptr;
    int32_t* col_d = nullptr;
    unsigned long long* slot_ids = nullptr;
    int* err_d = nullptr;
    std::vector<uint32_t> nd_h(L), cnt_h;
    std::vector<uint64_t> off_h((size_t)L + 1, 0);
    *out = DeviceEncoding();
    out->n = n;
    out->L = L;
    // phase times (with a device sync at each mark) when verbose
    double t_mark = 0;
    auto mark = [&](const char* phase) {
        if (!verbose) return;
        cudaDeviceSynchronize();
        const double t = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
        if (t_mark > 0) fprintf(stderr, "tch encoder: %-26s %8.1f ms\n", phase, (t - t_mark) * 1e3);
        t_mark = t;
    };
    mark("start");

    TCH_CK(e, cudaSetDevice(device));
    TCH_CK(e, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    TCH_CK(e, dalloc(&err_d, 1, nullptr));
    TCH_CK(e, cudaMemset(err_d, 0, sizeof(int)));
    TCH_CK(e, dalloc(&nd, (size_t)L, nullptr));
    TCH_CK(e, cudaMemset(nd, 0, (size_t)L * 4));
    TCH_CK(e, dalloc(&out->x, (size_t)n * L, &out->bytes));
    TCH_CK(e, dalloc(&keys, C * nk_max, &tmp_bytes));
    TCH_CK(e, dalloc(&cnts, C * nk_max, &tmp_bytes));
    TCH_CK(e, dalloc(&rank_slot, C * nk_max, &tmp_bytes));
    TCH_CK(e, dalloc(&list_keys, (size_t)lcap * nk_max, &tmp_bytes));
    TCH_CK(e, dalloc(&list_slots, (size_t)lcap * nk_max, &tmp_bytes));
    TCH_CK(e, dalloc(&cnt_off_d, (size_t)L + 1, nullptr));

    // ---- 1-3: ranks and counts, batch by batch
    {
        std::vector<uint32_t> cnt_parts;
        for (int k0 = 0; k0 < L; k0 += nk_max) {
            const int nk = std::min(nk_max, L - k0);
            TCH_CK(e, cudaMemset(keys, 0, C * nk * sizeof(unsigned long long)));
            TCH_CK(e, cudaMemset(cnts, 0, C * nk * sizeof(uint32_t)));
            insert_kernel<<<grid_for((size_t)n * nk, sms), 256>>>(d_calls, n, L, k0, nk, keys, cnts, logC, nd, err_d);
            TCH_CK(e, cudaGetLastError());
            TCH_CK(e, cudaMemcpy(nd_h.data() + k0, nd + k0, (size_t)nk * 4, cudaMemcpyDeviceToHost));
            TCH_CK(e, cudaMemcpy(&hflag, err_d, sizeof(int), cudaMemcpyDeviceToHost));
            if (hflag) { e.set("a locus has more than 65535 distinct alleles (limit 65535)"); goto fail; }
            for (int kk = 0; kk < nk; kk++) {
                if (nd_h[k0 + kk] > kMaxDistinct) {
                    e.set("locus %d has %u distinct alleles (limit 65535)", k0 + kk, nd_h[k0 + kk]);
                    goto fail;
                }
                off_h[k0 + kk + 1] = off_h[k0 + kk] + nd_h[k0 + kk] + 1;
            }
        }
        // flat counts need every offset: a second sweep ranks the batches
        TCH_CK(e, cudaMemcpy(cnt_off_d, off_h.data(), ((size_t)L + 1) * 8, cudaMemcpyHostToDevice));
        TCH_CK(e, dalloc(&cnt_flat, off_h[L], &tmp_bytes));
        TCH_CK(e, cudaMemset(cnt_flat, 0, std::max<uint64_t>(off_h[L], 1) * 4));
        if (query_maps) {
            TCH_CK(e, dalloc(&slot_ids, off_h[L], nullptr));
            TCH_CK(e, cudaMemset(slot_ids, 0, std::max<uint64_t>(off_h[L], 1) * 8));
        }
        const bool one_batch = nk_max >= L;  // the first sweep's tables are still in place
        if (!one_batch) TCH_CK(e, cudaMemset(nd, 0, (size_t)L * 4));
        for (int k0 = 0; k0 < L; k0 += nk_max) {
            const int nk = std::min(nk_max, L - k0);
            if (!one_batch) {
                TCH_CK(e, cudaMemset(keys, 0, C * nk * sizeof(unsigned long long)));
                TCH_CK(e, cudaMemset(cnts, 0, C * nk * sizeof(uint32_t)));
                insert_kernel<<<grid_for((size_t)n * nk, sms), 256>>>(d_calls, n, L, k0, nk, keys, cnts, logC, nd,
                                                                       err_d);
                TCH_CK(e, cudaGetLastError());
            }
            rank_kernel<<<nk, 512>>>(k0, keys, cnts, logC, nd, cnt_off_d, cnt_flat, rank_slot, list_keys, list_slots,
                                     slot_ids, lcap, err_d);
            TCH_CK(e, cudaGetLastError());
            cell_rank_kernel<<<grid_for((size_t)n * nk, sms), 256>>>(d_calls, n, L, k0, nk, keys, rank_slot, logC,
                                                                      out->x, err_d);
            TCH_CK(e, cudaGetLastError());
        }
        TCH_CK(e, cudaMemcpy(&hflag, err_d, sizeof(int), cudaMemcpyDeviceToHost));
        if (hflag) { e.set("device encoder: hash table error 0x%x", hflag); goto fail; }
        cnt_h.resize(off_h[L]);
        if (off_h[L]) TCH_CK(e, cudaMemcpy(cnt_h.data(), cnt_flat, off_h[L] * 4, cudaMemcpyDeviceToHost));
    }
    cudaFree(keys); keys = nullptr;
    cudaFree(cnts); cnts = nullptr;
    cudaFree(rank_slot); rank_slot = nullptr;
    cudaFree(list_keys); list_keys = nullptr;
    cudaFree(list_slots); list_slots = nullptr;

    mark("ranks and counts");
    // ---- host: tau, frequent columns, rare groups
    {
        int tau = tau_req;
        TCH_CK(e, cudaMemGetInfo(&freeb, &totb));
        if (table) {  // candidates and features only
            tau_features(tau_rows(cnt_h, off_h, n, L, freeb, model, dense_rare), cnt_h, off_h, n, L, table);
            free_device_encoding(out);
            goto done;
        }
        if (tau <= 0) {
            tau = query_maps ? choose_tau_query(tau_rows(cnt_h, off_h, n, L, freeb, model, true), n, model, verbose)
                             : choose_tau_gb300(device, cnt_h, off_h, n, L, freeb, model, dense_rare, verbose,
                                                &out->sub_rows, &out->tile_group);
            if (!tau) { e.set("no tau fits in %.2f GB of free device memory", freeb / 1e9); goto fail; }
        }
        out->tau = tau;
        std::vector<int32_t> col(off_h[L], -1);
        std::vector<uint32_t> base((size_t)L + 1, 0);
        std::vector<uint64_t> goff(off_h[L] + 1, 0);
        std::vector<uint64_t> groups;  // (first, end, locus) of every rare group
        double n_rare_pairs = 0;
        uint64_t D = 0;
        for (int k = 0; k < L; k++) {
            base[k] = (uint32_t)D;
            uint32_t d = 0;
            for (uint64_t q = off_h[k]; q < off_h[k + 1]; q++) {
                const bool is_rank = q > off_h[k];
                const uint32_t c = cnt_h[q];
                const bool freq = is_rank && c >= (uint32_t)tau;
                if (freq) col[q] = (int32_t)d++;
                // a query database also keeps single-row groups: a new profile with that
                // allele equals its one row
                const bool rare = is_rank && !freq && c >= (query_maps ? 1u : 2u);
                goff[q + 1] = goff[q] + (rare ? c : 0);
                if (rare) {
                    groups.push_back(goff[q]);
                    groups.push_back(goff[q + 1]);
                    groups.push_back((uint64_t)k);
                    n_rare_pairs += (double)c * (double)(c - 1) / 2.0;
                }
            }
            D += d;
        }
        base[L] = (uint32_t)D;
        out->D = D;
        if (fp4_columns(L, D) / 2 > (size_t)INT32_MAX) { e.set("%llu one-hot columns: too many", (unsigned long long)D); goto fail; }
        out->kb = (int)(fp4_columns(L, D) / 2);
        out->x_rows = up((size_t)std::max(n, 1), 256);
        const uint64_t n_members = goff[off_h[L]];
        if (dense_rare && n_members >= (1ull << 32)) {
            e.set("%llu rare cells: more than 2^32 (lower tau)", (unsigned long long)n_members);
            goto fail;
        }
        TCH_CK(e, dalloc(&col_d, off_h[L], nullptr));
        TCH_CK(e, dalloc(&base_d, (size_t)L + 1, nullptr));
        TCH_CK(e, dalloc(&goff_d, off_h[L] + 1, nullptr));
        if (off_h[L]) TCH_CK(e, cudaMemcpy(col_d, col.data(), off_h[L] * 4, cudaMemcpyHostToDevice));
        TCH_CK(e, cudaMemcpy(base_d, base.data(), ((size_t)L + 1) * 4, cudaMemcpyHostToDevice));
        TCH_CK(e, cudaMemcpy(goff_d, goff.data(), (off_h[L] + 1) * 8, cudaMemcpyHostToDevice));

        mark("tau and column maps");
        // ---- 4: operand rows: pos by nibble, neg from pos
        {
            if (!chunk_width_for(out->kb, out->x_rows, max_chunk_bytes)) {
                e.set("the operand needs more than %d K chunks of %zu bytes", kMaxKChunks, max_chunk_bytes);
                goto fail;
            }
            TCH_CK(e, alloc_fp4(&out->X, out->x_rows, out->kb, max_chunk_bytes, true, true, &out->bytes));
            for (int c = 0; c < out->X.pos.n; c++)
                TCH_CK(e, cudaMemset(out->X.pos.p[c], 0, out->x_rows * (size_t)out->X.pos.width_of(c)));
        }
        pack_x_kernel<<<grid_for((size_t)n * L, sms), 256>>>(out->x, n, L, cnt_off_d, col_d, base_d, out->X.pos);
        TCH_CK(e, cudaGetLastError());
        TCH_CK(e, launch_negate_onehot(out->X, L, 0));

        mark("operand rows");
        // ---- 5: rare groups, sorted
        const size_t ngroups = groups.size() / 3;
        TCH_CK(e, dalloc(&members, n_members, &tmp_bytes));
        TCH_CK(e, dalloc(&sorted, n_members, &tmp_bytes));
        TCH_CK(e, dalloc(&gfill, off_h[L], &tmp_bytes));
        TCH_CK(e, cudaMemset(gfill, 0, std::max<uint64_t>(off_h[L], 1) * 4));
        if (dense_rare) {  // cells in no rare group keep the sentinel: the rare counts skip them
            TCH_CK(e, dalloc(&mpos, (size_t)n * L, &tmp_bytes));
            TCH_CK(e, cudaMemset(mpos, 0xFF, std::max<size_t>((size_t)n * L, 1) * 4));
        }
        if (ngroups) {
            TCH_CK(e, dalloc(&groups_d, groups.size(), &tmp_bytes));
            TCH_CK(e, cudaMemcpy(groups_d, groups.data(), groups.size() * 8, cudaMemcpyHostToDevice));
            group_fill_kernel<<<grid_for((size_t)n * L, sms), 256>>>(out->x, n, L, cnt_off_d, goff_d, gfill, members);
            TCH_CK(e, cudaGetLastError());
            for (size_t g0 = 0; g0 < ngroups; g0 += 65535) {
                const unsigned gcount = (unsigned)std::min<size_t>(65535, ngroups - g0);
                group_sort_kernel<<<gcount, 256>>>(groups_d + 3 * g0, members, sorted, mpos, L);
                TCH_CK(e, cudaGetLastError());
            }
        }

        mark("rare groups");
        if (dense_rare && !query_maps && n > 1) {  // the partner runs of every row, for triangle solves
            TCH_CK(e, dalloc(&row_count, (size_t)n, &tmp_bytes));
            const int rgrid = (int)std::min<size_t>(((size_t)n + 7) / 8, (size_t)sms * 16);
            row_runs_kernel<<<rgrid, 256>>>(out->x, n, L, cnt_off_d, goff_d, mpos, 0, row_count, nullptr, nullptr,
                                            nullptr, nullptr);
            TCH_CK(e, cudaGetLastError());
            std::vector<uint32_t> rc_h((size_t)n);
            TCH_CK(e, cudaMemcpy(rc_h.data(), row_count, (size_t)n * 4, cudaMemcpyDeviceToHost));
            std::vector<uint64_t> roff_h((size_t)n + 1);
            uint64_t acc = 0;
            for (int i = 0; i < n; i++) roff_h[i] = acc, acc += rc_h[i];
            roff_h[n] = acc;
            TCH_CK(e, dalloc(&out->roff, (size_t)n + 1, &out->bytes));
            TCH_CK(e, dalloc(&out->rlo, std::max<uint64_t>(acc, 1), &out->bytes));
            TCH_CK(e, dalloc(&out->rpre, std::max<uint64_t>(acc, 1), &out->bytes));
            TCH_CK(e, dalloc(&out->rtot, (size_t)n, &out->bytes));
            TCH_CK(e, cudaMemcpy(out->roff, roff_h.data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
            row_runs_kernel<<<rgrid, 256>>>(out->x, n, L, cnt_off_d, goff_d, mpos, 1, nullptr, out->roff, out->rlo,
                                            out->rpre, out->rtot);
            TCH_CK(e, cudaGetLastError());
            mark("row runs");
        }
        if (dense_rare) {  // the groups themselves are the rare term; no pair list
            TCH_CK(e, cudaDeviceSynchronize());
            out->dense = true;
            out->n_rare = (size_t)n_rare_pairs;
            out->cnt_off = cnt_off_d;
            out->goff = goff_d;
            out->members = sorted;
            out->mpos = mpos;
            out->bytes += ((size_t)L + 1) * 8 + (off_h[L] + 1) * 8 + n_members * 4 + (size_t)n * L * 4;
            if (query_maps) {  // what new profiles need to be encoded like these
                out->slot_ids = reinterpret_cast<uint64_t*>(slot_ids);
                out->col = col_d;
                out->base = base_d;
                out->bytes += off_h[L] * 12 + ((size_t)L + 1) * 4;
                slot_ids = nullptr;
                col_d = nullptr;
                base_d = nullptr;
            }
            cnt_off_d = nullptr;
            goff_d = nullptr;
            sorted = nullptr;
            mpos = nullptr;
            goto done;
        }
        // ---- 6: CSR of rare pairs, ascending per row
        TCH_CK(e, dalloc(&row_count, (size_t)n, &tmp_bytes));
        TCH_CK(e, dalloc(&start64, (size_t)n + 1, &tmp_bytes));
        const int rr_smem = kJC * 2;
        TCH_CK(e, cudaFuncSetAttribute(rare_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, rr_smem));
        const int rr_grid = std::max(1, std::min(n, sms * 1));
        if (ngroups && n > 1) {
            rare_rows_kernel<<<rr_grid, RR_THREADS, rr_smem>>>(out->x, n, L, cnt_off_d, goff_d, sorted, 0, row_count,
                                                              nullptr, nullptr);
            TCH_CK(e, cudaGetLastError());
        } else {
            TCH_CK(e, cudaMemset(row_count, 0, (size_t)std::max(n, 1) * 4));
        }
        std::vector<uint32_t> rc_h((size_t)n);
        if (n) TCH_CK(e, cudaMemcpy(rc_h.data(), row_count, (size_t)n * 4, cudaMemcpyDeviceToHost));
        std::vector<uint32_t> start_h((size_t)n + 1);
        std::vector<uint64_t> start64_h((size_t)n + 1);
        uint64_t acc = 0;
        for (int i = 0; i < n; i++) {
            start_h[i] = (uint32_t)acc;
            start64_h[i] = acc;
            acc += rc_h[i];
            if (acc >= (1ull << 32)) { e.set("too many rare pairs: raise --tau"); goto fail; }
        }
        start_h[n] = (uint32_t)acc;
        start64_h[n] = acc;
        out->n_rare = acc;
        TCH_CK(e, dalloc(&out->start, (size_t)n + 1, &out->bytes));
        TCH_CK(e, dalloc(&out->js, acc, &out->bytes));
        TCH_CK(e, cudaMemcpy(out->start, start_h.data(), ((size_t)n + 1) * 4, cudaMemcpyHostToDevice));
        TCH_CK(e, cudaMemcpy(start64, start64_h.data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
        if (acc) {
            rare_rows_kernel<<<rr_grid, RR_THREADS, rr_smem>>>(out->x, n, L, cnt_off_d, goff_d, sorted, 1, nullptr,
                                                              start64, out->js);
            TCH_CK(e, cudaGetLastError());
        }
        TCH_CK(e, cudaDeviceSynchronize());
        mark("rare CSR (2 passes)");
    }
done:
    cudaFree(err_d); cudaFree(nd); cudaFree(cnt_off_d); cudaFree(cnt_flat); cudaFree(col_d); cudaFree(base_d);
    cudaFree(goff_d); cudaFree(members); cudaFree(sorted); cudaFree(gfill); cudaFree(groups_d); cudaFree(row_count);
    cudaFree(start64); cudaFree(mpos); cudaFree(slot_ids);
    return 0;
fail:
    cudaFree(err_d); cudaFree(nd); cudaFree(cnt_off_d); cudaFree(cnt_flat); cudaFree(col_d); cudaFree(base_d);
    cudaFree(goff_d); cudaFree(members); cudaFree(sorted); cudaFree(gfill); cudaFree(groups_d); cudaFree(row_count);
    cudaFree(start64); cudaFree(keys); cudaFree(cnts); cudaFree(rank_slot); cudaFree(list_keys); cudaFree(list_slots);
    cudaFree(mpos); cudaFree(slot_ids);
    free_device_encoding(out);
    return 1;
}

void free_device_encoding(DeviceEncoding* d) {
    cudaFree(d->x);
    free_fp4(&d->X);
    cudaFree(d->start);
    cudaFree(d->js);
    cudaFree(d->cnt_off);
    cudaFree(d->goff);
    cudaFree(d->members);
    cudaFree(d->mpos);
    cudaFree(d->roff);
    cudaFree(d->rlo);
    cudaFree(d->rpre);
    cudaFree(d->rtot);
    d->roff = nullptr;
    d->rlo = d->rpre = d->rtot = nullptr;
    cudaFree(d->slot_ids);
    cudaFree(d->col);
    cudaFree(d->base);
    d->slot_ids = nullptr;
    d->col = nullptr;
    d->base = nullptr;
    d->x = nullptr;
    d->X = Fp4Operands();
    d->start = d->js = nullptr;
    d->cnt_off = d->goff = nullptr;
    d->members = d->mpos = nullptr;
}

}  // namespace tch
