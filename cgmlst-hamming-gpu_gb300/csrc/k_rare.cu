// Dense rare counts of a stripe, built on the device from the rare groups.
//
// The rare term R[i, j] = #{loci k : x[i,k] == x[j,k] != 0 and that allele is
// rare} (the reference applies it pair by pair from the host-built lists,
// tensorcore/rs/src/main.rs:416-447 and tensorcore/rs/cuda/tch.cu:31-38).
// Here the encoder keeps every rare allele as a group of rows (ascending)
// plus each row's own place in its groups; row i's partners at locus k are
// the group members after its own entry.  Per stripe this kernel counts them
// into a u16 block laid out like the output, which the tensor-core epilogue
// subtracts with 16-byte loads: no pair list is ever materialised.
//
// One CTA per stripe row (persistent over the rows).  The counters of the
// row's columns sit in shared memory as u16 pairs (65536 columns per pass),
// each partner adds 1 with a shared atomic, and the finished row is written
// out with coalesced 16-byte stores.  The partner runs of up to 2048 loci are
// laid end to end by a block-wide scan of their lengths and cut into 32 equal
// parts, one per warp, so every warp of the CTA has the same number of
// partners whatever the group sizes are; a warp walks its part run by run
// with its lanes on consecutive members (coalesced loads, up to eight in
// flight per lane).

#include <climits>

#include "tch_internal.cuh"

namespace tch {
namespace {

#ifndef TCH_RARE_NARROW_T
#define TCH_RARE_NARROW_T 128
#endif
constexpr int NT = TCH_RARE_NARROW_T;      // threads per CTA of the narrow-row kernels (one row each)
constexpr int RD_WORDS = 32768;          // u32 counter words in shared memory (128 KB): 65 536 columns per pass

// Counter words a launch needs (a narrow stripe takes less shared memory, so
// more CTAs fit on an SM when several solves run side by side).
inline int counter_words(size_t width) { return (int)std::min<size_t>(RD_WORDS, width / 2); }
template <int T>
inline int rd_smem(int cwords) { return cwords * 4 + (2 * T + 1) * 4 + 2 * T * 4 + 64 * 4; }
constexpr unsigned FULL = 0xFFFFFFFFu;

__device__ __forceinline__ uint64_t lower_bound_m(const uint32_t* __restrict__ m, uint64_t lo, uint64_t hi,
                                                  uint32_t key) {
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo) / 2;
        if (__ldg(m + mid) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Partner run of row i at locus k inside columns [jlo, jhi): members[lo, lo +
// len).  a = x[i, k], mp = mpos[i, k], coff = cnt_off[k], loaded by the caller.
__device__ __forceinline__ uint32_t partner_run(const RareGroups& g, int i, uint32_t a, uint32_t mp, uint64_t coff,
                                                uint32_t jlo, uint32_t jhi, uint32_t* lo_out) {
    if (!a || mp == kNoGroup) return 0;  // missing, or in no rare group: no lookup at all
    const uint64_t g1 = __ldg(g.goff + coff + a + 1);
    uint64_t b = (uint64_t)mp + 1, e = g1;  // empty when i is the group's last member
    if (b >= e) return 0;
    // members after i's own entry are > i; clip to the pass's columns (only a
    // pass that starts after i + 1 or ends before n needs it)
    if (jlo > (uint32_t)i + 1 && b < e && __ldg(g.members + b) < jlo) b = lower_bound_m(g.members, b, e, jlo);
    if (jhi < (uint32_t)g.n && b < e && __ldg(g.members + e - 1) >= jhi) e = lower_bound_m(g.members, b, e, jhi);
    *lo_out = (uint32_t)b;
    return (uint32_t)(e - b);
}

// This thread's two loci of a row: ranks and own positions.
struct CellPair {
    uint32_t a0 = 0, a1 = 0, m0 = 0, m1 = 0;
};

__device__ __forceinline__ CellPair load_cells(const RareGroups& g, int i, int k0) {
    CellPair c;
    const size_t base = (size_t)i * g.L + k0;
    if (k0 < g.L) {
        c.a0 = g.x[base];
        c.m0 = g.mpos[base];
    }
    if (k0 + 1 < g.L) {
        c.a1 = g.x[base + 1];
        c.m1 = g.mpos[base + 1];
    }
    return c;
}

// A part whose runs hold this many items on average is walked run by run
// (measured on the long-tail profiles: 256 beats 0, 64, 1024 and never).
constexpr uint32_t kWalkMin = 256;

__device__ __forceinline__ void count_col(uint32_t* cnt, uint32_t c) {
    atomicAdd(cnt + (c >> 1), 1u << ((c & 1u) * 16u));
}

// Items [e_begin, e_end) of runs laid end to end (run q: items pre[q] ..
// pre[q + 1] - 1, members run[q] ..; pre[nr] bounds the last one), counted at
// column j - wb by one warp.  A part of long runs (kWalkMin items or more on
// average) is walked run by run, the lanes on consecutive members; otherwise
// 256 items at a time, lane l on items e + l + 32 u, several short runs in one
// pass, each lane keeping its current run (start, end, first member) in
// registers.
__device__ __forceinline__ void walk_part(uint32_t* cnt, const uint32_t* pre, const uint32_t* run, int nr,
                                          uint32_t e_begin, uint32_t e_end, const uint32_t* __restrict__ members,
                                          int wb, int lane) {
    if (e_begin >= e_end) return;
    int p = 0;  // the run holding e_begin: the last p with pre[p] <= e_begin
    {
        int hi = nr;
        while (hi - p > 1) {
            const int m = (p + hi) >> 1;
            if (pre[m] <= e_begin) p = m; else hi = m;
        }
    }
    // long runs on average: walk run by run, the lanes on consecutive members
    // with no per-item bookkeeping
    int pe = p;  // the run holding e_end - 1
    {
        int hi = nr;
        while (hi - pe > 1) {
            const int m = (pe + hi) >> 1;
            if (pre[m] <= e_end - 1) pe = m; else hi = m;
        }
    }
    if ((e_end - e_begin) >= kWalkMin * (uint32_t)(pe - p + 1)) {
        uint32_t e = e_begin;
        for (int q = p; e < e_end; q++) {
            const uint32_t stop = min(pre[q + 1], e_end);
            const uint32_t* src = members + run[q] + (e - pre[q]);
            const uint32_t c = stop - e;
            uint32_t k = (uint32_t)lane;
            for (; k + 224 < c; k += 256) {  // eight loads in flight per lane
                uint32_t jj[8];
#pragma unroll
                for (int u = 0; u < 8; u++) jj[u] = __ldg(src + k + 32 * u);
#pragma unroll
                for (int u = 0; u < 8; u++) count_col(cnt, jj[u] - (uint32_t)wb);
            }
            if (k + 96 < c) {
                uint32_t jj[4];
#pragma unroll
                for (int u = 0; u < 4; u++) jj[u] = __ldg(src + k + 32 * u);
#pragma unroll
                for (int u = 0; u < 4; u++) count_col(cnt, jj[u] - (uint32_t)wb);
                k += 128;
            }
            for (; k < c; k += 32) count_col(cnt, __ldg(src + k) - (uint32_t)wb);
            e = stop;
        }
        return;
    }
    uint32_t a = pre[p], b = pre[p + 1], r = run[p];  // this lane's current run
    uint32_t e0 = e_begin;
    for (; e0 + 256 <= e_end; e0 += 256) {  // whole batches: no bounds checks
        uint32_t j[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const uint32_t e = e0 + (uint32_t)(u * 32 + lane);
            while (e >= b) {  // next run (pre[nr] = total > e bounds it)
                ++p;
                a = b;
                b = pre[p + 1];
                r = run[p];
            }
            j[u] = __ldg(members + r + (e - a));
        }
#pragma unroll
        for (int u = 0; u < 8; u++) count_col(cnt, j[u] - (uint32_t)wb);
    }
    for (; e0 < e_end; e0 += 256) {  // the last, partial batch
        uint32_t idx[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const uint32_t e = e0 + (uint32_t)(u * 32 + lane);
            idx[u] = 0xFFFFFFFFu;
            if (e < e_end) {
                while (e >= b) {  // next run (pre[nr] = total > e bounds it)
                    ++p;
                    a = b;
                    b = pre[p + 1];
                    r = run[p];
                }
                idx[u] = r + (e - a);
            }
        }
        uint32_t j[8];
#pragma unroll
        for (int u = 0; u < 8; u++) j[u] = idx[u] != 0xFFFFFFFFu ? __ldg(members + idx[u]) : 0u;
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (idx[u] != 0xFFFFFFFFu) count_col(cnt, j[u] - (uint32_t)wb);
    }
}

// Lays this thread's two runs (l0 partners from members[lo0], l1 from
// members[lo1]) end to end with every other thread's non-empty runs (a block
// scan of item and run counts compacts them), cuts the items into one equal
// part per warp, and counts every partner j at column j - wb (walk_part).
// Called by all threads of the CTA (it synchronises them).
template <int T>
__device__ __forceinline__ void count_runs(uint32_t* cnt, uint32_t* pre, uint32_t* run, uint32_t* wsum, uint32_t l0,
                                           uint32_t lo0, uint32_t l1, uint32_t lo1,
                                           const uint32_t* __restrict__ members, int wb) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NWARPS = T / 32;
    __shared__ uint32_t tot[2];  // items, runs
    const uint32_t mi = l0 + l1, mc = (l0 ? 1u : 0u) + (l1 ? 1u : 0u);
    uint32_t ii = mi, ic = mc;  // inclusive warp scans of items and runs
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t ti = __shfl_up_sync(FULL, ii, d), tc = __shfl_up_sync(FULL, ic, d);
        if (lane >= d) ii += ti, ic += tc;
    }
    if (lane == 31) wsum[warp] = ii, wsum[32 + warp] = ic;
    __syncthreads();  // also orders the counter zeroing and the previous chunk's readers
    if (warp == 0) {
        const uint32_t vi = lane < NWARPS ? wsum[lane] : 0u, vc = lane < NWARPS ? wsum[32 + lane] : 0u;
        uint32_t xi = vi, xc = vc;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t ti = __shfl_up_sync(FULL, xi, d), tc = __shfl_up_sync(FULL, xc, d);
            if (lane >= d) xi += ti, xc += tc;
        }
        if (lane < NWARPS) wsum[lane] = xi - vi, wsum[32 + lane] = xc - vc;
        if (lane == 31) tot[0] = xi, tot[1] = xc;
    }
    __syncthreads();
    {
        const uint32_t ei = wsum[warp] + ii - mi;        // items before this thread's runs
        uint32_t q = wsum[32 + warp] + ic - mc;          // their places among the non-empty runs
        if (l0) pre[q] = ei, run[q] = lo0, q++;
        if (l1) pre[q] = ei + l0, run[q] = lo1;
        if (tid == 0) pre[tot[1]] = tot[0];
    }
    __syncthreads();
    const uint32_t total = tot[0];
    const uint32_t part = (total + NWARPS - 1) / NWARPS;
    const uint32_t e_begin = min(total, (uint32_t)warp * part), e_end = min(total, e_begin + part);
    walk_part(cnt, pre, run, (int)tot[1], e_begin, e_end, members, wb, lane);
}

// Row i's partners from its precomputed runs (RareGroups::roff ..), counted
// at column j - wb: up to 2T runs at a time are copied into pre / run
// (coalesced), their items cut into one equal part per warp and walked.  The
// row's partners must all lie in this pass's columns.  Called by all threads
// of the CTA after the counters are zeroed (it synchronises them).
template <int T>
__device__ __forceinline__ void count_row_runs(uint32_t* cnt, uint32_t* pre, uint32_t* run, const RareGroups& g, int i,
                                               int wb) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NWARPS = T / 32;
    const uint64_t q0 = g.roff[i];
    const uint32_t nrun = (uint32_t)(g.roff[i + 1] - q0);
    for (uint32_t c0 = 0; c0 < nrun; c0 += 2 * T) {
        const uint32_t cn = min(2u * T, nrun - c0);
        __syncthreads();  // the zeroing, or the previous group of runs' readers
        for (uint32_t t = tid; t < cn; t += T) {
            pre[t] = __ldg(g.rpre + q0 + c0 + t);
            run[t] = __ldg(g.rlo + q0 + c0 + t);
        }
        if (tid == 0) pre[cn] = c0 + cn < nrun ? __ldg(g.rpre + q0 + c0 + cn) : __ldg(g.rtot + i);
        __syncthreads();
        const uint32_t base = pre[0], total = pre[cn] - base;
        const uint32_t part = (total + NWARPS - 1) / NWARPS;
        const uint32_t e_begin = base + min(total, (uint32_t)warp * part);
        const uint32_t e_end = base + min(total, (uint32_t)warp * part + part);
        walk_part(cnt, pre, run, (int)cn, e_begin, e_end, g.members, wb, lane);
    }
}

// Many sets' whole triangles in one launch (batched solves): the rows of
// every job laid end to end (row_job: the job of every row), one CTA per row
// as in rare_dense_kernel, each row counted in one pass (the launcher checks
// that every job's width fits the counters).
struct RareJob {
    RareGroups g;
    uint16_t* R;
    size_t ldr;
    int cend;  // up(n, 256): the job's stripe is its whole triangle (r0 = 0)
    int row0;  // the job's first row in the launch
};

template <int T>
__global__ void __launch_bounds__(T, 1024 / T)
    rare_batch_kernel(const RareJob* __restrict__ jobs, const int* __restrict__ row_job, int total_rows,
                      int cwords) {
    extern __shared__ uint4 smem_rd[];
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem_rd);
    uint32_t* pre = cnt + cwords;
    uint32_t* run = pre + (2 * T) + 1;
    uint32_t* wsum = run + (2 * T);
    const int tid = threadIdx.x;
    for (int gr = blockIdx.x; gr < total_rows; gr += gridDim.x) {
        const RareJob& jb = jobs[__ldg(row_job + gr)];
        const RareGroups g = jb.g;
        const int i = gr - jb.row0;
        const int n = g.n, L = g.L;
        const int cbeg = i & ~(kRareDenseAlign - 1);  // first column of the row's diagonal tile
        const int nq = (jb.cend - cbeg) >> 3;
        for (int w = tid; w < nq; w += T) smem_rd[w] = make_uint4(0, 0, 0, 0);
        const uint32_t jlo = (uint32_t)(i + 1), jhi = (uint32_t)n;
        if (g.roff) {  // the row's precomputed runs
            count_row_runs<T>(cnt, pre, run, g, i, cbeg);
        } else {
            for (int kc = 0; jlo < jhi && kc < L; kc += (2 * T)) {
                const int k0 = kc + 2 * tid;
                uint32_t lo0 = 0, lo1 = 0, l0 = 0, l1 = 0;
                const CellPair c = load_cells(g, i, k0);
                if (k0 < L) l0 = partner_run(g, i, c.a0, c.m0, g.cnt_off[k0], jlo, jhi, &lo0);
                if (k0 + 1 < L) l1 = partner_run(g, i, c.a1, c.m1, g.cnt_off[k0 + 1], jlo, jhi, &lo1);
                count_runs<T>(cnt, pre, run, wsum, l0, lo0, l1, lo1, g.members, cbeg);
            }
        }
        __syncthreads();
        uint4* dst = reinterpret_cast<uint4*>(jb.R + (size_t)i * jb.ldr + (size_t)cbeg);
        for (int w = tid; w < nq; w += T) dst[w] = smem_rd[w];
        __syncthreads();
    }
}

template <int T>
__global__ void __launch_bounds__(T, 1024 / T)
    rare_dense_kernel(const RareGroups g, int r0, int rows, uint16_t* __restrict__ R, size_t ldr, int cend,
                      int cwords) {
    extern __shared__ uint4 smem_rd[];
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem_rd);
    uint32_t* pre = cnt + cwords;          // 2T + 1: exclusive prefix of the run lengths
    uint32_t* run = pre + (2 * T) + 1;     // 2T: first member index of each run
    uint32_t* wsum = run + (2 * T);        // 64: per-warp totals of the scans
    const int tid = threadIdx.x;
    const int n = g.n, L = g.L;
    // with every locus in one scan (L <= 2T) a thread keeps the same two
    // loci for all rows: their count offsets stay in registers and the next
    // row's ranks and positions are fetched while this row is counted
    // the rows' precomputed runs, when there are any and every row's partners
    // fit one counter pass; otherwise the runs are found per locus
    const bool row_runs = g.roff != nullptr && cend - r0 <= 2 * cwords;
    const bool one_chunk = !row_runs && L <= (2 * T);
    uint64_t co0 = 0, co1 = 0;
    if (one_chunk) {
        if (2 * tid < L) co0 = g.cnt_off[2 * tid];
        if (2 * tid + 1 < L) co1 = g.cnt_off[2 * tid + 1];
    }
    CellPair next;
    if (one_chunk && (int)blockIdx.x < rows) next = load_cells(g, r0 + (int)blockIdx.x, 2 * tid);
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int i = r0 + r;
        const CellPair cur = next;
        if (one_chunk && r + (int)gridDim.x < rows) next = load_cells(g, i + (int)gridDim.x, 2 * tid);
        const int cbeg = r0 + (r & ~(kRareDenseAlign - 1));  // first column of the row's diagonal tile
        uint4* Rrow = reinterpret_cast<uint4*>(R + (size_t)r * ldr + (size_t)(cbeg - r0));
        for (int wb = cbeg; wb < cend; wb += 2 * cwords) {
            const int we = min(cend, wb + 2 * cwords);
            const int nq = (we - wb) >> 3;  // uint4 of counters (8 columns each); we - wb is a multiple of 256
            for (int w = tid; w < nq; w += T) smem_rd[w] = make_uint4(0, 0, 0, 0);
            const uint32_t jlo = (uint32_t)max(wb, i + 1), jhi = (uint32_t)min(we, n);
            if (row_runs) count_row_runs<T>(cnt, pre, run, g, i, wb);
            for (int kc = 0; !row_runs && jlo < jhi && kc < L; kc += (2 * T)) {
                // this thread's two loci, then a block-wide exclusive scan of the run lengths
                const int k0 = kc + 2 * tid;
                uint32_t lo0 = 0, lo1 = 0, l0 = 0, l1 = 0;
                if (one_chunk) {
                    l0 = partner_run(g, i, cur.a0, cur.m0, co0, jlo, jhi, &lo0);
                    l1 = partner_run(g, i, cur.a1, cur.m1, co1, jlo, jhi, &lo1);
                } else {
                    const CellPair c = load_cells(g, i, k0);
                    if (k0 < L) l0 = partner_run(g, i, c.a0, c.m0, g.cnt_off[k0], jlo, jhi, &lo0);
                    if (k0 + 1 < L) l1 = partner_run(g, i, c.a1, c.m1, g.cnt_off[k0 + 1], jlo, jhi, &lo1);
                }
                count_runs<T>(cnt, pre, run, wsum, l0, lo0, l1, lo1, g.members, wb);
            }
            __syncthreads();
            uint4* dst = Rrow + ((wb - cbeg) >> 3);
            for (int w = tid; w < nq; w += T) dst[w] = smem_rd[w];
            __syncthreads();
        }
    }
}

// Group run of a new profile at locus k: every member of the group of its
// allele (a = its rank in the groups' numbering; 0 missing, kNovelRank not in
// the set), clipped to columns [jlo, jhi).
__device__ __forceinline__ uint32_t group_run(const RareGroups& g, uint32_t a, uint64_t coff, uint32_t jlo,
                                              uint32_t jhi, uint32_t* lo_out) {
    if (!a || a == kNovelRank) return 0;
    const uint64_t q = coff + a;
    uint64_t b = __ldg(g.goff + q), e = __ldg(g.goff + q + 1);
    if (e <= b) return 0;  // frequent in the set: counted by the one-hot columns
    if (jlo > 0 && __ldg(g.members + b) < jlo) b = lower_bound_m(g.members, b, e, jlo);
    if (jhi < (uint32_t)g.n && b < e && __ldg(g.members + e - 1) >= jhi) e = lower_bound_m(g.members, b, e, jhi);
    *lo_out = (uint32_t)b;
    return (uint32_t)(e - b);
}

// Rare counts of m new profiles against every row of the set:
// R[r * ldr + j] = loci where new profile r and row j share an allele that is
// rare in the set, for j < n (0 up to cend).  Same counting as rare_dense_kernel.
template <int T>
__global__ void __launch_bounds__(T, 1024 / T)
    rare_query_kernel(const RareGroups g, const uint32_t* __restrict__ xq, int m, uint16_t* __restrict__ R,
                      size_t ldr, int cend, int cwords) {
    extern __shared__ uint4 smem_rd[];
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem_rd);
    uint32_t* pre = cnt + cwords;
    uint32_t* run = pre + (2 * T) + 1;
    uint32_t* wsum = run + (2 * T);
    const int tid = threadIdx.x;
    const int n = g.n, L = g.L;
    for (int r = blockIdx.x; r < m; r += gridDim.x) {
        uint4* Rrow = reinterpret_cast<uint4*>(R + (size_t)r * ldr);
        for (int wb = 0; wb < cend; wb += 2 * cwords) {
            const int we = min(cend, wb + 2 * cwords);
            const int nq = (we - wb) >> 3;
            for (int w = tid; w < nq; w += T) smem_rd[w] = make_uint4(0, 0, 0, 0);
            const uint32_t jlo = (uint32_t)wb, jhi = (uint32_t)min(we, n);
            for (int kc = 0; jlo < jhi && kc < L; kc += (2 * T)) {
                const int k0 = kc + 2 * tid;
                uint32_t lo0 = 0, lo1 = 0, l0 = 0, l1 = 0;
                if (k0 < L) l0 = group_run(g, xq[(size_t)r * L + k0], g.cnt_off[k0], jlo, jhi, &lo0);
                if (k0 + 1 < L) l1 = group_run(g, xq[(size_t)r * L + k0 + 1], g.cnt_off[k0 + 1], jlo, jhi, &lo1);
                count_runs<T>(cnt, pre, run, wsum, l0, lo0, l1, lo1, g.members, wb);
            }
            __syncthreads();
            uint4* dst = Rrow + (wb >> 3);
            for (int w = tid; w < nq; w += T) dst[w] = smem_rd[w];
            __syncthreads();
        }
    }
}

// The same block from pair lists: one CTA per stripe row (persistent), the
// row's partners read once per counter pass with consecutive threads on
// consecutive entries, each partner in the pass's columns adding 1 with a
// shared atomic.  A partner outside (i, n) is reported and skipped.
__global__ void __launch_bounds__(1024, 1)
    rare_lists_kernel(const uint32_t* __restrict__ start, const uint32_t* __restrict__ js, int n, int r0, int rows,
                      uint16_t* __restrict__ R, size_t ldr, int cend, int cwords, int* err) {
    extern __shared__ uint4 smem_rd[];
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem_rd);
    const int tid = threadIdx.x;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int i = r0 + r;
        const uint32_t pa = __ldg(start + i), pb = __ldg(start + i + 1);
        const int cbeg = r0 + (r & ~(kRareDenseAlign - 1));  // first column of the row's diagonal tile
        uint4* Rrow = reinterpret_cast<uint4*>(R + (size_t)r * ldr + (size_t)(cbeg - r0));
        for (int wb = cbeg; wb < cend; wb += 2 * cwords) {
            const int we = min(cend, wb + 2 * cwords);
            const int nq = (we - wb) >> 3;
            for (int w = tid; w < nq; w += blockDim.x) smem_rd[w] = make_uint4(0, 0, 0, 0);
            __syncthreads();
            for (uint32_t p = pa + (uint32_t)tid; p < pb; p += blockDim.x) {
                const uint32_t j = __ldg(js + p);
                if (j <= (uint32_t)i || j >= (uint32_t)n) {
                    if (wb == cbeg) atomicOr(err, DEVERR_RARE_PAIR);
                    continue;
                }
                if (j >= (uint32_t)wb && j < (uint32_t)we) count_col(cnt, j - (uint32_t)wb);
            }
            __syncthreads();
            uint4* dst = Rrow + ((wb - cbeg) >> 3);
            for (int w = tid; w < nq; w += blockDim.x) dst[w] = smem_rd[w];
            __syncthreads();
        }
    }
}

}  // namespace

cudaError_t launch_rare_from_lists(const uint32_t* start, const uint32_t* js, int n, int r0, int rows, uint16_t* R,
                                   size_t ldr, int* err, int sms, cudaStream_t st) {
    if (rows <= 0) return cudaSuccess;
    const size_t width = up((size_t)(n - r0), kRareDenseAlign);
    if (ldr < width || (ldr & 7) || ((uintptr_t)R & 15)) return cudaErrorInvalidValue;
    static bool attrs[kMaxDevices] = {};
    bool& attr = attrs[current_device()];
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(rare_lists_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   RD_WORDS * 4);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int cwords = counter_words(width);
    rare_lists_kernel<<<std::max(1, std::min(rows, sms)), 1024, cwords * 4, st>>>(start, js, n, r0, rows, R, ldr,
                                                                                 r0 + (int)width, cwords, err);
    return cudaGetLastError();
}

cudaError_t rare_batch_prepare(const std::vector<RareBatchItem>& items, RareBatchPlan* plan) {
    std::vector<RareJob> jobs;
    std::vector<int> row_job;
    int row0 = 0, cwords = 1;
    for (const RareBatchItem& it : items) {
        if (it.g.n < 2) continue;
        const size_t width = up((size_t)it.g.n, kRareDenseAlign);
        if (it.ldr < width || (it.ldr & 7) || ((uintptr_t)it.R & 15)) return cudaErrorInvalidValue;
        if (width > (size_t)2 * RD_WORDS) return cudaErrorInvalidValue;  // one counter pass per row
        RareJob j;
        j.g = it.g;
        j.R = it.R;
        j.ldr = it.ldr;
        j.cend = (int)width;
        j.row0 = row0;
        row0 += it.g.n;
        cwords = std::max(cwords, (int)(width / 2));
        row_job.insert(row_job.end(), (size_t)it.g.n, (int)jobs.size());
        jobs.push_back(j);
    }
    rare_batch_release(plan);
    plan->njobs = (int)jobs.size();
    plan->total_rows = row0;
    plan->cwords = cwords;
    if (jobs.empty()) return cudaSuccess;
    cudaError_t e = cudaMalloc(&plan->d_jobs, jobs.size() * sizeof(RareJob));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_row_job, row_job.size() * sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemcpy(plan->d_jobs, jobs.data(), jobs.size() * sizeof(RareJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(plan->d_row_job, row_job.data(), row_job.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    static bool attrs[kMaxDevices] = {};
    bool& attr = attrs[current_device()];
    if (!attr) {
        e = cudaFuncSetAttribute(rare_batch_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 rd_smem<NT>(RD_WORDS));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return cudaSuccess;
}

cudaError_t launch_rare_batch(const RareBatchPlan& plan, int sms, cudaStream_t st) {
    if (!plan.njobs || !plan.total_rows) return cudaSuccess;
    // one CTA per row, as the per-set launches: rows differ widely in work
    // (the sets' widths and taus), and the block scheduler balances them
    (void)sms;
    const int grid = std::max(1, plan.total_rows);
    rare_batch_kernel<NT><<<grid, NT, rd_smem<NT>(plan.cwords), st>>>(
        static_cast<const RareJob*>(plan.d_jobs), static_cast<const int*>(plan.d_row_job), plan.total_rows,
        plan.cwords);
    return cudaGetLastError();
}

void rare_batch_release(RareBatchPlan* plan) {
    if (plan->d_jobs) cudaFree(plan->d_jobs);
    if (plan->d_row_job) cudaFree(plan->d_row_job);
    plan->d_jobs = plan->d_row_job = nullptr;
    plan->njobs = plan->total_rows = 0;
}

cudaError_t launch_rare_dense(const RareGroups& g, int r0, int rows, uint16_t* R, size_t ldr, int sms,
                              cudaStream_t st) {
    if (rows <= 0) return cudaSuccess;
    const size_t width = up((size_t)(g.n - r0), kRareDenseAlign);
    if (ldr < width || (ldr & 7) || ((uintptr_t)R & 15)) return cudaErrorInvalidValue;
    static bool attrs[kMaxDevices] = {};  // once per device (also keeps it out of graph captures)
    bool& attr = attrs[current_device()];
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(rare_dense_kernel<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             rd_smem<1024>(RD_WORDS));

        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(rare_dense_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     rd_smem<NT>(RD_WORDS));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int cwords = counter_words(width);
    // a narrow stripe takes CTAs of NT (128) threads, one row each: eight fit on
    // an SM, so eight rows' chains of dependent steps overlap, and solves that
    // run side by side share the SMs.  Narrow rows carry little counting work,
    // so their time is those chains: the 512-set batch (50-5 000 profiles each)
    // took 17.4 ms with 128 threads per row and 18.5 ms with 256.
    // TCH_RARE_SMALL_ROWS sets a row limit for it.
    static int small_rows = -1;
    if (small_rows < 0) {
        const char* v = getenv("TCH_RARE_SMALL_ROWS");
        small_rows = v ? std::max(0, atoi(v)) : INT_MAX;
    }
    if (rows < small_rows && width <= 8192) {
        rare_dense_kernel<NT><<<std::max(1, rows), NT, rd_smem<NT>(cwords), st>>>(g, r0, rows, R, ldr,
                                                                                   r0 + (int)width, cwords);
    } else {
        const int grid = std::max(1, std::min(rows, sms));
        rare_dense_kernel<1024><<<grid, 1024, rd_smem<1024>(cwords), st>>>(g, r0, rows, R, ldr, r0 + (int)width,
                                                                            cwords);
    }
    return cudaGetLastError();
}

}  // namespace tch

namespace tch {

cudaError_t launch_rare_query(const RareGroups& g, const uint32_t* xq, int m, uint16_t* R, size_t ldr, int sms,
                              cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    const size_t width = up((size_t)std::max(g.n, 1), kRareDenseAlign);
    if (ldr < width || (ldr & 7) || ((uintptr_t)R & 15)) return cudaErrorInvalidValue;
    static bool attrs[kMaxDevices] = {};
    bool& attr = attrs[current_device()];
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(rare_query_kernel<1024>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   rd_smem<1024>(RD_WORDS));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int cwords = counter_words(width);
    rare_query_kernel<1024><<<std::max(1, std::min(m, sms)), 1024, rd_smem<1024>(cwords), st>>>(g, xq, m, R, ldr,
                                                                                               (int)width, cwords);
    return cudaGetLastError();
}

}  // namespace tch
