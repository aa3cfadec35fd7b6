// Tensor-core contraction for sm_103a: tcgen05.mma with TMEM accumulators,
// operands staged by TMA, one fused epilogue writing u16 distances.
//
// Operands: X is n_rows x kb bytes, row = [presence part (kp bytes) |
// one-hot part (kb - kp bytes)], one byte per element, 0 or +1 in e4m3
// (0x38).  One output tile (128 rows i x 256 columns j) is
//
//   D = X_i[:, :kp] X_j[:, :kp]^T  -  X_i[:, kp:] X_j[:, kp:]^T  =  P Pt - O Ot
//
// with the minus taken by the instruction descriptor's negate-B bit on the
// one-hot stages.  Every partial sum is an integer with |value| <= number of
// loci < 2^24, so fp32 accumulation is exact; the epilogue re-checks the
// integrality of every value anyway and reports a device error if it ever
// fails.  This replaces the reference's two CUTLASS b1 GEMMs
// (tensorcore/rs/cuda/tch.cu:22-32, 128-129): on GB300 the b1 and s8 warp
// MMAs issue at ~150 TOPS, and tcgen05 kind::i8 does not exist on sm_103a.
//
// CTA = 6 warps, persistent over the stripe's tiles (upper triangle only):
//   warp 0   TMA producer     4-stage ring of (A 128x128 B, B 256x128 B) tiles
//   warp 1   MMA issuer       4 x tcgen05.mma (K = 32 bytes) per stage into one
//                             of two 256-column TMEM accumulators
//   warps 2-5 epilogue        tcgen05.ld 32 columns at a time -> int -> u16
//                             in shared memory -> rare pairs of the row
//                             subtracted (ascending CSR walk) -> coalesced
//                             stores of the valid cells
// Tiles are visited in groups of 8 row blocks (column-major inside a group) so
// that concurrently running CTAs share A and B tiles in L2.
//
// Every mbarrier wait is bounded (about 2 s of %globaltimer); on a timeout the
// CTA records DEVERR_TIMEOUT, stops issuing work, drains what it issued,
// frees its TMEM and returns.

#include <cuda.h>
#include <cudaTypedefs.h>

#include "tc_ptx.cuh"
#include "tch_internal.cuh"

namespace tch {
namespace {

constexpr int BM = 128;            // tile rows (TMEM lanes)
constexpr int BN = 256;            // tile columns (MMA N)
constexpr int BK = 128;            // bytes of K per stage = one 128-byte swizzle row
constexpr int STAGES = 4;
constexpr int A_BYTES = BM * BK;   // 16 KB
constexpr int B_BYTES = BN * BK;   // 32 KB
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int EPI_WARPS = 8;      // two per TMEM lane quarter, one per column half
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int EPI_PITCH = 34;      // u16 per staged row: 32 + 2 keeps row writes conflict-free
constexpr int EPI_BYTES = EPI_WARPS * 32 * EPI_PITCH * 2;
constexpr int TMEM_COLS = 2 * BN;  // two accumulators
constexpr int GROUP_M = 16;        // row blocks per raster group (default; TCH_TC_GROUP overrides)
constexpr int RBUF = 16;           // rare partners fetched per batch in the epilogue
constexpr int SMEM_BYTES = 1024 + STAGES * STAGE_BYTES + EPI_BYTES + 256;

enum Kind { KIND_F8 = 0, KIND_I8 = 1 };

using namespace ptx;

// ---------------------------------------------------------------- tile order
// A cluster of CM CTAs works on CM vertically adjacent 128-row blocks (a
// "super-row" sr of CM * 128 rows) against one 256-column block bj; CTA rank r
// owns row block bi = sr * CM + r.  With CM = 2 the two CTAs share the B tile:
// each loads one 128-row half and multicasts it to both.
// Row blocks per raster group: GROUP_M unless TCH_TC_GROUP gives another even
// count in [2, 256].  Larger groups read the column side of the operand fewer
// times (once per group) at the cost of a larger row-side working set.
int group_row_blocks() {
    static int g = 0;
    if (!g) {
        const char* v = getenv("TCH_TC_GROUP");
        const int x = v ? atoi(v) : 0;
        g = (x >= 2 && x <= 256 && x % 2 == 0) ? x : GROUP_M;
    }
    return g;
}

struct TileSpace {
    int nsr, nbj;  // super-rows of the stripe, column blocks of [c0, n)
    int cm;        // row blocks per super-row (cluster size)
    int gs;        // super-rows per raster group
    int rect;      // 1: every tile of the rectangle (rows of one set against columns of another)
};

// Columns of super-row sr: bj >= sr * cm / 2 (128-row blocks against 256-wide
// column blocks that both start at r0; earlier columns lie below the diagonal);
// all of them for a rectangle.
__host__ __device__ __forceinline__ int first_col(const TileSpace& ts, int sr) {
    return ts.rect ? 0 : sr * ts.cm / 2;
}

__host__ __device__ __forceinline__ long long count_tiles(const TileSpace& ts) {
    long long c = 0;
    for (int sr = 0; sr < ts.nsr; sr++) c += ts.nbj > first_col(ts, sr) ? ts.nbj - first_col(ts, sr) : 0;
    return c;
}

constexpr int MAX_GROUPS = 1024;   // raster groups with a precomputed first tile

// First tile index of every raster group (groups of gs super-rows,
// column-major inside a group), so a tile's coordinates cost a binary search
// over groups plus a few steps instead of a walk over the whole stripe.
struct GroupTable {
    int ngroups;
    int first[MAX_GROUPS + 1];
};

__host__ __device__ __forceinline__ int group_tiles(const TileSpace& ts, int g0, int g1) {
    int cnt = 0;
    for (int sr = g0; sr < g1; sr++) cnt += ts.nbj > first_col(ts, sr) ? ts.nbj - first_col(ts, sr) : 0;
    return cnt;
}

// t -> (sr, bj).
__device__ bool tile_coords(const TileSpace& ts, const GroupTable& gt, int t, int* sr_out, int* bj_out) {
    const int gs = ts.gs;
    int lo = 0, hi = gt.ngroups;     // last group whose first tile is <= t
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (gt.first[mid] <= t) lo = mid; else hi = mid;
    }
    t -= gt.first[lo];
    const int g0 = lo * gs, g1 = min(ts.nsr, g0 + gs);
    // columns where only part of the group lies on or above the diagonal
    // (super-row sr is present in column bj iff sr * cm <= 2 bj + 1)
    int bj = first_col(ts, g0);
    for (; !ts.rect && bj < ts.nbj; bj++) {
        const int rows = min(g1 - 1, (2 * bj + 1) / ts.cm) - g0 + 1;
        if (rows == g1 - g0) break;  // from here on every column holds the whole group
        if (rows > 0) {
            if (t < rows) {
                *sr_out = g0 + t;
                *bj_out = bj;
                return true;
            }
            t -= rows;
        }
    }
    const int full = g1 - g0;
    bj += t / full;
    if (bj >= ts.nbj) return false;
    *sr_out = g0 + t % full;
    *bj_out = bj;
    return true;
}

// Tensor maps of every K chunk of the operand: A boxes (128 rows) and B boxes
// (256 / CM rows), and the 128-byte K blocks of each chunk.
struct TcMaps {
    CUtensorMap a[kMaxKChunks];
    CUtensorMap b[kMaxKChunks];
    int kblocks[kMaxKChunks];
    int n;
};

struct TcParams {
    int n, r0, rows;  // columns end at n; rows [r0, r0 + rows) of the A operand
    int c0;           // first column: r0 (upper triangle) or 0 (rectangle against the B operand)
    int kblocks, kblocks_p;  // K stages in total and in the presence part
    TileSpace ts;
    GroupTable gt;
    int num_tiles;
    const uint32_t* start;
    const uint32_t* js;
    int fuse_rare;
    const int* unsorted;  // optional device flag: non-zero turns the fused subtraction off
    const uint16_t* rdense;  // dense rare counts of the stripe (row stride ldr, column j at j - r0), or null
    size_t ldr;
    uint16_t* out;
    size_t ldo;
    int* err;
};

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* __restrict__ js, uint32_t lo, uint32_t hi,
                                                    uint32_t key) {
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (__ldg(js + mid) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <int KIND, int CM>
__global__ void __launch_bounds__(THREADS, 1)
tc_stripe_kernel(const __grid_constant__ TcMaps maps,
                 const TcParams p) {
    static_assert(CM == 1 || CM == 2, "cluster of 1 or 2 CTAs");
    constexpr int B_PART = B_BYTES / CM;  // bytes of the B tile this CTA loads per stage
    const uint32_t rank = CM == 1 ? 0u : cluster_ctarank();
    const int cid = CM == 1 ? (int)blockIdx.x : (int)cluster_id_x();
    const int ncl = CM == 1 ? (int)gridDim.x : (int)num_clusters_x();
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte alignment of the swizzled stage buffers
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* stage_a = smem;
    uint8_t* stage_b = smem + STAGES * A_BYTES;
    uint16_t* epi = (uint16_t*)(smem + STAGES * STAGE_BYTES);
    uint64_t* bars = (uint64_t*)(smem + STAGES * STAGE_BYTES + EPI_BYTES);
    uint64_t* full = bars;                  // STAGES
    uint64_t* empty = bars + STAGES;        // STAGES
    uint64_t* tfull = bars + 2 * STAGES;    // 2
    uint64_t* tempty = bars + 2 * STAGES + 2;  // 2
    uint64_t* drain = bars + 2 * STAGES + 4;   // 1
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 5);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], CM);  // released by the MMA warp of every CTA that reads the stage
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], EPI_WARPS);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int c = 0; c < maps.n; c++) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&maps.a[c]) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&maps.b[c]) : "memory");
        }
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    if (CM > 1) cluster_sync();  // the peer's barriers exist before any multicast reaches them
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            int s = 0;
            uint32_t ph = 0;
            bool ok = true;
            int issued[STAGES];
            uint32_t issued_ph[STAGES];
            for (int q = 0; q < STAGES; q++) issued[q] = 0, issued_ph[q] = 0;
            for (int t = cid; ok && t < p.num_tiles; t += ncl) {
                int sr, bj;
                if (!tile_coords(p.ts, p.gt, t, &sr, &bj)) break;
                const int bi = sr * CM + (int)rank;
                const int y_a = p.r0 + bi * BM, y_b = p.c0 + bj * BN + (int)rank * (BN / CM);
                int ch = 0, kbl = 0;  // K chunk and block inside it
                for (int kb = 0; kb < p.kblocks; kb++) {
                    if (!mbar_wait(&empty[s], ph ^ 1, abort_flag, p.err)) { ok = false; break; }
                    mbar_expect_tx(&full[s], STAGE_BYTES);  // A + both halves of B land here
                    tma_load_2d(&maps.a[ch], &full[s], stage_a + s * A_BYTES, kbl * BK, y_a);
                    if (CM == 1)
                        tma_load_2d(&maps.b[ch], &full[s], stage_b + s * B_BYTES, kbl * BK, y_b);
                    else
                        tma_load_2d_multicast(&maps.b[ch], &full[s], stage_b + s * B_BYTES + rank * B_PART, kbl * BK,
                                              y_b, (uint16_t)((1u << CM) - 1));
                    if (++kbl == maps.kblocks[ch]) kbl = 0, ch++;
                    issued[s] = 1;
                    issued_ph[s] = ph;
                    if (++s == STAGES) s = 0, ph ^= 1;
                }
            }
            if (ok) {
                // tail: every stage released by the MMA warp (all commits arrived)
                for (int q = 0; q < STAGES; q++) {
                    if (!mbar_wait(&empty[s], ph ^ 1, abort_flag, p.err)) break;
                    if (++s == STAGES) s = 0, ph ^= 1;
                }
            } else {
                // abort: let the loads already issued land before the CTA exits
                for (int q = 0; q < STAGES; q++)
                    if (issued[q]) {
                        const unsigned long long t0 = gtimer();
                        while (!mbar_test(&full[q], issued_ph[q]) && gtimer() - t0 < WAIT_NS) {}
                    }
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t id_pos = KIND == KIND_F8 ? make_idesc(1, 0, 0, BM, BN) : make_idesc(2, 1, 0, BM, BN);
            const uint32_t id_neg = KIND == KIND_F8 ? make_idesc(1, 0, 1, BM, BN) : make_idesc(2, 1, 0, BM, BN);
            int s = 0, acc = 0;
            uint32_t ph = 0, aph = 0;
            bool ok = true;
            for (int t = cid; ok && t < p.num_tiles; t += ncl) {
                if (!mbar_wait(&tempty[acc], aph ^ 1, abort_flag, p.err)) { ok = false; break; }
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + (uint32_t)(acc * BN);
                for (int kb = 0; kb < p.kblocks; kb++) {
                    if (!mbar_wait(&full[s], ph, abort_flag, p.err)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(stage_a + s * A_BYTES), b0 = smem_u32(stage_b + s * B_BYTES);
                    const uint32_t idesc = kb < p.kblocks_p ? id_pos : id_neg;
#pragma unroll
                    for (int k = 0; k < BK / 32; k++)
                        tc_mma_f8(d_tmem, sw128_desc(a0 + 32 * k), sw128_desc(b0 + 32 * k), idesc,
                                     (kb | k) ? 1u : 0u);
                    // stage free once these MMAs have read it (in every CTA whose B half it holds)
                    if (CM == 1) tc_commit(&empty[s]);
                    else tc_commit_multicast(&empty[s], (uint16_t)((1u << CM) - 1));
                    if (++s == STAGES) s = 0, ph ^= 1;
                }
                if (!ok) break;
                tc_commit(&tfull[acc]);  // accumulator ready for the epilogue
                if (++acc == 2) acc = 0, aph ^= 1;
            }
            // every MMA issued by this thread has completed before TMEM is freed
            tc_commit(drain);
            const unsigned long long t0 = gtimer();
            while (!mbar_test(drain, 0) && gtimer() - t0 < WAIT_NS) {}
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3;  // TMEM lanes [32 q, 32 q + 32) belong to this warp
        const int half = (warp - 2) / 4;  // columns [128 half, 128 half + 128) of the tile
        constexpr int CHUNKS = BN / 32 / 2;
        uint16_t* stg = epi + (warp - 2) * 32 * EPI_PITCH;
        const int iend = p.r0 + p.rows;
        const bool fuse = p.fuse_rare && !(p.unsorted && *p.unsorted);
        const bool dense = p.rdense != nullptr;
        int acc = 0;
        uint32_t aph = 0;
        int bad = 0;
        for (int t = cid; t < p.num_tiles; t += ncl) {
            int sr, bj;
            if (!tile_coords(p.ts, p.gt, t, &sr, &bj)) break;
            const int bi = sr * CM + (int)rank;
            const int i0 = p.r0 + bi * BM, j0 = p.c0 + bj * BN;
            const int my_i = i0 + q * 32 + lane;
            // this row's rare partners inside the tile: an ascending run of js
            uint32_t rp = 0, rhi = 0;
            if (fuse && my_i < iend) {
                rhi = __ldg(p.start + my_i + 1);
                rp = lower_bound_u32(p.js, __ldg(p.start + my_i), rhi, (uint32_t)(j0 + half * (BN / 2)));
            }
            // the next RBUF partners, fetched together (independent loads);
            // entries [bpos, nbuf) are still to be applied
            uint32_t rbuf[RBUF];
            int bpos = 0, nbuf = 0;
            if (!mbar_wait(&tfull[acc], aph, abort_flag, p.err)) break;
            tc_fence_after();
            const uint32_t tbase = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN);
#pragma unroll 1
            for (int cc = 0; cc < CHUNKS; cc++) {
                const int c = half * CHUNKS + cc;
                const uint32_t cb = (uint32_t)(j0 + c * 32);
                // this row's dense rare counts for the chunk's 32 columns (64 bytes),
                // fetched before the accumulator read so the two overlap
                uint4 rq[4] = {};
                if (dense && my_i < iend) {
                    const uint4* src = reinterpret_cast<const uint4*>(p.rdense + (size_t)(my_i - p.r0) * p.ldr +
                                                                      (size_t)(cb - (uint32_t)p.c0));
#pragma unroll
                    for (int u = 0; u < 4; u++) rq[u] = __ldg(src + u);
                }
                uint32_t v[32];
                tmem_ld32(tbase + (uint32_t)(c * 32), v);
                tmem_wait_ld();
                if (cc == CHUNKS - 1) {  // this warp's part of the accumulator is read: hand it back
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[acc]);
                }
                // own row -> staging buffer (u16)
                uint32_t* row32 = reinterpret_cast<uint32_t*>(stg + lane * EPI_PITCH);
#pragma unroll
                for (int w = 0; w < 16; w++) {
                    int x0, x1;
                    if (KIND == KIND_F8) {
                        const float f0 = __uint_as_float(v[2 * w]), f1 = __uint_as_float(v[2 * w + 1]);
                        x0 = __float2int_rn(f0);
                        x1 = __float2int_rn(f1);
                        bad |= (__int2float_rn(x0) != f0) | (__int2float_rn(x1) != f1);
                    } else {
                        x0 = (int)v[2 * w];
                        x1 = (int)v[2 * w + 1];
                    }
                    if (dense) {
                        const uint4& r4 = rq[w / 4];
                        const uint32_t rw = (w % 4 == 0) ? r4.x : (w % 4 == 1) ? r4.y : (w % 4 == 2) ? r4.z : r4.w;
                        x0 -= (int)(rw & 0xFFFF);
                        x1 -= (int)(rw >> 16);
                    }
                    row32[w] = (uint32_t)(x0 & 0xFFFF) | ((uint32_t)(x1 & 0xFFFF) << 16);
                }
                // rare pairs of this row in columns [cb, cb + 32)
                for (;;) {
                    if (bpos == nbuf) {
                        if (rp >= rhi) break;
                        nbuf = rhi - rp < (uint32_t)RBUF ? (int)(rhi - rp) : RBUF;
#pragma unroll
                        for (int q = 0; q < RBUF; q++) rbuf[q] = q < nbuf ? __ldg(p.js + rp + q) : 0xFFFFFFFFu;
                        rp += (uint32_t)nbuf;
                        bpos = 0;
                    }
                    // ascending: the entries below cb + 32 form a prefix of what is left
#pragma unroll
                    for (int q = 0; q < RBUF; q++)
                        if (q >= bpos && q < nbuf && rbuf[q] < cb + 32) {
                            // (a shared atomicSub on the 32-bit word measured slower than this
                            // plain read-modify-write of the lane's own row)
                            stg[lane * EPI_PITCH + (int)(rbuf[q] - cb)] -= 1;
                            bpos = q + 1;
                        }
                    if (bpos < nbuf) break;  // the next partner lies beyond this chunk
                }
                __syncwarp();
                // coalesced store: 16 lanes x 4 bytes per row, 2 rows per step
#pragma unroll 4
                for (int st = 0; st < 16; st++) {
                    const int rr = st * 2 + lane / 16, w = lane % 16;
                    const int i = i0 + q * 32 + rr;
                    const int j = (int)cb + 2 * w;
                    if (i < iend && j < p.n) {
                        const uint32_t val = reinterpret_cast<const uint32_t*>(stg + rr * EPI_PITCH)[w];
                        uint16_t* dst = p.out + (size_t)(i - p.r0) * p.ldo + (size_t)(j - p.c0);
                        if (j + 1 < p.n) *reinterpret_cast<uint32_t*>(dst) = val;
                        else *dst = (uint16_t)(val & 0xFFFF);
                    }
                }
                __syncwarp();
            }
            if (++acc == 2) acc = 0, aph ^= 1;
        }
        if (bad) atomicOr(p.err, DEVERR_OVERFLOW);
    }

    tc_fence_before();
    __syncthreads();
    // no CTA leaves while its peer may still multicast into it or arrive on its barriers
    if (CM > 1) cluster_sync();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS)
                     : "memory");
    }
}

// ---------------------------------------------------------------- host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

bool make_map(CUtensorMap* m, const uint8_t* X, size_t rows, int kb, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)kb, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kb};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)X, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The K chunks of an operand (one chunk when it is a single allocation).
KChunks chunks_of(const ByteOperands& ops) {
    KChunks ch = ops.chunks;
    if (ch.n == 0) {
        ch.p[0] = const_cast<uint8_t*>(ops.X);
        ch.n = 1;
        ch.width = ops.kb;
        ch.kb = ops.kb;
    }
    return ch;
}

// ops: the A operand (the stripe's rows); bops: the B operand (the columns),
// the same rows for the upper triangle, another set for a rectangle.
template <int KIND, int CM>
cudaError_t launch_kind(const ByteOperands& ops, const ByteOperands& bops, const RareCSR& rare, const StripeArgs& a,
                        int num_sms, cudaStream_t st) {
    static bool attrs[kMaxDevices] = {};
    static int max_clusters_of[kMaxDevices] = {};
    const int dev = current_device();
    bool& attr = attrs[dev];
    int& max_clusters = max_clusters_of[dev];
    auto kern = tc_stripe_kernel<KIND, CM>;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute lattr[1];
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = SMEM_BYTES;
    cfg.stream = st;
    if (CM > 1) {
        lattr[0].id = cudaLaunchAttributeClusterDimension;
        lattr[0].val.clusterDim.x = CM;
        lattr[0].val.clusterDim.y = 1;
        lattr[0].val.clusterDim.z = 1;
        cfg.attrs = lattr;
        cfg.numAttrs = 1;
    }
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) return e;
        if (CM > 1) {
            cfg.gridDim = dim3(CM * std::max(num_sms / CM, 1));
            e = cudaOccupancyMaxActiveClusters(&max_clusters, kern, &cfg);
            if (e != cudaSuccess) return e;
            if (max_clusters < 1) return cudaErrorInvalidConfiguration;
        }
        attr = true;
    }
    if ((ops.kb % BK) || (ops.kp % BK) || ops.kb <= 0) return cudaErrorInvalidValue;
    if (bops.kb != ops.kb || bops.kp != ops.kp) return cudaErrorInvalidValue;
    if ((a.ldo & 1) || ((uintptr_t)a.out & 3)) return cudaErrorInvalidValue;
    if (a.rect && !rare.dense && rare.n_rare > 0) return cudaErrorInvalidValue;  // rectangles take dense counts
    const KChunks ch = chunks_of(ops), chb = chunks_of(bops);
    if (ch.kb != ops.kb || (ch.width % BK)) return cudaErrorInvalidValue;
    if (chb.n != ch.n || chb.width != ch.width || chb.kb != ch.kb) return cudaErrorInvalidValue;
    TcMaps maps;
    maps.n = ch.n;
    for (int c = 0; c < ch.n; c++) {
        const int wc = ch.width_of(c);
        if (wc <= 0 || (wc % BK)) return cudaErrorInvalidValue;
        if (!make_map(&maps.a[c], ch.p[c], ops.n_rows, wc, BM) ||
            !make_map(&maps.b[c], chb.p[c], bops.n_rows, wc, BN / CM))
            return cudaErrorInvalidValue;
        maps.kblocks[c] = wc / BK;
    }
    TcParams p;
    p.n = a.n;
    p.r0 = a.r0;
    p.c0 = a.rect ? 0 : a.r0;
    p.rows = a.rows;
    p.kblocks = ops.kb / BK;
    p.kblocks_p = ops.kp / BK;
    p.ts.cm = CM;
    p.ts.gs = group_row_blocks() / CM;
    p.ts.nsr = ((a.rows + BM - 1) / BM + CM - 1) / CM;
    p.ts.rect = a.rect ? 1 : 0;
    p.ts.nbj = (a.n - p.c0 + BN - 1) / BN;
    p.num_tiles = (int)count_tiles(p.ts);
    {
        const int gs = p.ts.gs;
        p.gt.ngroups = (p.ts.nsr + gs - 1) / gs;
        if (p.gt.ngroups > MAX_GROUPS) return cudaErrorInvalidValue;  // callers split taller stripes
        int acc = 0;
        for (int g = 0; g < p.gt.ngroups; g++) {
            p.gt.first[g] = acc;
            acc += group_tiles(p.ts, g * gs, std::min(p.ts.nsr, g * gs + gs));
        }
        p.gt.first[p.gt.ngroups] = acc;
    }
    p.start = rare.start;
    p.js = rare.js;
    p.fuse_rare = (!rare.dense && rare.n_rare > 0 && (rare.sorted || rare.unsorted_flag)) ? 1 : 0;
    p.unsorted = rare.unsorted_flag;
    p.rdense = rare.dense;
    p.ldr = rare.ldr;
    if (rare.dense && ((rare.ldr & 7) || ((uintptr_t)rare.dense & 15))) return cudaErrorInvalidValue;
    p.out = a.out;
    p.ldo = a.ldo;
    p.err = a.err;
    if (p.num_tiles == 0) return cudaSuccess;
    const int clusters = std::min(p.num_tiles, CM > 1 ? max_clusters : std::max(num_sms, 1));
    cfg.gridDim = dim3(CM * clusters);
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, maps, p);
    if (e != cudaSuccess) return e;
    if (!rare.dense && rare.n_rare > 0 && !rare.sorted) return launch_rare_atomic(rare, a, st);
    return cudaSuccess;
}

// Cluster size of the stripe kernel: 2 (B tile shared by multicast) unless
// TCH_TC_CLUSTER=1 asks for single CTAs.
int cluster_size() {
    static int cm = 0;
    if (!cm) {
        const char* v = getenv("TCH_TC_CLUSTER");
        cm = (v && v[0] == '1') ? 1 : 2;
    }
    return cm;
}

}  // namespace

// kind::i8 does not exist on sm_103a (ptxas: "Feature '.kind::i8' not
// supported on .target 'sm_103a'"), so TCH_KERNEL_TC_I8 is never compiled in.
bool tc_kernel_compiled(int kernel) { return kernel == TCH_KERNEL_TC_F8; }

cudaError_t launch_tc_stripe(int kernel, const ByteOperands& ops, const ByteOperands* bops, const RareCSR& rare,
                             const StripeArgs& a, int num_sms, cudaStream_t st) {
    if (a.rows <= 0 || (!a.rect && a.r0 >= a.n) || (a.rect && a.n <= 0)) return cudaSuccess;
    if (a.rect && !bops) return cudaErrorInvalidValue;
    const ByteOperands& b = bops ? *bops : ops;
    if (kernel != TCH_KERNEL_TC_F8) return cudaErrorNotSupported;
    // one launch covers at most MAX_GROUPS raster groups of rows; a taller
    // stripe runs as consecutive sub-stripes writing into the same output
    const int max_rows = MAX_GROUPS * group_row_blocks() * BM;
    for (int done = 0; done < a.rows; done += max_rows) {
        StripeArgs s = a;
        s.r0 = a.r0 + done;
        s.rows = std::min(max_rows, a.rows - done);
        const size_t col = a.rect ? 0 : (size_t)done;  // a triangle's columns start at its first row
        s.out = a.out + (size_t)done * a.ldo + col;
        RareCSR rs = rare;
        if (rare.dense) rs.dense = rare.dense + (size_t)done * rare.ldr + col;
        const int cm = (a.cluster == 1 || a.cluster == 2) ? a.cluster : cluster_size();
        const cudaError_t e = cm == 2 ? launch_kind<KIND_F8, 2>(ops, b, rs, s, num_sms, st)
                                      : launch_kind<KIND_F8, 1>(ops, b, rs, s, num_sms, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace tch
