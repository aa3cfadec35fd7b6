// Tensor-core tile pass for sm_103a: block-scaled fp4 tcgen05.mma
// (kind::mxf4, every scale factor 1.0) with TMEM accumulators, operands staged
// by TMA, one fused epilogue writing u16 distances.
//
// Operands (Fp4Operands): packed e2m1 rows [presence | one-hot | zeros], two
// elements per byte, 0 or +1.0 in the `pos` copy, which is read as A, and 0
// or +1.0 / -1.0 (one-hot part) in the `neg` copy, which is read as B.  One
// output tile (128 rows i x 224 columns j) is
//
//   D = pos_i . neg_j^T  =  P Pt - O Ot
//
// Every product is 0 or +-1 and every partial sum an integer of magnitude at
// most the number of loci (< 2^24), so the fp32 accumulation is exact; the
// epilogue re-checks the integrality of every value and reports a device
// error if it ever fails.  This replaces the reference's two CUTLASS b1 GEMMs
// (tensorcore/rs/cuda/tch.cu:22-32, 128-129): on GB300 the b1 warp MMA issues
// at ~150 TOPS, kind::i8 does not exist on sm_103a, and the fp4 kinds run at
// twice the fp8 rate from half the operand bytes (tch-peak).  The fp4 kinds
// have no negate bit, hence the second operand copy with the one-hot sign in
// the data.
//
// CTA = 10 warps, one CTA per SM, persistent over the stripe's tiles (upper
// triangle only, or every tile of a rectangle):
//   warp 0    TMA producer   5-stage ring of (A 128 x 128 B, B 224 x 128 B)
//   warp 1    MMA issuer     4 x tcgen05.mma (K = 64 elements) per stage into
//                            one of two 224-column TMEM accumulators
//   warps 2-9 epilogue       two per TMEM lane quarter, one per column half:
//                            tcgen05.ld 16 columns -> int -> minus the dense
//                            rare counts (16-byte loads issued before the TMEM
//                            read) -> u16 -> 32-byte stores from registers
// TMEM: accumulators at columns 0 and 256, the scale factors (1.0, written
// once by the epilogue warps before the first MMA) in columns 480-511.
// Tiles are visited in raster groups of 8 row blocks, column-major inside a
// group, so that the CTAs running at the same time share A and B tiles in L2.
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

constexpr int BM = 128;             // tile rows (TMEM lanes)
constexpr int BN = 224;             // tile columns (MMA N)
constexpr int BK = 128;             // bytes of K per stage: one 128-byte swizzle row, 256 elements
constexpr int STAGES = 5;
constexpr int A_BYTES = BM * BK;    // 16 KB
constexpr int B_BYTES = BN * BK;    // 28 KB
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int EPI_WARPS = 8;
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int ACC_STRIDE = 256;     // TMEM columns from one accumulator to the next
constexpr int SF_COL = 480;         // 32 TMEM columns of scale factors
constexpr int TMEM_COLS = 512;
constexpr int CHUNK = 16;           // accumulator columns per tcgen05.ld
constexpr int WARP_CHUNKS = BN / CHUNK / 2;  // chunks per epilogue warp (its column half)
constexpr int GROUP_M = 8;          // row blocks per raster group (default; TCH_TC_GROUP overrides)
constexpr int BAR_BYTES = 256;
constexpr int SMEM_BYTES = 1024 + STAGES * STAGE_BYTES + BAR_BYTES;
static_assert(SMEM_BYTES <= 232448, "shared memory per CTA");
static_assert(BN % (2 * CHUNK) == 0 && BN <= ACC_STRIDE && ACC_STRIDE + BN <= SF_COL, "TMEM layout");
static_assert(A_BYTES % 1024 == 0 && B_BYTES % 1024 == 0, "stages stay 1024-byte aligned (128-byte swizzle)");

using namespace ptx;

// Row blocks per raster group: GROUP_M unless TCH_TC_GROUP gives another
// count in [1, 256].  Larger groups read the column side of the operand fewer
// times (once per group) at the cost of a larger row-side working set.
int group_row_blocks() {
    static int g = 0;
    if (!g) {
        const char* v = getenv("TCH_TC_GROUP");
        const int x = v ? atoi(v) : 0;
        g = (x >= 1 && x <= 256) ? x : GROUP_M;
    }
    return g;
}

// ---------------------------------------------------------------- tile order
// Row block bi covers rows a_r0 + BM bi .. + BM of the A operand, column block
// bj columns c0 + BN bj .. + BN.  In a triangle (c0 = r0) the row block's
// first column block is the one holding its first diagonal cell.
struct TileSpace {
    int nbi, nbj;  // row blocks of the stripe, column blocks of [c0, n)
    int gs;        // row blocks per raster group
    int rect;      // 1: every tile (rows of one set against columns of another)
};

__host__ __device__ __forceinline__ int first_col(const TileSpace& ts, int bi) {
    return ts.rect ? 0 : (BM * bi) / BN;
}
// The last row block present in column block bj.
__host__ __device__ __forceinline__ int last_row(const TileSpace& ts, int bj) {
    const int r = ((bj + 1) * BN - 1) / BM;
    return ts.rect || r > ts.nbi - 1 ? ts.nbi - 1 : r;
}

__host__ __device__ __forceinline__ long long tiles_in(const TileSpace& ts, int b0, int b1) {
    long long c = 0;
    for (int bi = b0; bi < b1; bi++) c += ts.nbj > first_col(ts, bi) ? ts.nbj - first_col(ts, bi) : 0;
    return c;
}

constexpr int MAX_GROUPS = 1024;  // raster groups with a precomputed first tile

// First tile index of every raster group, so a tile's coordinates cost a
// binary search over groups plus a few steps.
struct GroupTable {
    int ngroups;
    int first[MAX_GROUPS + 1];
};

// t -> (bi, bj).
__device__ bool tile_coords(const TileSpace& ts, const GroupTable& gt, int t, int* bi_out, int* bj_out) {
    int lo = 0, hi = gt.ngroups;  // last group whose first tile is <= t
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (gt.first[mid] <= t) lo = mid; else hi = mid;
    }
    t -= gt.first[lo];
    const int g0 = lo * ts.gs, g1 = min(ts.nbi, g0 + ts.gs);
    // columns that hold only part of the group (those that cross the diagonal)
    int bj = first_col(ts, g0);
    for (; bj < ts.nbj; bj++) {
        const int rows = min(g1 - 1, last_row(ts, bj)) - g0 + 1;  // rows g0 .. of the group in column bj
        if (rows == g1 - g0) break;  // from here on every column holds the whole group
        if (t < rows) {
            *bi_out = g0 + t;
            *bj_out = bj;
            return true;
        }
        t -= rows;
    }
    const int full = g1 - g0;
    bj += t / full;
    if (bj >= ts.nbj) return false;
    *bi_out = g0 + t % full;
    *bj_out = bj;
    return true;
}

// Tensor maps of every K chunk: A boxes (128 rows of the pos copy) and B
// boxes (224 rows of the neg copy), and the 128-byte K blocks of each chunk.
struct TcMaps {
    CUtensorMap a[kMaxKChunks];
    CUtensorMap b[kMaxKChunks];
    int kblocks[kMaxKChunks];
    int n;
};

// One triangle of a batch: its geometry, K stages, tensor maps and output.
struct TcJob {
    int n, rows, kblocks;  // rows [0, rows) against columns [0, n) of one set (r0 = c0 = 0)
    int nchunks;           // K chunks: A maps at jmaps[map0 ..), B maps at jmaps[map0 + nchunks ..)
    int kbl[kMaxKChunks];  // K stages of each chunk
    int map0;
    int tile0;             // first tile of the job in the launch
    TileSpace ts;          // one raster group
    const uint16_t* rdense;
    size_t ldr;
    uint16_t* out;
    size_t ldo;
    int vec_store;
};

// One stripe (the fields below `err` unused), or a batch of triangles
// (MULTI: `jobs`, their tensor maps `jmaps` and the job of every tile
// `tile_job`, all in device memory, written before the launch).
struct TcParams {
    int n, r0, rows;  // columns end at n; rows [r0, r0 + rows) of the A operand
    int c0;           // first column: r0 (upper triangle) or 0 (rectangle)
    int kblocks;      // K stages per tile
    TileSpace ts;
    GroupTable gt;
    int num_tiles;
    const uint16_t* rdense;  // dense rare counts (row stride ldr, column j at j - c0), or null
    size_t ldr;
    uint16_t* out;
    size_t ldo;
    int vec_store;  // 1: 16-byte stores (ldo a multiple of 8, out 16-byte aligned)
    int* err;
    const TcJob* jobs;
    const CUtensorMap* jmaps;
    const int* tile_job;
};

// t -> (bi, bj) when the whole triangle is one raster group (a batch job).
__device__ bool tile_coords_one_group(const TileSpace& ts, int t, int* bi_out, int* bj_out) {
    const int g1 = ts.nbi;
    int bj = first_col(ts, 0);
    for (; bj < ts.nbj; bj++) {
        const int rows = min(g1 - 1, last_row(ts, bj)) + 1;
        if (rows == g1) break;
        if (t < rows) {
            *bi_out = t;
            *bj_out = bj;
            return true;
        }
        t -= rows;
    }
    bj += t / g1;
    if (bj >= ts.nbj) return false;
    *bi_out = t % g1;
    *bj_out = bj;
    return true;
}

template <bool MULTI>
__global__ void __launch_bounds__(THREADS, 1) tc_stripe_kernel(const __grid_constant__ TcMaps maps, const TcParams p) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* stage_a = smem;
    uint8_t* stage_b = smem + STAGES * A_BYTES;
    uint64_t* bars = (uint64_t*)(smem + STAGES * STAGE_BYTES);
    uint64_t* full = bars;                     // STAGES
    uint64_t* empty = bars + STAGES;           // STAGES
    uint64_t* tfull = bars + 2 * STAGES;       // 2
    uint64_t* tempty = bars + 2 * STAGES + 2;  // 2
    uint64_t* drain = bars + 2 * STAGES + 4;   // 1
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 5);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    // this CTA's tiles: every gridDim.x-th one (in a batch the CTAs then work
    // on the same set's tiles at the same time, which keeps its operand in L2:
    // one contiguous range of tiles per CTA, split by work, measured 43.1 ms
    // against 34.1 ms on 512 sets)
    const int t_begin = blockIdx.x, t_end = p.num_tiles, t_step = gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], EPI_WARPS);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (!MULTI)
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
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    // scale factors 1.0 in every lane of the 32 scale-factor columns, one
    // epilogue warp per lane quarter, before any MMA reads them
    if (warp >= 2 && warp < 6) {
        tmem_fill32(tmem_base + ((uint32_t)((warp & 3) * 32) << 16) + SF_COL, 0x01010101u * kUe8m0One);
        tmem_wait_st();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            int s = 0;
            uint32_t ph = 0;
            bool ok = true;
            int issued[STAGES];
            uint32_t issued_ph[STAGES];
            for (int q = 0; q < STAGES; q++) issued[q] = 0, issued_ph[q] = 0;
            int last_job = -1;  // MULTI: the job whose maps this thread has acquired
            for (int t = t_begin; ok && t < t_end; t += t_step) {
                int bi, bj, y_a, y_b, kblocks;
                const CUtensorMap* ma = maps.a;
                const CUtensorMap* mb = maps.b;
                const int* kbls = maps.kblocks;
                if (!MULTI) {
                    if (!tile_coords(p.ts, p.gt, t, &bi, &bj)) break;
                    y_a = p.r0 + bi * BM;
                    y_b = p.c0 + bj * BN;
                    kblocks = p.kblocks;
                } else {
                    const int job = __ldg(p.tile_job + t);
                    const TcJob& jb = p.jobs[job];
                    if (!tile_coords_one_group(jb.ts, t - jb.tile0, &bi, &bj)) break;
                    y_a = bi * BM;
                    y_b = bj * BN;
                    kblocks = jb.kblocks;
                    ma = p.jmaps + jb.map0;
                    mb = ma + jb.nchunks;
                    kbls = jb.kbl;
                    if (job != last_job) {
                        for (int c = 0; c < 2 * jb.nchunks; c++) tensormap_acquire(ma + c);
                        last_job = job;
                    }
                }
                int ch = 0, kbl = 0;  // K chunk and block inside it
                int kbl_end = kbls[0];
                for (int kb = 0; kb < kblocks; kb++) {
                    if (!mbar_wait(&empty[s], ph ^ 1, abort_flag, p.err)) { ok = false; break; }
                    mbar_expect_tx(&full[s], STAGE_BYTES);
                    tma_load_2d(ma + ch, &full[s], stage_a + s * A_BYTES, kbl * BK, y_a);
                    tma_load_2d(mb + ch, &full[s], stage_b + s * B_BYTES, kbl * BK, y_b);
                    if (++kbl == kbl_end) {
                        kbl = 0;
                        if (++ch < kMaxKChunks) kbl_end = kbls[ch];
                    }
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
            const uint32_t idesc = make_idesc_mx(kE2M1, 1, BM, BN);
            const uint32_t sf = tmem_base + SF_COL;
            int s = 0, acc = 0;
            uint32_t ph = 0, aph = 0;
            bool ok = true;
            for (int t = t_begin; ok && t < t_end; t += t_step) {
                const int kblocks = MULTI ? p.jobs[__ldg(p.tile_job + t)].kblocks : p.kblocks;
                if (!mbar_wait(&tempty[acc], aph ^ 1, abort_flag, p.err)) { ok = false; break; }
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + (uint32_t)(acc * ACC_STRIDE);
                for (int kb = 0; kb < kblocks; kb++) {
                    if (!mbar_wait(&full[s], ph, abort_flag, p.err)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(stage_a + s * A_BYTES), b0 = smem_u32(stage_b + s * B_BYTES);
#pragma unroll
                    for (int k = 0; k < BK / 32; k++)
                        tc_mma_mxf4(d_tmem, sw128_desc(a0 + 32 * k), sw128_desc(b0 + 32 * k), idesc, sf, sf,
                                    (kb | k) ? 1u : 0u);
                    tc_commit(&empty[s]);  // stage free once these MMAs have read it
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
        const int q = warp & 3;           // TMEM lanes [32 q, 32 q + 32) belong to this warp
        const int half = (warp - 2) / 4;  // column half of the tile
        int acc = 0;
        uint32_t aph = 0;
        int bad = 0;
        for (int t = t_begin; t < t_end; t += t_step) {
            int bi, bj;
            int n = p.n, r0 = p.r0, c0 = p.c0, iend = p.r0 + p.rows, vec_store = p.vec_store;
            const uint16_t* rdense = p.rdense;
            uint16_t* out = p.out;
            size_t ldo = p.ldo, ldr = p.ldr;
            if (!MULTI) {
                if (!tile_coords(p.ts, p.gt, t, &bi, &bj)) break;
            } else {
                const TcJob& jb = p.jobs[__ldg(p.tile_job + t)];
                if (!tile_coords_one_group(jb.ts, t - jb.tile0, &bi, &bj)) break;
                n = jb.n;
                r0 = 0;
                c0 = 0;
                iend = jb.rows;
                vec_store = jb.vec_store;
                rdense = jb.rdense;
                out = jb.out;
                ldo = jb.ldo;
                ldr = jb.ldr;
            }
            const bool dense = rdense != nullptr;
            const int i = r0 + bi * BM + q * 32 + lane;  // this lane's row
            const int j0 = c0 + bj * BN;
            const bool row_ok = i < iend;
            const size_t orow = (size_t)(i - r0) * ldo;
            const size_t rrow = (size_t)(i - r0) * ldr;
            if (!mbar_wait(&tfull[acc], aph, abort_flag, p.err)) break;
            tc_fence_after();
            const uint32_t tbase = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * ACC_STRIDE);
#pragma unroll 1
            for (int cc = 0; cc < WARP_CHUNKS; cc++) {
                const int c = half * WARP_CHUNKS + cc;
                const int cb = j0 + c * CHUNK;  // first column of the chunk
                const bool live = row_ok && cb < n;
                // this row's rare counts for the chunk (32 bytes), fetched before
                // the accumulator read so the two overlap; a row of the block is
                // at least up(n - c0, 16) wide, so a live chunk is in bounds
                uint4 r4[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
                if (dense && live) {
                    const uint4* src = reinterpret_cast<const uint4*>(rdense + rrow + (size_t)(cb - c0));
                    r4[0] = __ldg(src);
                    r4[1] = __ldg(src + 1);
                }
                uint32_t v[16];
                tmem_ld16(tbase + (uint32_t)(c * CHUNK), v);
                tmem_wait_ld();
                if (cc == WARP_CHUNKS - 1) {  // this warp's part of the accumulator is read: hand it back
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[acc]);
                }
                uint32_t w[8];
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const float f0 = __uint_as_float(v[2 * e]), f1 = __uint_as_float(v[2 * e + 1]);
                    int x0 = __float2int_rn(f0), x1 = __float2int_rn(f1);
                    bad |= (__int2float_rn(x0) != f0) | (__int2float_rn(x1) != f1);
                    const uint4& r = r4[e / 4];
                    const uint32_t rw = (e % 4 == 0) ? r.x : (e % 4 == 1) ? r.y : (e % 4 == 2) ? r.z : r.w;
                    x0 -= (int)(rw & 0xFFFF);
                    x1 -= (int)(rw >> 16);
                    w[e] = (uint32_t)(x0 & 0xFFFF) | ((uint32_t)(x1 & 0xFFFF) << 16);
                }
                if (live) {
                    uint16_t* dst = out + orow + (size_t)(cb - c0);
                    if (cb + CHUNK <= n) {
                        if (vec_store) {
                            uint4* d4 = reinterpret_cast<uint4*>(dst);
                            d4[0] = make_uint4(w[0], w[1], w[2], w[3]);
                            d4[1] = make_uint4(w[4], w[5], w[6], w[7]);
                        } else {
                            uint32_t* d1 = reinterpret_cast<uint32_t*>(dst);
#pragma unroll
                            for (int e = 0; e < 8; e++) d1[e] = w[e];
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < CHUNK; e++)
                            if (cb + e < n) dst[e] = (uint16_t)(w[e / 2] >> (16 * (e & 1)));
                    }
                }
            }
            if (++acc == 2) acc = 0, aph ^= 1;
        }
        if (bad) atomicOr(p.err, DEVERR_OVERFLOW);
    }

    tc_fence_before();
    __syncthreads();
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

// rows x kb bytes, boxes of 128 bytes of K x box_rows rows, 128-byte swizzle.
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

bool same_chunking(const KChunks& x, const KChunks& y) { return x.n == y.n && x.width == y.width && x.kb == y.kb; }

cudaError_t launch_one(const Fp4Operands& A, const Fp4Operands& B, const uint16_t* R, size_t ldr,
                       const StripeArgs& a, int num_sms, cudaStream_t st) {
    static bool attrs[kMaxDevices] = {};
    const int dev = current_device();
    if (!attrs[dev]) {
        const cudaError_t e = cudaFuncSetAttribute(tc_stripe_kernel<false>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) return e;
        attrs[dev] = true;
    }
    const KChunks& ka = A.pos;
    const KChunks& kb = B.neg;
    if (A.kb <= 0 || (A.kb % BK) || B.kb != A.kb) return cudaErrorInvalidValue;
    if (ka.n < 1 || ka.kb != A.kb || !same_chunking(ka, kb) || (ka.width % BK)) return cudaErrorInvalidValue;
    if ((a.ldo & 1) || ((uintptr_t)a.out & 3)) return cudaErrorInvalidValue;
    if (R && ((ldr & 7) || ((uintptr_t)R & 15))) return cudaErrorInvalidValue;
    TcMaps maps;
    maps.n = ka.n;
    for (int c = 0; c < ka.n; c++) {
        const int wc = ka.width_of(c);
        if (wc <= 0 || (wc % BK)) return cudaErrorInvalidValue;
        if (!make_map(&maps.a[c], ka.p[c], A.n_rows, wc, BM) || !make_map(&maps.b[c], kb.p[c], B.n_rows, wc, BN))
            return cudaErrorInvalidValue;
        maps.kblocks[c] = wc / BK;
    }
    TcParams p;
    p.n = a.n;
    p.r0 = a.r0;
    p.c0 = a.rect ? 0 : a.r0;
    p.rows = a.rows;
    p.kblocks = A.kb / BK;
    p.ts.gs = a.group > 0 ? std::min(a.group, 256) : group_row_blocks();
    p.ts.nbi = (a.rows + BM - 1) / BM;
    p.ts.rect = a.rect ? 1 : 0;
    p.ts.nbj = (a.n - p.c0 + BN - 1) / BN;
    const long long tiles = tiles_in(p.ts, 0, p.ts.nbi);
    if (tiles > INT32_MAX) return cudaErrorInvalidValue;
    p.num_tiles = (int)tiles;
    {
        const int gs = p.ts.gs;
        p.gt.ngroups = (p.ts.nbi + gs - 1) / gs;
        if (p.gt.ngroups > MAX_GROUPS) return cudaErrorInvalidValue;  // callers split taller stripes
        long long acc = 0;
        for (int g = 0; g < p.gt.ngroups; g++) {
            p.gt.first[g] = (int)acc;
            acc += tiles_in(p.ts, g * gs, std::min(p.ts.nbi, g * gs + gs));
        }
        p.gt.first[p.gt.ngroups] = (int)acc;
    }
    p.rdense = R;
    p.ldr = ldr;
    p.out = a.out;
    p.ldo = a.ldo;
    p.vec_store = ((a.ldo & 7) == 0 && ((uintptr_t)a.out & 15) == 0) ? 1 : 0;
    p.err = a.err;
    p.jobs = nullptr;
    p.jmaps = nullptr;
    p.tile_job = nullptr;
    if (p.num_tiles == 0) return cudaSuccess;
    const int grid = std::min(p.num_tiles, std::max(num_sms, 1));
    tc_stripe_kernel<false><<<grid, THREADS, SMEM_BYTES, st>>>(maps, p);
    return cudaGetLastError();
}

}  // namespace

cudaError_t tc_batch_prepare(const std::vector<TcBatchItem>& items, int num_sms, TcBatchPlan* plan, int* err) {
    std::vector<TcJob> jobs;
    std::vector<CUtensorMap> mh;
    std::vector<int> tile_job;
    int tile0 = 0;
    for (const TcBatchItem& it : items) {
        const Fp4Operands& A = *it.ops;
        if (it.n < 2) continue;
        const KChunks& ka = A.pos;
        const KChunks& kb = A.neg;
        if (A.kb <= 0 || (A.kb % BK) || ka.n < 1 || ka.kb != A.kb || !same_chunking(ka, kb) || (ka.width % BK))
            return cudaErrorInvalidValue;
        if ((it.ldo & 1) || ((uintptr_t)it.out & 3)) return cudaErrorInvalidValue;
        if (it.R && ((it.ldr & 7) || ((uintptr_t)it.R & 15))) return cudaErrorInvalidValue;
        TcJob jb = TcJob{};
        jb.n = it.n;
        jb.rows = it.n;
        jb.kblocks = A.kb / BK;
        jb.nchunks = ka.n;
        jb.map0 = (int)mh.size();
        for (int c = 0; c < ka.n; c++) {
            CUtensorMap m;
            if (!make_map(&m, ka.p[c], A.n_rows, ka.width_of(c), BM)) return cudaErrorInvalidValue;
            mh.push_back(m);
            jb.kbl[c] = ka.width_of(c) / BK;
        }
        for (int c = 0; c < ka.n; c++) {
            CUtensorMap m;
            if (!make_map(&m, kb.p[c], A.n_rows, kb.width_of(c), BN)) return cudaErrorInvalidValue;
            mh.push_back(m);
        }
        jb.ts.nbi = (it.n + BM - 1) / BM;
        jb.ts.nbj = (it.n + BN - 1) / BN;
        jb.ts.gs = jb.ts.nbi;
        jb.ts.rect = 0;
        jb.rdense = it.R;
        jb.ldr = it.ldr;
        jb.out = it.out;
        jb.ldo = it.ldo;
        jb.vec_store = ((it.ldo & 7) == 0 && ((uintptr_t)it.out & 15) == 0) ? 1 : 0;
        const long long tiles = tiles_in(jb.ts, 0, jb.ts.nbi);
        if ((long long)tile0 + tiles > INT32_MAX) return cudaErrorInvalidValue;
        jb.tile0 = tile0;
        tile0 += (int)tiles;
        tile_job.insert(tile_job.end(), (size_t)tiles, (int)jobs.size());
        jobs.push_back(jb);
    }
    tc_batch_release(plan);
    plan->err = err;
    plan->njobs = (int)jobs.size();
    plan->num_tiles = tile0;
    if (jobs.empty()) return cudaSuccess;
    plan->grid = std::max(1, std::min(tile0, num_sms));
    cudaError_t e = cudaMalloc(&plan->d_jobs, jobs.size() * sizeof(TcJob));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_maps, mh.size() * sizeof(CUtensorMap));
    if (e == cudaSuccess) e = cudaMalloc(&plan->d_tile_job, tile_job.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(plan->d_jobs, jobs.data(), jobs.size() * sizeof(TcJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(plan->d_maps, mh.data(), mh.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(plan->d_tile_job, tile_job.data(), tile_job.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    static bool attrs[kMaxDevices] = {};
    const int dev = current_device();
    if (!attrs[dev]) {
        e = cudaFuncSetAttribute(tc_stripe_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) return e;
        attrs[dev] = true;
    }
    return cudaSuccess;
}

cudaError_t launch_tc_batch(const TcBatchPlan& plan, cudaStream_t st) {
    if (plan.num_tiles == 0 || plan.njobs == 0) return cudaSuccess;
    TcMaps maps;  // the batch's maps are in device memory
    maps.n = 0;
    TcParams p = TcParams{};
    p.gt.ngroups = 0;
    p.num_tiles = plan.num_tiles;
    p.err = plan.err;
    p.jobs = static_cast<const TcJob*>(plan.d_jobs);
    p.jmaps = static_cast<const CUtensorMap*>(plan.d_maps);
    p.tile_job = static_cast<const int*>(plan.d_tile_job);
    tc_stripe_kernel<true><<<plan.grid, THREADS, SMEM_BYTES, st>>>(maps, p);
    return cudaGetLastError();
}

void tc_batch_release(TcBatchPlan* plan) {
    plan->grid = 0;
    if (plan->d_jobs) cudaFree(plan->d_jobs);
    if (plan->d_maps) cudaFree(plan->d_maps);
    if (plan->d_tile_job) cudaFree(plan->d_tile_job);
    plan->d_jobs = plan->d_maps = plan->d_tile_job = nullptr;
    plan->njobs = plan->num_tiles = 0;
}

cudaError_t launch_tc_stripe(const Fp4Operands& ops, const Fp4Operands* bops, const uint16_t* R, size_t ldr,
                             const StripeArgs& a, int num_sms, cudaStream_t st) {
    if (a.rows <= 0 || (!a.rect && a.r0 >= a.n) || (a.rect && a.n <= 0)) return cudaSuccess;
    if (a.rect && !bops) return cudaErrorInvalidValue;
    const Fp4Operands& b = bops ? *bops : ops;
    // one launch covers at most MAX_GROUPS raster groups of rows; a taller
    // stripe runs as consecutive sub-stripes writing into the same output
    const int group = a.group > 0 ? std::min(a.group, 256) : group_row_blocks();
    const int max_rows = MAX_GROUPS * group * BM;
    for (int done = 0; done < a.rows; done += max_rows) {
        StripeArgs s = a;
        s.r0 = a.r0 + done;
        s.rows = std::min(max_rows, a.rows - done);
        const size_t col = a.rect ? 0 : (size_t)done;  // a triangle's columns start at its first row
        s.out = a.out + (size_t)done * a.ldo + col;
        const uint16_t* Rs = R ? R + (size_t)done * ldr + col : nullptr;
        const cudaError_t e = launch_one(ops, b, Rs, ldr, s, num_sms, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace tch
