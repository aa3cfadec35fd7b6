// CUDA-core contraction: LOP3 AND + popcount over the bit-packed rows.
//
// One CTA computes a 64 x 128 tile of one stripe:
//   acc(i, j) = sum_w popc(P_i[w] & P_j[w]) - sum_w popc(O_i[w] & O_j[w])
// i.e. P Pt - O Ot of the reference (tensorcore/rs/cuda/tch.cu:128-129, two
// b1 GEMMs with beta = -1), then the rare pairs of the tile's rows are
// subtracted in shared memory and the tile is narrowed to u16 and stored
// (tch.cu:130-131 fused).  Tiles entirely below the diagonal are skipped.
//
// This kernel is the CUDA-core baseline the tensor-core kernels are measured
// against, and it reads the reference's bit layout as is (no expansion).

#include "tch_internal.cuh"

namespace tch {
namespace {

constexpr int BM = 64, BN = 128, KW = 32, THREADS = 256;
constexpr int APITCH = KW + 1;  // words; +1 keeps column reads conflict-free
constexpr int CPITCH = BN + 1;

__device__ __forceinline__ void load_tile(uint32_t* __restrict__ sm, const uint32_t* __restrict__ src,
                                          int words_per_row, int row0, int nrows, int row_limit, int k0) {
    // nrows x KW words; consecutive threads read consecutive words of a row.
    for (int idx = threadIdx.x; idx < nrows * KW; idx += THREADS) {
        const int r = idx / KW, w = idx % KW, g = row0 + r;
        sm[r * APITCH + w] = g < row_limit ? __ldg(src + (size_t)g * words_per_row + k0 + w) : 0u;
    }
}

// Binary search: first index p in [lo, hi) with js[p] >= key.
__device__ __forceinline__ uint32_t lower_bound(const uint32_t* __restrict__ js, uint32_t lo, uint32_t hi,
                                                uint32_t key) {
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (__ldg(js + mid) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(THREADS)
popc_stripe_kernel(const uint32_t* __restrict__ P, int wP, const uint32_t* __restrict__ O, int wO, int n,
                   int r0, int rows, const uint32_t* __restrict__ start, const uint32_t* __restrict__ js,
                   int fuse_rare, uint16_t* __restrict__ out, size_t ldo) {
    extern __shared__ uint32_t smem[];
    const int i0 = r0 + blockIdx.y * BM;  // first row of the tile
    const int j0 = r0 + blockIdx.x * BN;  // first column of the tile
    if (j0 + BN <= i0) return;            // every cell has j < i
    const int iend = r0 + rows;

    uint32_t* As = smem;                   // BM x APITCH
    uint32_t* Bs = smem + BM * APITCH;     // BN x APITCH
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    int acc[4][8];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) acc[a][b] = 0;

    // presence part (+), then one-hot part (-)
    for (int part = 0; part < 2; part++) {
        const uint32_t* M = part == 0 ? P : O;
        const int wpr = part == 0 ? wP : wO;
        for (int k0 = 0; k0 < wpr; k0 += KW) {
            load_tile(As, M, wpr, i0, BM, iend, k0);
            load_tile(Bs, M, wpr, j0, BN, n, k0);
            __syncthreads();
#pragma unroll 4
            for (int w = 0; w < KW; w++) {
                uint32_t av[4], bv[8];
#pragma unroll
                for (int a = 0; a < 4; a++) av[a] = As[(ty + 16 * a) * APITCH + w];
#pragma unroll
                for (int b = 0; b < 8; b++) bv[b] = Bs[(tx + 16 * b) * APITCH + w];
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 8; b++) {
                        const int c = __popc(av[a] & bv[b]);
                        acc[a][b] += part == 0 ? c : -c;
                    }
            }
            __syncthreads();
        }
    }

    // tile -> shared memory (reuses the operand buffers)
    int* Cs = reinterpret_cast<int*>(smem);
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) Cs[(ty + 16 * a) * CPITCH + tx + 16 * b] = acc[a][b];
    __syncthreads();

    // rare pairs of this tile: one warp per row, lanes stride over the row's
    // partners inside [j0, j0 + BN) (ascending lists: binary search + walk)
    if (fuse_rare) {
        const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
        for (int r = warp; r < BM; r += THREADS / 32) {
            const int i = i0 + r;
            if (i >= iend) break;
            const uint32_t lo = lower_bound(js, __ldg(start + i), __ldg(start + i + 1), (uint32_t)j0);
            const uint32_t hi = __ldg(start + i + 1);
            for (uint32_t p = lo + lane; p < hi; p += 32) {
                const uint32_t j = __ldg(js + p);
                if (j >= (uint32_t)(j0 + BN)) break;
                atomicSub(&Cs[r * CPITCH + (int)(j - j0)], 1);
            }
        }
        __syncthreads();
    }

    // u16 store, coalesced along the row
    for (int idx = threadIdx.x; idx < BM * BN; idx += THREADS) {
        const int r = idx / BN, c = idx % BN, i = i0 + r, j = j0 + c;
        if (i < iend && j < n) out[(size_t)(i - r0) * ldo + (j - r0)] = (uint16_t)Cs[r * CPITCH + c];
    }
}

// The reference's sub_rare (tch.cu:36-43) for partner lists in any order, on
// the u16 stripe: one warp per row, 32-bit atomics on the word holding the
// cell (the cell never goes below zero, so no borrow reaches its neighbour).
__global__ void rare_atomic_kernel(uint16_t* __restrict__ out, size_t ldo, int n, int r0, int rows,
                                   const uint32_t* __restrict__ start, const uint32_t* __restrict__ js,
                                   int* err, const int* only_if_unsorted) {
    // with a check flag: the stripe kernel already subtracted ascending lists
    if (only_if_unsorted && *only_if_unsorted == 0) return;
    const int r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x % 32;
    if (r >= rows) return;
    const int i = r0 + r;
    const uint32_t hi = __ldg(start + i + 1);
    for (uint32_t p = __ldg(start + i) + lane; p < hi; p += 32) {
        const uint32_t j = __ldg(js + p);
        if (j <= (uint32_t)i || j >= (uint32_t)n) {
            atomicOr(err, DEVERR_RARE_PAIR);
            continue;
        }
        const size_t e = (size_t)r * ldo + (j - r0);
        uint32_t* word = reinterpret_cast<uint32_t*>(out) + (e >> 1);
        atomicSub(word, 1u << ((e & 1) * 16));
    }
}

// flag stays 0 iff every row is ascending and every partner is in (i, n)
__global__ void rare_check_kernel(const uint32_t* __restrict__ start, const uint32_t* __restrict__ js, int n,
                                  int r_begin, int r_end, int* bad) {
    const int i = r_begin + blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x % 32;
    if (i >= r_end) return;
    const uint32_t lo = __ldg(start + i), hi = __ldg(start + i + 1);
    int flag = 0;
    for (uint32_t p = lo + lane; p < hi; p += 32) {
        const uint32_t j = __ldg(js + p);
        if (j <= (uint32_t)i || j >= (uint32_t)n) flag |= 2;
        if (p > lo && __ldg(js + p - 1) > j) flag |= 1;
    }
    flag = __reduce_or_sync(0xffffffffu, flag);
    if (lane == 0 && flag) atomicOr(bad, flag);
}

}  // namespace

cudaError_t launch_popc_stripe(const BitOperands& ops, const RareCSR& rare, const StripeArgs& a,
                               cudaStream_t st) {
    if (a.rows <= 0 || a.r0 >= a.n) return cudaSuccess;
    const int w = a.n - a.r0;
    dim3 grid((w + BN - 1) / BN, (a.rows + BM - 1) / BM);
    const size_t smem = sizeof(uint32_t) * (size_t)((BM + BN) * APITCH > BM * CPITCH ? (BM + BN) * APITCH
                                                                                    : BM * CPITCH);
    const bool fuse = rare.n_rare > 0 && rare.sorted;
    popc_stripe_kernel<<<grid, THREADS, smem, st>>>(ops.P, ops.wP, ops.O, ops.wO, a.n, a.r0, a.rows, rare.start,
                                                    rare.js, fuse ? 1 : 0, a.out, a.ldo);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (rare.n_rare > 0 && !rare.sorted) return launch_rare_atomic(rare, a, st);
    return cudaSuccess;
}

cudaError_t launch_rare_atomic(const RareCSR& rare, const StripeArgs& a, cudaStream_t st) {
    if (rare.n_rare == 0 || a.rows <= 0) return cudaSuccess;
    rare_atomic_kernel<<<(a.rows + 7) / 8, 256, 0, st>>>(a.out, a.ldo, a.n, a.r0, a.rows, rare.start, rare.js,
                                                         a.err, rare.unsorted_flag);
    return cudaGetLastError();
}

cudaError_t launch_rare_check_sorted(const RareCSR& rare, int n, int* d_flag, cudaStream_t st, int r_begin,
                                     int r_end) {
    if (r_end < 0 || r_end > n) r_end = n;
    if (r_begin < 0) r_begin = 0;
    if (r_end <= r_begin) return cudaSuccess;
    rare_check_kernel<<<(r_end - r_begin + 7) / 8, 256, 0, st>>>(rare.start, rare.js, n, r_begin, r_end, d_flag);
    return cudaGetLastError();
}

}  // namespace tch
