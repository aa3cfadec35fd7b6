// Consumers of the distance matrix on the device: the exact minimum spanning
// tree, single-linkage clusters at thresholds and every profile's nearest
// neighbours -- the uses the reference's documentation names for the matrix
// (outbreak clustering, minimum spanning trees, nearest-neighbour searches;
// docs/index.html, "The problem").  The reference stops at the matrix.
//
// Both kernels read the full n x n u16 matrix in HBM row by row: a row is one
// contiguous run of n values that a CTA reads with 16-byte loads, so each
// pass over the matrix is bound by HBM bandwidth (2 n^2 bytes per pass).
//
// Minimum spanning tree (Borůvka).  Edges are ordered by (distance, smaller
// index, larger index), a strict order, so the tree is unique and equals
// Kruskal's under the same order.  Each round:
//   scan    every row's lightest edge to another component.  Within a row the
//           order above is (distance, column), so a thread keeps the first
//           column of its smallest distance while it walks its columns in
//           ascending order; the CTA reduces the row and one atomicMin folds it
//           into the best key of the row's component.  A CTA takes kScanRows
//           rows at once, so the component labels of the columns are loaded
//           once for all of them.
//   hook    every component root across its best edge to the component on
//           the other side, recording the edge (of two components that chose
//           the same edge, only the larger root hooks, which breaks the only
//           cycles such a choice can make);
//   relabel pointer doubling over the roots, ceil(log2 n) + 1 steps, then
//           every profile takes its root's new root.
// Each round at least halves the number of components, so at most
// ceil(log2 n) rounds.  No step waits on another thread.
//
// Nearest neighbours.  A CTA per row finds the k-th smallest distance T by a
// radix select on the u16 value (two passes of a 256-bin histogram in shared
// memory; lanes with the same bin are counted with one atomic), then a third
// pass collects the distances below T and, in column order, the first
// columns at distance T, and the k results are ranked by (distance, column).

#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "tch_internal.cuh"

namespace tch {
namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr int kScanThreads = 256;
constexpr int kScanRows = 4;  // rows of one scan CTA, sharing the column-label loads
constexpr int kNbrThreads = 256;
constexpr int kMaxNeighbors = 32;
constexpr int kIndexBits = 21;  // a profile index in an edge key
constexpr uint32_t kIndexMask = (1u << kIndexBits) - 1;
constexpr unsigned long long kNoEdge = ~0ull;
constexpr uint32_t kNoDistance = 0x10000u;  // above every u16 distance

enum LinkErr : int {
    LINKERR_EDGE = 1,     // a component's best edge does not leave it
    LINKERR_COUNT = 2,    // more than n - 1 tree edges
    LINKERR_SELECT = 4,   // the neighbour selection lost count
};

// (distance, smaller index, larger index) as one integer.
__device__ __forceinline__ unsigned long long edge_key(uint32_t w, uint32_t i, uint32_t j) {
    const uint32_t a = i < j ? i : j, b = i < j ? j : i;
    return ((unsigned long long)w << (2 * kIndexBits)) | ((unsigned long long)a << kIndexBits) | b;
}

// Value e (0..7) of eight u16 values packed in a uint4.
__device__ __forceinline__ uint32_t lane16(const uint4& h, int e) {
    const uint32_t x = e < 2 ? h.x : e < 4 ? h.y : e < 6 ? h.z : h.w;
    return (e & 1) ? x >> 16 : x & 0xFFFFu;
}

__device__ __forceinline__ unsigned long long warp_min64(unsigned long long v) {
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(FULL, v, o);
        v = t < v ? t : v;
    }
    return v;
}

// comp[x] = x for x < n; the padding up to up(n, 8) is never used as a label.
__global__ void mst_init_kernel(uint32_t* comp, int n, int n8) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n8) comp[x] = x < n ? (uint32_t)x : 0xFFFFFFFFu;
}

// best[comp[i]] = min over rows i of the component and columns j of other
// components of edge_key(H[i][j], i, j).  comp holds up(n, 8) entries.
__global__ void __launch_bounds__(kScanThreads) mst_scan_kernel(const uint16_t* __restrict__ H, size_t ld, int n,
                                                                const uint32_t* __restrict__ comp,
                                                                unsigned long long* best) {
    __shared__ unsigned long long part[kScanThreads / 32][kScanRows];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nq = (n + 7) >> 3;  // 8-column chunks of a row
    const uint4* comp4 = reinterpret_cast<const uint4*>(comp);
    for (int i0 = blockIdx.x * kScanRows; i0 < n; i0 += gridDim.x * kScanRows) {  // uniform over the CTA
        uint32_t ci[kScanRows], bw[kScanRows], bj[kScanRows];
        const uint4* row[kScanRows];
#pragma unroll
        for (int r = 0; r < kScanRows; r++) {
            const int i = i0 + r < n ? i0 + r : n - 1;
            ci[r] = i0 + r < n ? __ldg(comp + i) : 0xFFFFFFFFu;
            row[r] = reinterpret_cast<const uint4*>(H + (size_t)i * ld);
            bw[r] = kNoDistance;
            bj[r] = 0xFFFFFFFFu;
        }
        for (int q = threadIdx.x; q < nq; q += kScanThreads) {
            const uint4 c0 = __ldg(comp4 + 2 * q), c1 = __ldg(comp4 + 2 * q + 1);
            const uint32_t cj[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
            for (int r = 0; r < kScanRows; r++) {
                if (i0 + r >= n) break;
                const uint4 h = __ldcs(row[r] + q);  // read once per round: do not keep it in L1
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const uint32_t w = lane16(h, e);
                    const int j = 8 * q + e;
                    if (j < n && cj[e] != ci[r] && w < bw[r]) {
                        bw[r] = w;
                        bj[r] = (uint32_t)j;
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < kScanRows; r++) {
            const unsigned long long m = warp_min64(((unsigned long long)bw[r] << 32) | bj[r]);
            if (lane == 0) part[warp][r] = m;
        }
        __syncthreads();
        if (threadIdx.x < kScanRows && i0 + (int)threadIdx.x < n) {
            const int r = threadIdx.x;
            unsigned long long m = part[0][r];
            for (int w = 1; w < kScanThreads / 32; w++) m = part[w][r] < m ? part[w][r] : m;
            const uint32_t w = (uint32_t)(m >> 32), j = (uint32_t)m;
            if (w < kNoDistance) atomicMin(best + ci[r], edge_key(w, (uint32_t)(i0 + r), j));
        }
        __syncthreads();
    }
}

// parent[c] = the root that c hooks to this round (c itself when it does not).
__global__ void mst_hook_kernel(int n, const uint32_t* __restrict__ comp, const unsigned long long* __restrict__ best,
                                uint32_t* parent, unsigned long long* edges, unsigned int* nedges, int* err) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    uint32_t p = (uint32_t)c;
    const unsigned long long key = best[c];
    if (comp[c] == (uint32_t)c && key != kNoEdge) {
        const uint32_t u = (uint32_t)(key >> kIndexBits) & kIndexMask, v = (uint32_t)key & kIndexMask;
        if (u >= (uint32_t)n || v >= (uint32_t)n) {
            atomicOr(err, LINKERR_EDGE);
        } else {
            const uint32_t cu = comp[u], cv = comp[v];
            const uint32_t d = cu == (uint32_t)c ? cv : cu;
            if ((cu != (uint32_t)c && cv != (uint32_t)c) || d == (uint32_t)c || d >= (uint32_t)n) {
                atomicOr(err, LINKERR_EDGE);
            } else if (!(best[d] == key && (uint32_t)c < d)) {
                p = d;
                const unsigned int slot = atomicAdd(nedges, 1u);
                if (slot < (unsigned int)(n - 1))
                    edges[slot] = key;
                else
                    atomicOr(err, LINKERR_COUNT);
            }
        }
    }
    parent[c] = p;
}

__global__ void mst_jump_kernel(int n, const uint32_t* __restrict__ pa, uint32_t* __restrict__ pb) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) pb[x] = pa[pa[x]];
}

__global__ void mst_relabel_kernel(int n, uint32_t* comp, const uint32_t* __restrict__ root) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) comp[x] = root[comp[x]];
}

// Row i's k nearest columns (j != i) by (distance, column).
__global__ void __launch_bounds__(kNbrThreads) neighbors_kernel(const uint16_t* __restrict__ H, size_t ld, int n,
                                                                int k, uint32_t* idx, uint16_t* dist, int* err) {
    __shared__ uint32_t hist[256];
    __shared__ uint32_t wsum[kNbrThreads / 32];
    __shared__ unsigned long long res[kMaxNeighbors];
    __shared__ uint32_t pick[2];
    __shared__ uint32_t nlt;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nq = (n + 7) >> 3;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {  // uniform over the CTA
        const uint4* row = reinterpret_cast<const uint4*>(H + (size_t)i * ld);
        // radix select of T, the k-th smallest distance: high byte, then low byte
        uint32_t hi = 0, below = 0, want = (uint32_t)k, T = 0, c_lt = 0;
        for (int pass = 0; pass < 2; pass++) {
            for (int b = threadIdx.x; b < 256; b += kNbrThreads) hist[b] = 0;
            __syncthreads();
            for (int q0 = warp * 32; q0 < nq; q0 += kNbrThreads) {  // uniform over the warp
                const int q = q0 + lane;
                uint4 h = make_uint4(0, 0, 0, 0);
                if (q < nq) h = __ldg(row + q);
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const uint32_t w = lane16(h, e);
                    const int j = 8 * q + e;
                    const bool ok = q < nq && j < n && j != i && (pass == 0 || (w >> 8) == hi);
                    const uint32_t bin = pass == 0 ? w >> 8 : w & 0xFFu;
                    const unsigned peers = __match_any_sync(FULL, ok ? bin : 256u);
                    if (ok && lane == __ffs(peers) - 1) atomicAdd(hist + bin, (uint32_t)__popc(peers));
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t cum = 0, b = 0;
                for (; b < 255; b++) {
                    if (cum + hist[b] >= want) break;
                    cum += hist[b];
                }
                pick[0] = b;
                pick[1] = cum;
            }
            __syncthreads();
            if (pass == 0) {
                hi = pick[0];
                below = pick[1];
                want = (uint32_t)k - below;
            } else {
                T = (hi << 8) | pick[0];
                c_lt = below + pick[1];
            }
            __syncthreads();  // pick is rewritten by the next pass
        }
        // collect: every distance below T, then the first columns at T
        const uint32_t need = (uint32_t)k - c_lt;  // >= 1
        if (threadIdx.x == 0) nlt = 0;
        __syncthreads();
        uint32_t eq_base = 0;
        for (int q0 = 0; q0 < nq; q0 += kNbrThreads) {  // uniform over the CTA
            const int q = q0 + threadIdx.x;
            uint4 h = make_uint4(0, 0, 0, 0);
            if (q < nq) h = __ldg(row + q);
            uint32_t cnt = 0;
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const uint32_t w = lane16(h, e);
                const int j = 8 * q + e;
                const bool ok = q < nq && j < n && j != i;
                if (ok && w < T) {
                    const uint32_t s = atomicAdd(&nlt, 1u);
                    if (s < (uint32_t)kMaxNeighbors) res[s] = ((unsigned long long)w << 32) | (uint32_t)j;
                }
                cnt += (ok && w == T) ? 1u : 0u;
            }
            // exclusive scan of cnt over the CTA's threads (thread order = column order)
            uint32_t incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane == 31) wsum[warp] = incl;
            __syncthreads();
            uint32_t wbase = 0, total = 0;
            for (int w2 = 0; w2 < kNbrThreads / 32; w2++) {
                const uint32_t s2 = wsum[w2];
                wbase += w2 < warp ? s2 : 0u;
                total += s2;
            }
            uint32_t r = eq_base + wbase + incl - cnt;
            if (cnt && r < need) {
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const uint32_t w = lane16(h, e);
                    const int j = 8 * q + e;
                    if (q < nq && j < n && j != i && w == T) {
                        if (r < need) res[c_lt + r] = ((unsigned long long)w << 32) | (uint32_t)j;
                        r++;
                    }
                }
            }
            eq_base += total;
            __syncthreads();  // wsum is rewritten by the next chunk
        }
        if (threadIdx.x == 0 && (nlt != c_lt || eq_base < need)) atomicOr(err, LINKERR_SELECT);
        if ((int)threadIdx.x < k) {
            const unsigned long long key = res[threadIdx.x];
            int rank = 0;
            for (int s = 0; s < k; s++) rank += res[s] < key ? 1 : 0;
            idx[(size_t)i * k + rank] = (uint32_t)key;
            dist[(size_t)i * k + rank] = (uint16_t)(key >> 32);
        }
        __syncthreads();  // res and nlt are reused by the next row
    }
}

int check_matrix(const uint16_t* d_H, size_t ld, int n, Err& e) {
    if (n < 0) return e.set("n must be >= 0");
    if (n >= (1 << kIndexBits)) return e.set("n must be below %d", 1 << kIndexBits);
    if (n > 0 && !d_H) return e.set("null matrix");
    if (ld < (size_t)n || (ld & 7)) return e.set("ld must be >= n and a multiple of 8");
    if ((uintptr_t)d_H & 15) return e.set("the matrix must be 16-byte aligned");
    return 0;
}

int mst_on_device(const uint16_t* d_H, size_t ld, int n, cudaStream_t st, std::vector<unsigned long long>& keys,
                  Err& e) {
    keys.clear();
    if (check_matrix(d_H, ld, n, e)) return 1;
    if (n < 2) return 0;
    const size_t n8 = up((size_t)n, 8);
    char* ws = nullptr;
    uint32_t *comp, *pa, *pb;
    unsigned long long *best, *edges;
    unsigned int* nedges;
    int* derr;
    int dev = 0, sms = 0, rc = 1;
    unsigned int got = 0, prev = 0;
    int herr = 0;
    const int steps = 32 - __builtin_clz((unsigned)(n - 1)) + 1;  // ceil(log2 n) + 1
    const size_t bytes = n8 * 4 * 3 + (size_t)n * 8 * 2 + 64;
    TCH_CK(e, cudaGetDevice(&dev));
    TCH_CK(e, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TCH_CK(e, cudaMallocAsync(&ws, bytes, st));
    comp = reinterpret_cast<uint32_t*>(ws);
    pa = comp + n8;
    pb = pa + n8;
    best = reinterpret_cast<unsigned long long*>(pb + n8);
    edges = best + n;
    nedges = reinterpret_cast<unsigned int*>(edges + n);
    derr = reinterpret_cast<int*>(nedges + 4);
    TCH_CK(e, cudaMemsetAsync(nedges, 0, 32, st));
    mst_init_kernel<<<(unsigned)((n8 + 255) / 256), 256, 0, st>>>(comp, n, (int)n8);
    TCH_CK(e, cudaGetLastError());
    {
        const int rows_grid = (n + kScanRows - 1) / kScanRows;
        const int grid = std::max(1, std::min(rows_grid, sms * (2048 / kScanThreads)));
        const unsigned vgrid = (unsigned)((n + 255) / 256);
        // each round at least halves the components: ceil(log2 n) rounds at most
        for (int round = 0; got < (unsigned)(n - 1); round++) {
            if (round > steps) {
                e.set("minimum spanning tree: %u of %d edges after %d rounds", got, n - 1, round);
                goto fail;
            }
            TCH_CK(e, cudaMemsetAsync(best, 0xFF, (size_t)n * 8, st));
            mst_scan_kernel<<<grid, kScanThreads, 0, st>>>(d_H, ld, n, comp, best);
            mst_hook_kernel<<<vgrid, 256, 0, st>>>(n, comp, best, pa, edges, nedges, derr);
            uint32_t *from = pa, *to = pb;
            for (int s = 0; s < steps; s++) {
                mst_jump_kernel<<<vgrid, 256, 0, st>>>(n, from, to);
                std::swap(from, to);
            }
            mst_relabel_kernel<<<vgrid, 256, 0, st>>>(n, comp, from);
            TCH_CK(e, cudaGetLastError());
            TCH_CK(e, cudaMemcpyAsync(&got, nedges, 4, cudaMemcpyDeviceToHost, st));
            TCH_CK(e, cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st));
            TCH_CK(e, cudaStreamSynchronize(st));
            if (herr) {
                e.set("minimum spanning tree: device check failed (code %d)", herr);
                goto fail;
            }
            if (got == prev) {
                e.set("minimum spanning tree: no edge added in round %d", round);
                goto fail;
            }
            prev = got;
        }
    }
    keys.resize((size_t)n - 1);
    TCH_CK(e, cudaMemcpyAsync(keys.data(), edges, keys.size() * 8, cudaMemcpyDeviceToHost, st));
    TCH_CK(e, cudaStreamSynchronize(st));
    std::sort(keys.begin(), keys.end());
    {  // the edges must join every profile: n - 1 unions
        std::vector<uint32_t> p((size_t)n);
        std::iota(p.begin(), p.end(), 0u);
        auto find = [&](uint32_t x) {
            while (p[x] != x) x = p[x] = p[p[x]];
            return x;
        };
        for (unsigned long long k : keys) {
            const uint32_t a = find((uint32_t)(k >> kIndexBits) & kIndexMask), b = find((uint32_t)k & kIndexMask);
            if (a == b) {
                e.set("minimum spanning tree: the edges contain a cycle");
                goto fail;
            }
            p[std::max(a, b)] = std::min(a, b);
        }
    }
    rc = 0;
fail:
    if (ws) {
        cudaFreeAsync(ws, st);
        cudaStreamSynchronize(st);
    }
    if (rc) keys.clear();
    return rc;
}

int neighbors_on_device(const uint16_t* d_H, size_t ld, int n, int k, cudaStream_t st, uint32_t* idx,
                        uint16_t* dist, Err& e) {
    if (check_matrix(d_H, ld, n, e)) return 1;
    if (k < 1 || k > kMaxNeighbors) return e.set("k must be 1-%d", kMaxNeighbors);
    if (k >= n) return e.set("k must be below n (%d)", n);
    if (!idx || !dist) return e.set("null output");
    char* ws = nullptr;
    uint32_t* d_idx;
    uint16_t* d_dist;
    int* derr;
    int dev = 0, sms = 0, rc = 1, herr = 0;
    const size_t cells = (size_t)n * k;
    TCH_CK(e, cudaGetDevice(&dev));
    TCH_CK(e, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TCH_CK(e, cudaMallocAsync(&ws, cells * 6 + 64, st));
    d_idx = reinterpret_cast<uint32_t*>(ws);
    derr = reinterpret_cast<int*>(d_idx + cells);
    d_dist = reinterpret_cast<uint16_t*>(derr + 4);
    TCH_CK(e, cudaMemsetAsync(derr, 0, 4, st));
    neighbors_kernel<<<std::max(1, std::min(n, sms * (2048 / kNbrThreads))), kNbrThreads, 0, st>>>(d_H, ld, n, k,
                                                                                                 d_idx, d_dist, derr);
    TCH_CK(e, cudaGetLastError());
    TCH_CK(e, cudaMemcpyAsync(idx, d_idx, cells * 4, cudaMemcpyDeviceToHost, st));
    TCH_CK(e, cudaMemcpyAsync(dist, d_dist, cells * 2, cudaMemcpyDeviceToHost, st));
    TCH_CK(e, cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st));
    TCH_CK(e, cudaStreamSynchronize(st));
    if (herr) {
        e.set("nearest neighbours: device check failed (code %d)", herr);
        goto fail;
    }
    rc = 0;
fail:
    if (ws) {
        cudaFreeAsync(ws, st);
        cudaStreamSynchronize(st);
    }
    return rc;
}

// The solver's full matrix in device memory (upper triangle, then mirrored).
int full_matrix(tch_solver* s, int* n_out, uint16_t** H, size_t* ld, cudaStream_t st, char* err, int errlen) {
    Err e{err, errlen};
    tch_info info;
    *H = nullptr;
    if (!s || tch_solver_info(s, &info)) return e.set("bad solver");
    const int n = info.n;
    *n_out = n;
    *ld = up((size_t)std::max(n, 1), 8);
    if (n < 2) return 0;
    if (cudaMalloc(H, (size_t)n * *ld * 2) != cudaSuccess) {
        cudaGetLastError();
        *H = nullptr;
        return e.set("the full %d x %d matrix (%.1f GB) does not fit in device memory", n, n,
                     (double)n * *ld * 2 / 1e9);
    }
    if (tch_solver_stripe(s, 0, n, *H, *ld, st, err, errlen)) goto fail;
    TCH_CK(e, launch_mirror(*H, *ld, n, st));
    TCH_CK(e, cudaStreamSynchronize(st));
    if (tch_solver_check(s, err, errlen)) goto fail;
    return 0;
fail:
    cudaStreamSynchronize(st);
    cudaFree(*H);
    *H = nullptr;
    return 1;
}

void decode_edges(const std::vector<unsigned long long>& keys, uint32_t* u, uint32_t* v, uint16_t* w,
                  uint64_t* total) {
    uint64_t t = 0;
    for (size_t q = 0; q < keys.size(); q++) {
        const unsigned long long k = keys[q];
        const uint32_t dw = (uint32_t)(k >> (2 * kIndexBits));
        if (u) u[q] = (uint32_t)(k >> kIndexBits) & kIndexMask;
        if (v) v[q] = (uint32_t)k & kIndexMask;
        if (w) w[q] = (uint16_t)dw;
        t += dw;
    }
    if (total) *total = t;
}

struct StreamGuard {
    cudaStream_t st = nullptr;
    bool own = false;
    int make(void* stream) {
        if (stream) {
            st = (cudaStream_t)stream;
            return 0;
        }
        own = true;
        return cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess;
    }
    ~StreamGuard() {
        if (own && st) cudaStreamDestroy(st);
    }
};

}  // namespace
}  // namespace tch

using namespace tch;

extern "C" int tch_mst_device(const uint16_t* d_H, size_t ld, int n, void* stream, uint32_t* u, uint32_t* v,
                              uint16_t* w, uint64_t* total, char* err, int errlen) {
    Err e{err, errlen};
    StreamGuard g;
    if (g.make(stream)) return e.set("could not create a stream");
    std::vector<unsigned long long> keys;
    if (mst_on_device(d_H, ld, n, g.st, keys, e)) return 1;
    decode_edges(keys, u, v, w, total);
    return 0;
}

extern "C" int tch_neighbors_device(const uint16_t* d_H, size_t ld, int n, int k, void* stream, uint32_t* idx,
                                    uint16_t* dist, char* err, int errlen) {
    Err e{err, errlen};
    StreamGuard g;
    if (g.make(stream)) return e.set("could not create a stream");
    return neighbors_on_device(d_H, ld, n, k, g.st, idx, dist, e);
}

extern "C" int tch_solver_mst(tch_solver* s, uint32_t* u, uint32_t* v, uint16_t* w, uint64_t* total, char* err,
                              int errlen) {
    Err e{err, errlen};
    StreamGuard g;
    uint16_t* H = nullptr;
    size_t ld = 0;
    int n = 0, rc = 1;
    std::vector<unsigned long long> keys;
    if (g.make(nullptr)) return e.set("could not create a stream");
    if (full_matrix(s, &n, &H, &ld, g.st, err, errlen)) return 1;
    if (n >= 2 && mst_on_device(H, ld, n, g.st, keys, e)) goto done;
    decode_edges(keys, u, v, w, total);
    rc = 0;
done:
    cudaFree(H);
    return rc;
}

extern "C" int tch_solver_neighbors(tch_solver* s, int k, uint32_t* idx, uint16_t* dist, char* err, int errlen) {
    Err e{err, errlen};
    tch_info info;
    StreamGuard g;
    uint16_t* H = nullptr;
    size_t ld = 0;
    int n = 0, rc;
    if (!s || tch_solver_info(s, &info)) return e.set("bad solver");
    if (k < 1 || k > kMaxNeighbors) return e.set("k must be 1-%d", kMaxNeighbors);
    if (k >= info.n) return e.set("k must be below n (%d)", info.n);
    if (g.make(nullptr)) return e.set("could not create a stream");
    if (full_matrix(s, &n, &H, &ld, g.st, err, errlen)) return 1;
    rc = neighbors_on_device(H, ld, n, k, g.st, idx, dist, e);
    cudaFree(H);
    return rc;
}

extern "C" int tch_mst_clusters(int n, const uint32_t* u, const uint32_t* v, const uint16_t* w, size_t m,
                                const uint32_t* thresholds, int nt, uint32_t* labels, char* err, int errlen) {
    Err e{err, errlen};
    if (n < 0 || nt < 0) return e.set("n and nt must be >= 0");
    if (nt > 0 && n > 0 && (!thresholds || !labels)) return e.set("null thresholds or labels");
    if (m > 0 && (!u || !v || !w)) return e.set("null edges");
    for (size_t q = 0; q < m; q++)
        if (u[q] >= (uint32_t)n || v[q] >= (uint32_t)n || u[q] == v[q])
            return e.set("edge %zu (%u, %u) is not between two of the %d profiles", q, u[q], v[q], n);
    std::vector<size_t> by_w(m);
    std::iota(by_w.begin(), by_w.end(), (size_t)0);
    std::stable_sort(by_w.begin(), by_w.end(), [&](size_t a, size_t b) { return w[a] < w[b]; });
    std::vector<int> by_t((size_t)nt);
    std::iota(by_t.begin(), by_t.end(), 0);
    std::stable_sort(by_t.begin(), by_t.end(), [&](int a, int b) { return thresholds[a] < thresholds[b]; });
    // union by the smaller root: a set's root is its smallest profile index
    std::vector<uint32_t> p((size_t)n);
    std::iota(p.begin(), p.end(), 0u);
    auto find = [&](uint32_t x) {
        while (p[x] != x) x = p[x] = p[p[x]];
        return x;
    };
    size_t q = 0;
    for (int t : by_t) {
        for (; q < m && w[by_w[q]] <= thresholds[t]; q++) {
            const uint32_t a = find(u[by_w[q]]), b = find(v[by_w[q]]);
            if (a != b) p[std::max(a, b)] = std::min(a, b);
        }
        uint32_t* out = labels + (size_t)t * n;
        for (int i = 0; i < n; i++) out[i] = find((uint32_t)i);
    }
    return 0;
}

extern "C" int tch_solver_clusters(tch_solver* s, const uint32_t* thresholds, int nt, uint32_t* labels, char* err,
                                   int errlen) {
    Err e{err, errlen};
    tch_info info;
    if (!s || tch_solver_info(s, &info)) return e.set("bad solver");
    const int n = info.n;
    const size_t m = n > 1 ? (size_t)n - 1 : 0;
    std::vector<uint32_t> u(m), v(m);
    std::vector<uint16_t> w(m);
    if (tch_solver_mst(s, u.data(), v.data(), w.data(), nullptr, err, errlen)) return 1;
    return tch_mst_clusters(n, u.data(), v.data(), w.data(), m, thresholds, nt, labels, err, errlen);
}
