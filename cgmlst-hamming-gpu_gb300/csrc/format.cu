// The distance matrix as TSV text, formatted on the GPU (the reference's
// write_matrix, tensorcore/rs/src/main.rs:224-265: a header line, then per
// sample its id and n distances, layout mask then cap, decimal, separator
// before every value, newline).
//
// The whole upper triangle is computed into HBM by the solver; a tiled
// transpose mirrors it into the lower half when the layout shows it.  Rows are
// then formatted in blocks: a warp per row sums the field lengths, one CTA
// scans them into offsets, and a warp per row writes its text, 32 values at a
// time (lane = value; a warp scan of the field lengths gives every lane its
// position).  Each block's text goes to pinned host memory while the next
// block is formatted, and the caller's callback receives the blocks in order.

#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "tch_internal.cuh"

namespace tch {
namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr int TT = 32;  // transpose tile

// H[i][j] = H[j][i] for j < i (i, j < n): the lower half from the upper.
__global__ void mirror_kernel(uint16_t* H, size_t ld, int n) {
    __shared__ uint16_t t[TT][TT + 1];
    const int ti = blockIdx.y, tj = blockIdx.x;  // destination tile (rows ti, columns tj), tj <= ti
    if (tj > ti) return;
    const int x = threadIdx.x;
    for (int y = threadIdx.y; y < TT; y += blockDim.y) {  // source: rows tj*TT + y, columns ti*TT + x
        const int r = tj * TT + y, c = ti * TT + x;
        t[y][x] = (r < n && c < n && c > r) ? H[(size_t)r * ld + c] : 0;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < TT; y += blockDim.y) {
        const int r = ti * TT + y, c = tj * TT + x;
        if (r < n && c < n && c < r) H[(size_t)r * ld + c] = t[x][y];
    }
}

__device__ __forceinline__ int digits(uint32_t v) { return v < 10 ? 1 : v < 100 ? 2 : v < 1000 ? 3 : v < 10000 ? 4 : 5; }

// The value printed at (i, j): layout mask (0 full, 1 lower-tri, 2 upper-tri),
// zero diagonal, then the cap.
__device__ __forceinline__ uint32_t cell(const uint16_t* H, size_t ld, int i, int j, int layout, int cap) {
    uint32_t v = 0;
    if (i != j && !(layout == 1 && j > i) && !(layout == 2 && j < i)) v = H[(size_t)i * ld + j];
    if (cap > 0 && v > (uint32_t)cap) v = (uint32_t)cap;
    return v;
}

__global__ void row_length_kernel(const uint16_t* H, size_t ld, int n, int r0, int rows, int layout, int cap,
                                  const uint64_t* id_off, int seplen, uint64_t* len) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    const int nw = gridDim.x * blockDim.x / 32;
    for (int r = warp; r < rows; r += nw) {
        const int i = r0 + r;
        uint64_t s = 0;
        for (int j = lane; j < n; j += 32) s += (uint64_t)(seplen + digits(cell(H, ld, i, j, layout, cap)));
#pragma unroll
        for (int d = 16; d; d >>= 1) s += __shfl_xor_sync(FULL, s, d);
        if (lane == 0) len[r] = (id_off[i + 1] - id_off[i]) + s + 1;
    }
}

// Exclusive scan of len[0..rows) into off[0..rows], one CTA.
__global__ void scan_kernel(const uint64_t* len, int rows, uint64_t* off) {
    __shared__ uint64_t part[1024];
    const int t = threadIdx.x, T = blockDim.x;
    const int per = (rows + T - 1) / T, a = min(rows, t * per), b = min(rows, a + per);
    uint64_t s = 0;
    for (int r = a; r < b; r++) s += len[r];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        uint64_t acc = 0;
        for (int q = 0; q < T; q++) {
            const uint64_t v = part[q];
            part[q] = acc;
            acc += v;
        }
        off[rows] = acc;
    }
    __syncthreads();
    uint64_t acc = part[t];
    for (int r = a; r < b; r++) {
        off[r] = acc;
        acc += len[r];
    }
}

__global__ void row_write_kernel(const uint16_t* H, size_t ld, int n, int r0, int rows, int layout, int cap,
                                 const char* ids, const uint64_t* id_off, const char* sep, int seplen,
                                 const uint64_t* off, char* out) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    const int nw = gridDim.x * blockDim.x / 32;
    for (int r = warp; r < rows; r += nw) {
        const int i = r0 + r;
        char* p = out + off[r];
        const uint64_t il = id_off[i + 1] - id_off[i];
        for (uint64_t c = lane; c < il; c += 32) p[c] = ids[id_off[i] + c];
        uint64_t pos = il;
        for (int j0 = 0; j0 < n; j0 += 32) {
            const int j = j0 + lane;
            uint32_t v = 0;
            int w = 0;
            if (j < n) {
                v = cell(H, ld, i, j, layout, cap);
                w = seplen + digits(v);
            }
            int x = w;  // inclusive scan of the field widths
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int t = __shfl_up_sync(FULL, x, d);
                if (lane >= d) x += t;
            }
            if (j < n) {
                char* q = p + pos + (x - w);
                for (int c = 0; c < seplen; c++) q[c] = sep[c];
                q += seplen;
                for (int c = w - seplen - 1; c >= 0; c--) {
                    q[c] = (char)('0' + v % 10);
                    v /= 10;
                }
            }
            pos += (uint64_t)__shfl_sync(FULL, x, 31);
        }
        if (lane == 0) p[pos] = '\n';
    }
}

// Page-locked text buffers cost far more to allocate than to fill, so the pair
// of the previous call is kept for the next (one pair per process; a call that
// finds it in use allocates its own).
std::mutex g_text_mu;
char* g_text[2] = {nullptr, nullptr};
size_t g_text_bytes = 0;
bool g_text_busy = false;

bool text_acquire(size_t bytes, char* out[2]) {
    std::lock_guard<std::mutex> lk(g_text_mu);
    if (g_text_busy) return false;
    if (g_text_bytes < bytes) {
        for (int b = 0; b < 2; b++) {
            if (g_text[b]) cudaFreeHost(g_text[b]);
            g_text[b] = nullptr;
        }
        g_text_bytes = 0;
        for (int b = 0; b < 2; b++)
            if (cudaMallocHost(&g_text[b], bytes) != cudaSuccess) return false;
        g_text_bytes = bytes;
    }
    g_text_busy = true;
    out[0] = g_text[0];
    out[1] = g_text[1];
    return true;
}

void text_release() {
    std::lock_guard<std::mutex> lk(g_text_mu);
    g_text_busy = false;
}

}  // namespace

cudaError_t launch_mirror(uint16_t* H, size_t ld, int n, cudaStream_t st) {
    if (n < 2) return cudaSuccess;
    const int nt = (n + TT - 1) / TT;
    mirror_kernel<<<dim3(nt, nt), dim3(TT, 8), 0, st>>>(H, ld, n);
    return cudaGetLastError();
}

}  // namespace tch

using namespace tch;

extern "C" int tch_solver_write_tsv(tch_solver* s, const char* const* ids, const char* osep, const char* index_name,
                                    int layout, int cap, int block_rows, tch_text_cb cb, void* ctx, char* err,
                                    int errlen) {
    Err e{err, errlen};
    tch_info info;
    uint16_t* H = nullptr;
    char *d_ids = nullptr, *d_sep = nullptr, *d_text[2] = {nullptr, nullptr}, *h_text[2] = {nullptr, nullptr};
    uint64_t *d_idoff = nullptr, *d_len = nullptr, *d_off[2] = {nullptr, nullptr};
    cudaStream_t st = nullptr;
    cudaEvent_t done[2] = {nullptr, nullptr};
    int dev = 0, sms = 0, rc = 1;
    std::vector<uint64_t> idoff;
    std::string head;
    size_t cap_bytes = 0;
    int prev = -1;
    bool pooled = false;
    uint64_t prev_len = 0, lens[2] = {0, 0};
    if (!s || !ids || !osep || !index_name || !cb) return e.set("null argument");
    if (layout < 0 || layout > 2) return e.set("layout must be 0 (full), 1 (lower-tri) or 2 (upper-tri)");
    if (tch_solver_info(s, &info)) return e.set("bad solver");
    const int n = info.n;
    const int seplen = (int)strlen(osep);
    if (seplen < 1 || seplen > 16) return e.set("output separator must be 1-16 bytes");
    if (block_rows <= 0) block_rows = 2048;
    block_rows = std::min(block_rows, std::max(n, 1));
    // header (host)
    head = index_name;
    idoff.assign((size_t)n + 1, 0);
    for (int i = 0; i < n; i++) {
        head += osep;
        head += ids[i];
        idoff[i + 1] = idoff[i] + strlen(ids[i]);
    }
    head += '\n';
    cb(ctx, head.data(), head.size());
    if (n == 0) return 0;
    const size_t ld = up((size_t)n, 8);
    TCH_CK(e, cudaGetDevice(&dev));
    TCH_CK(e, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TCH_CK(e, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    TCH_CK(e, cudaMalloc(&H, (size_t)n * ld * 2));
    if (n > 1) {
        if (tch_solver_stripe(s, 0, n, H, ld, st, err, errlen)) goto fail;
        TCH_CK(e, cudaStreamSynchronize(st));
        if (tch_solver_check(s, err, errlen)) goto fail;
        if (layout != 2) TCH_CK(e, launch_mirror(H, ld, n, st));
    }
    {
        std::string all_ids;
        for (int i = 0; i < n; i++) all_ids += ids[i];
        TCH_CK(e, cudaMalloc(&d_ids, std::max<size_t>(all_ids.size(), 1)));
        TCH_CK(e, cudaMalloc(&d_idoff, ((size_t)n + 1) * 8));
        TCH_CK(e, cudaMalloc(&d_sep, 16));
        if (!all_ids.empty())
            TCH_CK(e, cudaMemcpy(d_ids, all_ids.data(), all_ids.size(), cudaMemcpyHostToDevice));
        TCH_CK(e, cudaMemcpy(d_idoff, idoff.data(), ((size_t)n + 1) * 8, cudaMemcpyHostToDevice));
        TCH_CK(e, cudaMemcpy(d_sep, osep, seplen, cudaMemcpyHostToDevice));
    }
    // text buffers: the longest block of rows (longest ids x widest values)
    {
        size_t maxid = 0;
        for (int i = 0; i < n; i++) maxid = std::max<size_t>(maxid, idoff[i + 1] - idoff[i]);
        cap_bytes = (size_t)block_rows * (maxid + (size_t)n * (seplen + 5) + 1);
    }
    TCH_CK(e, cudaMalloc(&d_len, (size_t)block_rows * 8));
    pooled = text_acquire(cap_bytes, h_text);
    for (int b = 0; b < 2; b++) {
        TCH_CK(e, cudaMalloc(&d_off[b], ((size_t)block_rows + 1) * 8));
        TCH_CK(e, cudaMalloc(&d_text[b], cap_bytes));
        if (!pooled) TCH_CK(e, cudaMallocHost(&h_text[b], cap_bytes));
        TCH_CK(e, cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming));
    }
    for (int r0 = 0;; r0 += block_rows) {
        if (r0 < n) {
            const int rows = std::min(block_rows, n - r0), b = (r0 / block_rows) & 1;
            const int grid = std::max(1, std::min(sms * 8, (rows * 32 + 255) / 256));
            row_length_kernel<<<grid, 256, 0, st>>>(H, ld, n, r0, rows, layout, cap, d_idoff, seplen, d_len);
            scan_kernel<<<1, 1024, 0, st>>>(d_len, rows, d_off[b]);
            row_write_kernel<<<grid, 256, 0, st>>>(H, ld, n, r0, rows, layout, cap, d_ids, d_idoff, d_sep, seplen,
                                                   d_off[b], d_text[b]);
            TCH_CK(e, cudaGetLastError());
            TCH_CK(e, cudaMemcpyAsync(&lens[b], d_off[b] + rows, 8, cudaMemcpyDeviceToHost, st));
            TCH_CK(e, cudaStreamSynchronize(st));  // the block's length sizes its copy
            TCH_CK(e, cudaMemcpyAsync(h_text[b], d_text[b], lens[b], cudaMemcpyDeviceToHost, st));
            TCH_CK(e, cudaEventRecord(done[b], st));
        }
        if (prev >= 0) {  // hand the previous block over while this one is copied
            const int b = (prev / block_rows) & 1;
            TCH_CK(e, cudaEventSynchronize(done[b]));
            prev_len = lens[b];
            cb(ctx, h_text[b], prev_len);
        }
        if (r0 >= n) break;
        prev = r0;
    }
    rc = 0;
fail:
    if (st) cudaStreamSynchronize(st);
    cudaFree(H);
    cudaFree(d_ids);
    cudaFree(d_sep);
    cudaFree(d_idoff);
    cudaFree(d_len);
    for (int b = 0; b < 2; b++) {
        cudaFree(d_off[b]);
        cudaFree(d_text[b]);
        if (h_text[b] && !pooled) cudaFreeHost(h_text[b]);
        if (done[b]) cudaEventDestroy(done[b]);
    }
    if (st) cudaStreamDestroy(st);
    if (pooled) text_release();
    return rc;
}
