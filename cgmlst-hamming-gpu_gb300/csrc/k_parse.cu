// Device-side parse of the cgMLST allele table (tensorcore/rs/src/main.rs:286-311
// for the load, 95-113 for a cell, 313-348 for the completeness filters): the
// whole text goes to the GPU once and the calls matrix is built there, where the
// device encoder reads it; only the sample ids' offsets and a few counts come
// back.
//
//   lines         the text's lines as Rust's str::lines gives them: split at
//                 '\n', one '\r' before it dropped (a last line without '\n'
//                 keeps its '\r'); newlines counted per 64 KB chunk, their
//                 positions written in order after a scan of the counts
//   rows          line 0 is the header; every later non-empty line is a row
//                 (a flag per line, a scan, the rows' bounds in order)
//   cells         one thread per row: the sample id up to the first separator,
//                 then every cell read by parse_allele (trim of Unicode white
//                 space, one leading "INF-" dropped unless skip_repl, the
//                 missing token or an empty cell -> 0, all ASCII digits -> the
//                 u64 value, anything else -> 0); a value above 2^64 - 1 is an
//                 error; cells past L are dropped, missing ones are 0.  A cell of
//                 1-19 digits running up to the separator is read in the pass
//                 that finds its end (nothing else can apply to it when the
//                 separator is not a digit and the missing token is not all
//                 digits)
//   filters       non-missing calls per locus (column counts) and per sample
//                 (row counts); kept loci / samples gathered into a new matrix
//
// The text is UTF-8 checked by the caller, as the reference's read into a
// String does.

#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "tch_internal.cuh"

using namespace tch;

struct tch_tsv {
    int device = 0;
    int n = 0, L = 0;
    uint64_t* calls = nullptr;          // device, n x L
    std::vector<uint64_t> id_b, id_e;   // sample id of row i: text[id_b[i], id_e[i])
};

namespace tch {
namespace {

constexpr size_t kChunk = 1 << 16;  // bytes per newline-counting block
constexpr int kChunkThreads = 256;
constexpr int kMaxMissing = 64;

struct CellRules {
    char sep;
    int skip_repl;
    int fast;  // separator not a digit, missing token not all digits
    int mlen;
    char missing[kMaxMissing];
};

// Newline mask of the 16 bytes at text[p] (aligned; the text has 16 bytes of
// slack past its end): bit j set when text[p + j] == '\n' and p + j < end.
__device__ __forceinline__ uint32_t newline_mask(const char* text, size_t p, size_t end) {
    const uint4 v = *reinterpret_cast<const uint4*>(text + p);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    uint32_t m = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const uint32_t eq = __vcmpeq4(w[q], 0x0A0A0A0Au);  // 0xFF in every byte equal to '\n'
#pragma unroll
        for (int j = 0; j < 4; j++) m |= ((eq >> (8 * j)) & 1u) << (4 * q + j);
    }
    const size_t left = end - p;
    return left >= 16 ? m : m & ((1u << left) - 1u);
}

// Newlines of chunk blockIdx.x: each thread takes a contiguous, 16-byte
// aligned slice; pass 0 writes the chunk's count, pass 1 the positions in order
// from base[chunk].
__global__ void newlines_kernel(const char* __restrict__ text, size_t len, int pass, uint32_t* counts,
                                const uint64_t* __restrict__ base, uint64_t* nl) {
    __shared__ uint32_t scan[kChunkThreads];
    const size_t c0 = (size_t)blockIdx.x * kChunk, c1 = c0 + kChunk < len ? c0 + kChunk : len;
    const size_t slice = kChunk / kChunkThreads;
    const size_t s0a = c0 + threadIdx.x * slice;
    const size_t s0 = s0a < c1 ? s0a : c1, s1 = s0 + slice < c1 ? s0 + slice : c1;
    uint32_t cnt = 0;
    for (size_t p = s0; p < s1; p += 16) cnt += __popc(newline_mask(text, p, s1));
    scan[threadIdx.x] = cnt;
    __syncthreads();
    for (int d = 1; d < kChunkThreads; d <<= 1) {  // inclusive scan
        const uint32_t v = threadIdx.x >= d ? scan[threadIdx.x - d] : 0u;
        __syncthreads();
        scan[threadIdx.x] += v;
        __syncthreads();
    }
    if (pass == 0) {
        if (threadIdx.x == kChunkThreads - 1) counts[blockIdx.x] = scan[kChunkThreads - 1];
        return;
    }
    uint64_t q = base[blockIdx.x] + scan[threadIdx.x] - cnt;
    for (size_t p = s0; p < s1; p += 16) {
        uint32_t m = newline_mask(text, p, s1);
        while (m) {
            const int j = __ffs(m) - 1;
            nl[q++] = p + j;
            m &= m - 1;
        }
    }
}

// Line k's bounds (str::lines) from the newline positions.
__device__ __forceinline__ void line_bounds(const char* text, size_t len, const uint64_t* nl, uint64_t nnl, uint64_t k,
                                            uint64_t* b, uint64_t* e) {
    *b = k == 0 ? 0 : nl[k - 1] + 1;
    if (k < nnl) {
        uint64_t x = nl[k];
        if (x > *b && text[x - 1] == '\r') x--;
        *e = x;
    } else {
        *e = len;  // the last line, without '\n'
    }
}

// Rows: the non-empty lines after the header.  Pass 0 counts them per block of
// lines, pass 1 writes their bounds in order from base[block].
__global__ void rows_kernel(const char* __restrict__ text, size_t len, const uint64_t* __restrict__ nl, uint64_t nnl,
                            uint64_t nlines, int pass, uint32_t* counts, const uint64_t* __restrict__ base,
                            uint64_t* rb, uint64_t* re) {
    __shared__ uint32_t scan[256];
    const uint64_t k = 1 + (uint64_t)blockIdx.x * 256 + threadIdx.x;
    uint64_t b = 0, e = 0;
    uint32_t keep = 0;
    if (k < nlines) {
        line_bounds(text, len, nl, nnl, k, &b, &e);
        keep = e > b;
    }
    scan[threadIdx.x] = keep;
    __syncthreads();
    for (int d = 1; d < 256; d <<= 1) {
        const uint32_t v = threadIdx.x >= d ? scan[threadIdx.x - d] : 0u;
        __syncthreads();
        scan[threadIdx.x] += v;
        __syncthreads();
    }
    if (pass == 0) {
        if (threadIdx.x == 255) counts[blockIdx.x] = scan[255];
        return;
    }
    if (keep) {
        const uint64_t r = base[blockIdx.x] + scan[threadIdx.x] - 1;
        rb[r] = b;
        re[r] = e;
    }
}

// Decodes the UTF-8 code point at s[i] (validated input).
__device__ __forceinline__ uint32_t cp_at(const char* s, uint64_t i, uint32_t* n) {
    const uint32_t c = (unsigned char)s[i];
    if (c < 0x80) { *n = 1; return c; }
    if ((c >> 5) == 6) { *n = 2; return ((c & 0x1F) << 6) | ((unsigned char)s[i + 1] & 0x3F); }
    if ((c >> 4) == 14) {
        *n = 3;
        return ((c & 0x0F) << 12) | (((unsigned char)s[i + 1] & 0x3F) << 6) | ((unsigned char)s[i + 2] & 0x3F);
    }
    *n = 4;
    return ((c & 0x07) << 18) | (((unsigned char)s[i + 1] & 0x3F) << 12) | (((unsigned char)s[i + 2] & 0x3F) << 6) |
           ((unsigned char)s[i + 3] & 0x3F);
}

// Unicode White_Space: what Rust's str::trim removes.
__device__ __forceinline__ bool is_ws(uint32_t c) {
    return (c >= 0x09 && c <= 0x0D) || c == 0x20 || c == 0x85 || c == 0xA0 || c == 0x1680 ||
           (c >= 0x2000 && c <= 0x200A) || c == 0x2028 || c == 0x2029 || c == 0x202F || c == 0x205F || c == 0x3000;
}

// parse_allele on text[b, e) (main.rs:98-113); false on a u64 overflow.
__device__ bool parse_cell(const char* s, uint64_t b, uint64_t e, const CellRules& cr, uint64_t* out) {
    while (b < e) {  // trim
        uint32_t n;
        if (!is_ws(cp_at(s, b, &n))) break;
        b += n;
    }
    while (e > b) {
        uint64_t p = e - 1;
        while (p > b && ((unsigned char)s[p] & 0xC0) == 0x80) p--;
        uint32_t n;
        if (!is_ws(cp_at(s, p, &n))) break;
        e = p;
    }
    if (!cr.skip_repl && e - b >= 4 && s[b] == 'I' && s[b + 1] == 'N' && s[b + 2] == 'F' && s[b + 3] == '-') b += 4;
    *out = 0;
    if (b == e) return true;
    if (e - b == (uint64_t)cr.mlen) {
        bool same = true;
        for (int q = 0; q < cr.mlen && same; q++) same = s[b + q] == cr.missing[q];
        if (same) return true;
    }
    for (uint64_t p = b; p < e; p++)
        if (s[p] < '0' || s[p] > '9') return true;
    uint64_t v = 0;
    for (uint64_t p = b; p < e; p++) {
        const uint64_t d = (uint64_t)(s[p] - '0');
        if (v > (~0ull - d) / 10) return false;
        v = v * 10 + d;
    }
    *out = v;
    return true;
}

// One thread per row: the id's end, then every cell into calls[i * L ..).
// A cell that overflows u64 reads 0 and puts its row into *bad (the least).
__global__ void cells_kernel(const char* __restrict__ text, const uint64_t* __restrict__ rb,
                             const uint64_t* __restrict__ re, int n, int L, const CellRules cr, uint64_t* calls,
                             uint64_t* id_end, int* bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t e = re[i];
    uint64_t f = rb[i];
    while (f < e && text[f] != cr.sep) f++;
    id_end[i] = f;
    uint64_t* out = calls + (size_t)i * L;
    int k = 0;
    while (f < e) {  // f at the separator before a cell
        const uint64_t cb = f + 1;
        uint64_t q = cb, v = 0;
        if (cr.fast)
            while (q < e && q - cb < 19) {
                const unsigned d = (unsigned)(unsigned char)text[q] - (unsigned)'0';
                if (d > 9) break;
                v = v * 10 + d;
                q++;
            }
        uint64_t ce;
        if (cr.fast && q > cb && (q == e || text[q] == cr.sep)) {
            ce = q;
        } else {
            ce = q;
            while (ce < e && text[ce] != cr.sep) ce++;
            if (!parse_cell(text, cb, ce, cr, &v)) {
                atomicMin(bad, i);
                v = 0;
            }
        }
        if (k < L) out[k] = v;
        k++;
        f = ce;
    }
    for (; k < L; k++) out[k] = 0;
}

// Non-missing calls per locus over a block of rows (one thread per locus).
__global__ void locus_counts_kernel(const uint64_t* __restrict__ calls, int n, int L, int rows_per_block,
                                    unsigned long long* counts) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    const int i0 = blockIdx.y * rows_per_block, i1 = min(n, i0 + rows_per_block);
    unsigned long long c = 0;
    for (int i = i0; i < i1; i++) c += calls[(size_t)i * L + k] != 0;
    if (c) atomicAdd(counts + k, c);
}

// Non-missing calls per row (one warp per row).
__global__ void sample_counts_kernel(const uint64_t* __restrict__ calls, int n, int L, uint32_t* counts) {
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32), lane = threadIdx.x & 31;
    if (w >= n) return;
    uint32_t c = 0;
    for (int k = lane; k < L; k += 32) c += calls[(size_t)w * L + k] != 0;
    for (int d = 16; d; d >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, d);
    if (lane == 0) counts[w] = c;
}

// out[r][d] = in[rows[r]][cols[d]] (rows / cols null = identity).
__global__ void gather_kernel(const uint64_t* __restrict__ in, int L, const int* __restrict__ rows,
                              const int* __restrict__ cols, int n2, int L2, uint64_t* out) {
    const size_t total = (size_t)n2 * L2;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / L2), d = (int)(t % L2);
        const int i = rows ? rows[r] : r, k = cols ? cols[d] : d;
        out[t] = in[(size_t)i * L + k];
    }
}

// Exclusive scan of per-block counts on the host (a few thousand entries).
std::vector<uint64_t> host_scan(const std::vector<uint32_t>& c, uint64_t* total) {
    std::vector<uint64_t> b(c.size());
    uint64_t acc = 0;
    for (size_t k = 0; k < c.size(); k++) b[k] = acc, acc += c[k];
    *total = acc;
    return b;
}

// Host copies of the trim for the error message.
uint32_t host_cp_at(const char* s, uint64_t i, uint32_t* n) {
    const uint32_t c = (unsigned char)s[i];
    if (c < 0x80) { *n = 1; return c; }
    if ((c >> 5) == 6) { *n = 2; return ((c & 0x1F) << 6) | ((unsigned char)s[i + 1] & 0x3F); }
    if ((c >> 4) == 14) {
        *n = 3;
        return ((c & 0x0F) << 12) | (((unsigned char)s[i + 1] & 0x3F) << 6) | ((unsigned char)s[i + 2] & 0x3F);
    }
    *n = 4;
    return ((c & 0x07) << 18) | (((unsigned char)s[i + 1] & 0x3F) << 12) | (((unsigned char)s[i + 2] & 0x3F) << 6) |
           ((unsigned char)s[i + 3] & 0x3F);
}

bool host_is_ws(uint32_t c) {
    return (c >= 0x09 && c <= 0x0D) || c == 0x20 || c == 0x85 || c == 0xA0 || c == 0x1680 ||
           (c >= 0x2000 && c <= 0x200A) || c == 0x2028 || c == 0x2029 || c == 0x202F || c == 0x205F || c == 0x3000;
}

// The first cell of row text[b, e) whose id overflows u64, trimmed as the
// reference prints it (main.rs:301).
std::string bad_cell(const char* text, uint64_t b, uint64_t e, char sep, bool skip_repl) {
    uint64_t f = b;
    while (f < e && text[f] != sep) f++;
    while (f < e) {
        uint64_t cb = f + 1, ce = cb;
        while (ce < e && text[ce] != sep) ce++;
        f = ce;
        while (cb < ce) {
            uint32_t n;
            if (!host_is_ws(host_cp_at(text, cb, &n))) break;
            cb += n;
        }
        while (ce > cb) {
            uint64_t p = ce - 1;
            while (p > cb && ((unsigned char)text[p] & 0xC0) == 0x80) p--;
            uint32_t n;
            if (!host_is_ws(host_cp_at(text, p, &n))) break;
            ce = p;
        }
        uint64_t d = cb;
        if (!skip_repl && ce - d >= 4 && memcmp(text + d, "INF-", 4) == 0) d += 4;
        if (ce - d < 20) continue;  // 19 digits never overflow
        bool digits = true;
        for (uint64_t p = d; p < ce && digits; p++) digits = text[p] >= '0' && text[p] <= '9';
        if (!digits) continue;
        unsigned long long v = 0;
        for (uint64_t p = d; p < ce; p++) {
            const unsigned long long q = (unsigned long long)(text[p] - '0');
            if (v > (~0ull - q) / 10) return std::string(text + cb, ce - cb);
            v = v * 10 + q;
        }
    }
    return std::string();
}

}  // namespace
}  // namespace tch

extern "C" {

int tch_tsv_parse(int device, const char* text, size_t len, char sep, int skip_repl, const char* missing,
                  tch_tsv** out, char* err, int errlen) {
    Err e{err, errlen};
    char* d_text = nullptr;
    uint32_t* d_counts = nullptr;
    uint64_t *d_base = nullptr, *d_nl = nullptr, *d_rb = nullptr, *d_re = nullptr, *d_id = nullptr;
    int* d_bad = nullptr;
    tch_tsv* t = nullptr;
    std::vector<uint64_t> rb_h;
    if (!out || (!text && len)) return e.set("null argument");
    *out = nullptr;
    CellRules cr{};
    cr.sep = sep;
    cr.skip_repl = skip_repl ? 1 : 0;
    const std::string miss = missing ? missing : "";
    if (miss.size() > (size_t)kMaxMissing) return e.set("missing token longer than %d bytes", kMaxMissing);
    cr.mlen = (int)miss.size();
    memcpy(cr.missing, miss.data(), miss.size());
    bool digits = !miss.empty();
    for (char c : miss) digits = digits && c >= '0' && c <= '9';
    cr.fast = !(sep >= '0' && sep <= '9') && !digits;
    if (len == 0) return e.set("empty input");
    TCH_CK(e, cudaSetDevice(device));
    {
        // ---- text to the device (16 bytes of slack past the end)
        TCH_CK(e, cudaMalloc(&d_text, len + 16));
        TCH_CK(e, cudaMemcpy(d_text, text, len, cudaMemcpyHostToDevice));
        TCH_CK(e, cudaMemset(d_text + len, 0, 16));
        // ---- newlines
        const size_t chunks = (len + kChunk - 1) / kChunk;
        TCH_CK(e, cudaMalloc(&d_counts, std::max<size_t>(chunks, (len + 255) / 256 + 1) * 4));
        newlines_kernel<<<(unsigned)chunks, kChunkThreads>>>(d_text, len, 0, d_counts, nullptr, nullptr);
        TCH_CK(e, cudaGetLastError());
        std::vector<uint32_t> cnt(chunks);
        TCH_CK(e, cudaMemcpy(cnt.data(), d_counts, chunks * 4, cudaMemcpyDeviceToHost));
        uint64_t nnl = 0;
        std::vector<uint64_t> base = host_scan(cnt, &nnl);
        TCH_CK(e, cudaMalloc(&d_base, std::max<size_t>(chunks, 1) * 8));
        TCH_CK(e, cudaMemcpy(d_base, base.data(), chunks * 8, cudaMemcpyHostToDevice));
        TCH_CK(e, cudaMalloc(&d_nl, std::max<uint64_t>(nnl, 1) * 8));
        newlines_kernel<<<(unsigned)chunks, kChunkThreads>>>(d_text, len, 1, nullptr, d_base, d_nl);
        TCH_CK(e, cudaGetLastError());
        // str::lines: a last line without '\n' when text follows the last newline
        uint64_t last_nl = 0;
        if (nnl) TCH_CK(e, cudaMemcpy(&last_nl, d_nl + nnl - 1, 8, cudaMemcpyDeviceToHost));
        const uint64_t nlines = nnl + ((nnl == 0 || last_nl + 1 < len) ? 1 : 0);
        // ---- rows: the non-empty lines after the header
        const uint64_t rblocks = nlines > 1 ? (nlines - 1 + 255) / 256 : 0;
        uint64_t n = 0;
        std::vector<uint32_t> rc(rblocks);
        if (rblocks) {
            TCH_CK(e, cudaFree(d_counts));
            d_counts = nullptr;
            TCH_CK(e, cudaMalloc(&d_counts, rblocks * 4));
            rows_kernel<<<(unsigned)rblocks, 256>>>(d_text, len, d_nl, nnl, nlines, 0, d_counts, nullptr, nullptr,
                                                    nullptr);
            TCH_CK(e, cudaGetLastError());
            TCH_CK(e, cudaMemcpy(rc.data(), d_counts, rblocks * 4, cudaMemcpyDeviceToHost));
        }
        std::vector<uint64_t> rbase = host_scan(rc, &n);
        if (n > (uint64_t)INT32_MAX) {
            e.set("more than 2^31 - 1 samples");
            goto fail;
        }
        // the header's field count (line 0)
        uint64_t h_end = nnl ? 0 : len;
        if (nnl) TCH_CK(e, cudaMemcpy(&h_end, d_nl, 8, cudaMemcpyDeviceToHost));
        if (nnl && h_end > 0 && text[h_end - 1] == '\r') h_end--;
        uint64_t L = 1;
        for (uint64_t p = 0; p < h_end; p++) L += text[p] == sep;
        L -= 1;
        if (L > (uint64_t)INT32_MAX) {
            e.set("too many loci");
            goto fail;
        }
        t = new tch_tsv();
        t->device = device;
        t->n = (int)n;
        t->L = (int)L;
        TCH_CK(e, cudaMalloc(&t->calls, std::max<uint64_t>(n * L, 1) * 8));
        TCH_CK(e, cudaMalloc(&d_rb, std::max<uint64_t>(n, 1) * 8));
        TCH_CK(e, cudaMalloc(&d_re, std::max<uint64_t>(n, 1) * 8));
        TCH_CK(e, cudaMalloc(&d_id, std::max<uint64_t>(n, 1) * 8));
        TCH_CK(e, cudaMalloc(&d_bad, 4));
        const int none = INT32_MAX;
        TCH_CK(e, cudaMemcpy(d_bad, &none, 4, cudaMemcpyHostToDevice));
        if (rblocks) {
            TCH_CK(e, cudaFree(d_base));
            d_base = nullptr;
            TCH_CK(e, cudaMalloc(&d_base, rblocks * 8));
            TCH_CK(e, cudaMemcpy(d_base, rbase.data(), rblocks * 8, cudaMemcpyHostToDevice));
            rows_kernel<<<(unsigned)rblocks, 256>>>(d_text, len, d_nl, nnl, nlines, 1, nullptr, d_base, d_rb, d_re);
            TCH_CK(e, cudaGetLastError());
        }
        // ---- cells
        if (n) {
            cells_kernel<<<(unsigned)((n + 127) / 128), 128>>>(d_text, d_rb, d_re, (int)n, (int)L, cr, t->calls, d_id,
                                                               d_bad);
            TCH_CK(e, cudaGetLastError());
        }
        int bad = none;
        TCH_CK(e, cudaMemcpy(&bad, d_bad, 4, cudaMemcpyDeviceToHost));
        t->id_b.resize(n);
        t->id_e.resize(n);
        rb_h.resize(n);
        if (n) {
            TCH_CK(e, cudaMemcpy(t->id_b.data(), d_rb, n * 8, cudaMemcpyDeviceToHost));
            TCH_CK(e, cudaMemcpy(t->id_e.data(), d_id, n * 8, cudaMemcpyDeviceToHost));
        }
        if (bad != none) {
            uint64_t re_bad = 0;
            TCH_CK(e, cudaMemcpy(&re_bad, d_re + bad, 8, cudaMemcpyDeviceToHost));
            const std::string id(text + t->id_b[bad], t->id_e[bad] - t->id_b[bad]);
            e.set("sample %s: allele '%s' too large", id.c_str(),
                  bad_cell(text, t->id_b[bad], re_bad, sep, skip_repl != 0).c_str());
            goto fail;
        }
    }
    cudaFree(d_text);
    cudaFree(d_counts);
    cudaFree(d_base);
    cudaFree(d_nl);
    cudaFree(d_rb);
    cudaFree(d_re);
    cudaFree(d_id);
    cudaFree(d_bad);
    *out = t;
    return 0;
fail:
    cudaFree(d_text);
    cudaFree(d_counts);
    cudaFree(d_base);
    cudaFree(d_nl);
    cudaFree(d_rb);
    cudaFree(d_re);
    cudaFree(d_id);
    cudaFree(d_bad);
    tch_tsv_free(t);
    return 1;
}

int tch_tsv_shape(const tch_tsv* t, int* n, int* L) {
    if (!t) return 1;
    if (n) *n = t->n;
    if (L) *L = t->L;
    return 0;
}

int tch_tsv_ids(const tch_tsv* t, size_t* begin, size_t* end) {
    if (!t) return 1;
    for (int i = 0; i < t->n; i++) {
        if (begin) begin[i] = (size_t)t->id_b[i];
        if (end) end[i] = (size_t)t->id_e[i];
    }
    return 0;
}

int tch_tsv_filter(tch_tsv* t, double locus_pct, double sample_pct, char* err, int errlen) {
    Err e{err, errlen};
    unsigned long long* d_lc = nullptr;
    uint32_t* d_sc = nullptr;
    int *d_rows = nullptr, *d_cols = nullptr;
    uint64_t* d_new = nullptr;
    if (!t) return e.set("null table");
    TCH_CK(e, cudaSetDevice(t->device));
    if (locus_pct >= 0 && t->L > 0) {  // main.rs:313-330 (no samples: 0 / 0 keeps no locus)
        const int n = t->n, L = t->L, rpb = 1024;
        TCH_CK(e, cudaMalloc(&d_lc, (size_t)L * 8));
        TCH_CK(e, cudaMemset(d_lc, 0, (size_t)L * 8));
        if (n) {
            const dim3 grid((unsigned)((L + 255) / 256), (unsigned)((n + rpb - 1) / rpb));
            locus_counts_kernel<<<grid, 256>>>(t->calls, n, L, rpb, d_lc);
            TCH_CK(e, cudaGetLastError());
        }
        std::vector<unsigned long long> lc(L);
        TCH_CK(e, cudaMemcpy(lc.data(), d_lc, (size_t)L * 8, cudaMemcpyDeviceToHost));
        std::vector<int> keep;
        for (int k = 0; k < L; k++)
            if (((double)lc[k] / (double)n) * 100.0 >= locus_pct) keep.push_back(k);
        if ((int)keep.size() != L) {
            const int L2 = (int)keep.size();
            TCH_CK(e, cudaMalloc(&d_cols, std::max<size_t>(keep.size(), 1) * 4));
            if (L2) TCH_CK(e, cudaMemcpy(d_cols, keep.data(), keep.size() * 4, cudaMemcpyHostToDevice));
            TCH_CK(e, cudaMalloc(&d_new, std::max<size_t>((size_t)n * L2, 1) * 8));
            if ((size_t)n * L2)
                gather_kernel<<<(unsigned)std::min<size_t>(((size_t)n * L2 + 255) / 256, 65535), 256>>>(
                    t->calls, L, nullptr, d_cols, n, L2, d_new);
            TCH_CK(e, cudaGetLastError());
            TCH_CK(e, cudaDeviceSynchronize());
            cudaFree(t->calls);
            t->calls = d_new;
            d_new = nullptr;
            t->L = L2;
        }
    }
    if (sample_pct >= 0 && t->n > 0) {  // main.rs:331-345
        const int n = t->n, L = t->L;
        std::vector<uint32_t> sc(n, 0);
        if (L > 0) {
            TCH_CK(e, cudaMalloc(&d_sc, (size_t)n * 4));
            sample_counts_kernel<<<(unsigned)(((size_t)n * 32 + 255) / 256), 256>>>(t->calls, n, L, d_sc);
            TCH_CK(e, cudaGetLastError());
            TCH_CK(e, cudaMemcpy(sc.data(), d_sc, (size_t)n * 4, cudaMemcpyDeviceToHost));
        }
        std::vector<int> keep;
        for (int i = 0; i < n; i++)
            if (((double)sc[i] / (double)L) * 100.0 >= sample_pct) keep.push_back(i);
        if ((int)keep.size() != n) {
            const int n2 = (int)keep.size();
            TCH_CK(e, cudaMalloc(&d_rows, std::max<size_t>(keep.size(), 1) * 4));
            if (n2) TCH_CK(e, cudaMemcpy(d_rows, keep.data(), keep.size() * 4, cudaMemcpyHostToDevice));
            TCH_CK(e, cudaMalloc(&d_new, std::max<size_t>((size_t)n2 * L, 1) * 8));
            if ((size_t)n2 * L)
                gather_kernel<<<(unsigned)std::min<size_t>(((size_t)n2 * L + 255) / 256, 65535), 256>>>(
                    t->calls, L, d_rows, nullptr, n2, L, d_new);
            TCH_CK(e, cudaGetLastError());
            TCH_CK(e, cudaDeviceSynchronize());
            cudaFree(t->calls);
            t->calls = d_new;
            d_new = nullptr;
            std::vector<uint64_t> b2(n2), e2(n2);
            for (int r = 0; r < n2; r++) b2[r] = t->id_b[keep[r]], e2[r] = t->id_e[keep[r]];
            t->id_b.swap(b2);
            t->id_e.swap(e2);
            t->n = n2;
        }
    }
    cudaFree(d_lc);
    cudaFree(d_sc);
    cudaFree(d_rows);
    cudaFree(d_cols);
    return 0;
fail:
    cudaFree(d_lc);
    cudaFree(d_sc);
    cudaFree(d_rows);
    cudaFree(d_cols);
    cudaFree(d_new);
    return 1;
}

int tch_tsv_calls(const tch_tsv* t, uint64_t* calls) {
    if (!t || (!calls && (size_t)t->n * t->L)) return 1;
    if (cudaSetDevice(t->device) != cudaSuccess) return 1;
    if ((size_t)t->n * t->L &&
        cudaMemcpy(calls, t->calls, (size_t)t->n * t->L * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return 1;
    return 0;
}

int tch_solver_from_tsv(const tch_tsv* t, int tau, tch_solver** out, char* err, int errlen) {
    Err e{err, errlen};
    if (!t || !out) return e.set("null argument");
    if (t->L < 1) return e.set("no loci");
    const char* v = getenv("TCH_VERBOSE");
    return solver_from_device_calls(t->device, t->n, t->L, t->calls, tau, v && v[0] == '1', out, e);
}

void tch_tsv_free(tch_tsv* t) {
    if (!t) return;
    cudaSetDevice(t->device);
    cudaFree(t->calls);
    delete t;
}

}  // extern "C"
