// libtch: the C ABI, the solver object and the double-buffered stripe pipeline.
//
// tch_run keeps the reference's contract (tensorcore/rs/cuda/tch.cu:68-170):
// same arguments, same stripe order and callback timing, same error
// convention, the same host fallback for rare pairs that do not fit in device
// memory (tch.cu:105, 140-144).  Inside it, the work is organised GB300-first:
//
//   * operands are uploaded once and, for the tensor-core kernel, expanded
//     from bits to packed fp4 rows on the device (k_expand.cu);
//   * each stripe is a rare-count pass (the stripe's pair lists counted into a
//     u16 block) and ONE fused tile pass that writes u16 distances directly:
//     P Pt - O Ot accumulates on the tensor pipe (or CUDA cores), the rare
//     counts are subtracted inside the tile, and the int32 matrix the
//     reference materialises between its GEMMs, sub_rare and pack_u16 never
//     exists (3 passes over an int32 stripe -> 0);
//   * the u16 stripe is copied to pinned host memory on the stripe's own
//     stream while the other stream computes the next stripe.

#include <errno.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

#include "tch_internal.cuh"

namespace tch {

int Err::set(const char* fmt, ...) {
    if (buf && len > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, (size_t)len, fmt, ap);
        va_end(ap);
    }
    return 1;
}

static int g_kernel = -1;  // process default, resolved lazily

// Largest single allocation of the operand rows (bytes); 0 = one allocation.
// Set by tch_set_max_chunk_bytes or TCH_MAX_CHUNK_BYTES.
static long long g_max_chunk = -1;

size_t max_chunk_bytes() {
    if (g_max_chunk < 0) {
        const char* v = getenv("TCH_MAX_CHUNK_BYTES");
        g_max_chunk = v ? atoll(v) : 0;
        if (g_max_chunk < 0) g_max_chunk = 0;
    }
    return (size_t)g_max_chunk;
}

// Rare term of solvers built from calls: 1 = dense per-stripe counts from the
// rare groups, 0 = pair lists.  Set by tch_set_rare_term or TCH_RARE.
static int g_rare_dense = -1;

static bool rare_dense_default() {
    if (g_rare_dense < 0) {
        const char* v = getenv("TCH_RARE");
        g_rare_dense = (v && !strcmp(v, "lists")) ? 0 : 1;
    }
    return g_rare_dense == 1;
}

// Stream-ordered pool of the per-stripe rare-count blocks, one per device; it
// keeps freed blocks for the next stripe instead of returning them at every
// synchronisation.
static std::mutex g_pool_mu;
static cudaMemPool_t g_pool[64];

static cudaError_t stripe_pool(int device, cudaMemPool_t* out) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    if (!g_pool[device]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaError_t e = cudaMemPoolCreate(&g_pool[device], &props);
        if (e != cudaSuccess) return e;
        uint64_t keep = ~0ull;
        e = cudaMemPoolSetAttribute(g_pool[device], cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) return e;
    }
    *out = g_pool[device];
    return cudaSuccess;
}

static const char* kKernelNames[TCH_KERNEL_COUNT] = {"auto",  "popc",   "mma_b1", "tc_f8",
                                                      "tc_i8", "tc_f16", "tc_f4"};

// Compiled in: the CUDA-core baseline and the fp4 tensor-core kernel.  The b1
// and s8 warp MMAs issue at ~150 TOPS on GB300, kind::i8 does not exist on
// sm_103a, and the fp8 kind runs at half the fp4 rate from twice the bytes.
static bool kernel_compiled(int k) { return k == TCH_KERNEL_POPC || k == TCH_KERNEL_TC_F4; }

static int default_kernel() {
    if (g_kernel < 0) {
        g_kernel = TCH_KERNEL_AUTO;
        const char* env = getenv("TCH_KERNEL");
        if (env)
            for (int k = 0; k < TCH_KERNEL_COUNT; k++)
                if (!strcmp(env, kKernelNames[k])) g_kernel = k;
    }
    return g_kernel;
}

// AUTO: the fastest kernel measured on GB300 that is compiled in and exact
// for this problem (fp32 accumulation of 0/+-1 products is exact while every
// partial sum stays below 2^24; a distance never exceeds the loci count, and
// the presence part alone bounds every partial sum by L <= 65535).
static int resolve_kernel(int k) { return k == TCH_KERNEL_AUTO ? TCH_KERNEL_TC_F4 : k; }

static bool is_tc(int k) { return k == TCH_KERNEL_TC_F4; }

}  // namespace tch

using namespace tch;

struct tch_solver {
    int device = 0, n = 0, L = 0, tau = 0, kernel = TCH_KERNEL_POPC;
    size_t n_pad = 0, K1 = 0, K2 = 0, D = 0;
    uint32_t* dP = nullptr;  // bit operands (popc kernel)
    uint32_t* dO = nullptr;
    Fp4Operands X;           // packed fp4 rows of the tensor-core kernel, split along K
    int kb = 0, kp = 0;      // bytes per row, presence columns
    uint32_t* dStart = nullptr;
    uint32_t* dJs = nullptr;
    size_t n_rare = 0;
    bool sorted = false;
    bool rare_on_host = false;              // reference fallback (tch.cu:140-144)
    // tch_run uploads the partner list stripe by stripe, overlapped with the
    // previous stripe's work (borrowed host arrays, valid during tch_run)
    const uint32_t* defer_start = nullptr;
    const uint32_t* defer_js = nullptr;
    const uint32_t* hStart = nullptr;       // borrowed for the host fallback
    const uint32_t* hJs = nullptr;
    // dense rare term: the rare groups stay on the device and every stripe's
    // counts are built just before its tile pass
    bool dense = false;
    uint16_t* gx = nullptr;          // n x L ranks
    uint64_t* gcnt_off = nullptr;
    uint64_t* ggoff = nullptr;
    uint32_t* gmembers = nullptr;
    uint32_t* gmpos = nullptr;
    uint64_t* groff = nullptr;       // every row's partner runs
    uint32_t* grlo = nullptr;
    uint32_t* grpre = nullptr;
    uint32_t* grtot = nullptr;
    int gL = 0;                      // loci of the rank rows (>= 1)
    int sub_rows = 0;                // rows per rare-count + tile-pass pair inside a stripe (0 = whole)
    int tile_group = 0;              // row blocks per raster group of the tile pass (0 = default)
    int* dErr = nullptr;
    int num_sms = 0;
    size_t bytes = 0;
};

namespace tch {

static cudaError_t dmalloc(tch_solver* s, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e == cudaSuccess) s->bytes += bytes;
    return e;
}

void solver_free(tch_solver* s) {
    if (!s) return;
    int cur = -1;
    cudaGetDevice(&cur);
    cudaSetDevice(s->device);
    cudaFree(s->dP);
    cudaFree(s->dO);
    free_fp4(&s->X);
    cudaFree(s->dStart);
    cudaFree(s->dJs);
    cudaFree(s->dErr);
    cudaFree(s->gx);
    cudaFree(s->gcnt_off);
    cudaFree(s->ggoff);
    cudaFree(s->gmembers);
    cudaFree(s->gmpos);
    cudaFree(s->groff);
    cudaFree(s->grlo);
    cudaFree(s->grpre);
    cudaFree(s->grtot);
    if (s->dense) {  // hand the pool's idle stripe blocks back
        cudaMemPool_t pool;
        if (stripe_pool(s->device, &pool) == cudaSuccess) {
            cudaDeviceSynchronize();
            cudaMemPoolTrimTo(pool, 0);
        }
    }
    if (cur >= 0) cudaSetDevice(cur);
    delete s;
}

// Operands on the device from the reference's bit layout (host buffers).
static int solver_from_bits(int device, int n, size_t n_pad, const uint8_t* O, size_t K1, const uint8_t* P,
                            size_t K2, const uint32_t* start, const uint32_t* js, size_t n_rare, int kernel,
                            int stripe_for_fit, bool allow_host_rare, tch_solver** out, Err& e,
                            bool defer_js = false) {
    tch_solver* s = nullptr;
    int* dflag = nullptr;
    int hflag = 0;
    size_t freeb = 0, totb = 0;
    bool rare_gpu = true;
    *out = nullptr;
    if (n < 0) return e.set("n must be >= 0 (got %d)", n);
    if (n_pad < (size_t)n || (n_pad % 256) != 0) return e.set("n_pad must be a multiple of 256 and >= n");
    if (K1 == 0 || K2 == 0 || (K1 % 1024) != 0 || (K2 % 1024) != 0)
        return e.set("K1 and K2 must be positive multiples of 1024 (got %zu, %zu)", K1, K2);
    if ((n > 0 && (!O || !P)) || (n_rare > 0 && (!start || !js))) return e.set("null input buffer");
    if (n > 0 && start) {  // CSR bounds (host side; the device checks the partners)
        for (int i = 0; i < n; i++)
            if (start[i] > start[i + 1]) return e.set("rare CSR: start[%d] > start[%d]", i, i + 1);
        if ((size_t)start[n] > n_rare) return e.set("rare CSR: start[n] = %u > n_rare = %zu", start[n], n_rare);
    }
    kernel = resolve_kernel(kernel);
    if (!kernel_compiled(kernel)) return e.set("kernel %d (%s) is not available", kernel, tch_kernel_name(kernel));

    s = new tch_solver();
    s->device = device;
    s->n = n;
    s->n_pad = n_pad;
    s->K1 = K1;
    s->K2 = K2;
    s->kernel = kernel;
    s->n_rare = n_rare;
    TCH_CK(e, cudaSetDevice(device));
    TCH_CK(e, cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, device));
    TCH_CK(e, dmalloc(s, (void**)&s->dErr, sizeof(int)));
    TCH_CK(e, cudaMemset(s->dErr, 0, sizeof(int)));
    TCH_CK(e, dmalloc(s, (void**)&s->dP, n_pad * K2 / 8));
    TCH_CK(e, dmalloc(s, (void**)&s->dO, n_pad * K1 / 8));
    if (n_pad) {
        TCH_CK(e, cudaMemcpy(s->dP, P, n_pad * K2 / 8, cudaMemcpyHostToDevice));
        TCH_CK(e, cudaMemcpy(s->dO, O, n_pad * K1 / 8, cudaMemcpyHostToDevice));
    }
    if (is_tc(kernel)) {
        // packed fp4 rows [presence | one-hot]: only the bit words that hold a
        // set bit in some row (K2 and K1 carry the reference's padding to 1024)
        BitOperands bits;
        bits.P = s->dP;
        bits.O = s->dO;
        bits.wP = (int)(K2 / 32);
        bits.wO = (int)(K1 / 32);
        int wp = 0, wo = 0;
        TCH_CK(e, used_bit_words(bits, n_pad, &wp, &wo, 0));
        s->kp = 32 * wp;
        s->kb = (int)(fp4_columns((size_t)32 * wp, (size_t)32 * wo) / 2);
        if (!chunk_width_for(s->kb, up((size_t)std::max(n, 1), 256), max_chunk_bytes()))
            { e.set("the operand needs more than %d K chunks", kMaxKChunks); goto fail; }
        TCH_CK(e, alloc_fp4(&s->X, up((size_t)std::max(n, 1), 256), s->kb, max_chunk_bytes(), true, true, &s->bytes));
        TCH_CK(e, launch_expand_bits(bits, n, wp, wo, s->X, 0));
        TCH_CK(e, cudaDeviceSynchronize());
        cudaFree(s->dP);
        cudaFree(s->dO);
        s->bytes -= n_pad * K2 / 8 + n_pad * K1 / 8;
        s->dP = s->dO = nullptr;
    }
    // rare pairs: on the device when they fit (tch.cu:104-111), else on the host
    TCH_CK(e, cudaMemGetInfo(&freeb, &totb));
    {
        const size_t need = (n_rare + (size_t)n + 1) * 4 + (size_t)stripe_for_fit * up((size_t)n, 8) * 2 * 2 +
                            ((size_t)64 << 20);
        rare_gpu = need < freeb;
        const char* force = getenv("TCH_FORCE_HOST_RARE");  // test hook: behave as if they did not fit
        if (force && force[0] == '1') rare_gpu = false;
    }
    if (!rare_gpu && !allow_host_rare)
        { e.set("rare pairs (%zu) do not fit in device memory", n_rare); goto fail; }
    if (rare_gpu) {
        TCH_CK(e, dmalloc(s, (void**)&s->dStart, ((size_t)n + 1) * 4));
        TCH_CK(e, dmalloc(s, (void**)&s->dJs, std::max<size_t>(n_rare, 1) * 4));
        if (start) TCH_CK(e, cudaMemcpy(s->dStart, start, ((size_t)n + 1) * 4, cudaMemcpyHostToDevice));
        else TCH_CK(e, cudaMemset(s->dStart, 0, ((size_t)n + 1) * 4));
        if (defer_js && n_rare && is_tc(kernel)) {  // uploaded and checked per stripe by solver_run
            s->defer_start = start;
            s->defer_js = js;
            s->sorted = false;
            *out = s;
            return 0;
        }
        if (n_rare) TCH_CK(e, cudaMemcpy(s->dJs, js, n_rare * 4, cudaMemcpyHostToDevice));
        // ascending rows -> subtraction fused into the contraction's epilogue
        TCH_CK(e, cudaMalloc(&dflag, sizeof(int)));
        TCH_CK(e, cudaMemset(dflag, 0, sizeof(int)));
        {
            RareCSR rc;
            rc.start = s->dStart;
            rc.js = s->dJs;
            rc.n_rare = n_rare;
            TCH_CK(e, launch_rare_check_sorted(rc, n, dflag, 0));
        }
        TCH_CK(e, cudaMemcpy(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost));
        cudaFree(dflag);
        dflag = nullptr;
        if (hflag & 2) { e.set("rare CSR: a partner j is not in (i, n)"); goto fail; }
        s->sorted = (hflag & 1) == 0;
    } else {
        s->rare_on_host = true;
        s->hStart = start;
        s->hJs = js;
        for (int i = 0; i < n; i++)
            for (uint32_t p = start[i]; p < start[i + 1]; p++)
                if (js[p] <= (uint32_t)i || js[p] >= (uint32_t)n) {
                    e.set("rare CSR: a partner j is not in (i, n)");
                    goto fail;
                }
    }
    *out = s;
    return 0;
fail:
    if (dflag) cudaFree(dflag);
    solver_free(s);
    return 1;
}

static TauModel g_tau_model;

// Operands on the device straight from allele calls (host buffer, n x L u64,
// 0 = missing): the device encoder of k_encode.cu, then the tensor-core kernel.
// Ranks (u16, 0 = missing) as allele ids: equal ranks are equal alleles.
__global__ void widen_ranks_kernel(const uint16_t* __restrict__ x, size_t count, uint64_t* calls) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x)
        calls[t] = x[t];
}

// calls: host u64 allele ids, or (ranks != nullptr) host u16 ranks, or
// (dev_calls != nullptr, L >= 1) u64 allele ids already in device memory.
static int solver_from_input(int device, int n, int L, const uint64_t* calls, const uint16_t* ranks, int tau,
                             int kernel, bool verbose, tch_solver** out, Err& e,
                             const uint64_t* dev_calls = nullptr) {
    tch_solver* s = nullptr;
    uint64_t* d_calls = nullptr;
    uint16_t* d_ranks = nullptr;
    DeviceEncoding enc;
    *out = nullptr;
    if (n < 0 || L < 0) return e.set("negative size (n=%d, L=%d)", n, L);
    if (L > 65535) return e.set("more than 65535 loci (u16 distances)");
    if ((size_t)n * L && !calls && !ranks && !dev_calls) return e.set("null input buffer");
    if (dev_calls && L < 1) return e.set("device calls need L >= 1");
    kernel = resolve_kernel(kernel);
    if (kernel != TCH_KERNEL_TC_F4)
        return e.set("the device encoder feeds the tensor-core kernel (tc_f4); kernel %s is not supported here",
                     tch_kernel_name(kernel));
    const int Le = std::max(L, 1);  // no loci: one all-zero column keeps every shape valid
    s = new tch_solver();
    s->device = device;
    s->n = n;
    s->L = L;
    s->kernel = kernel;
    TCH_CK(e, cudaSetDevice(device));
    TCH_CK(e, cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, device));
    TCH_CK(e, dmalloc(s, (void**)&s->dErr, sizeof(int)));
    TCH_CK(e, cudaMemset(s->dErr, 0, sizeof(int)));
    if (!dev_calls) TCH_CK(e, cudaMalloc(&d_calls, std::max<size_t>((size_t)n * Le, 1) * 8));
    if (dev_calls) {
        // read in place
    } else if (L && ranks) {
        const size_t count = (size_t)n * L;
        TCH_CK(e, cudaMalloc(&d_ranks, std::max<size_t>(count, 1) * 2));
        if (count) {
            TCH_CK(e, cudaMemcpy(d_ranks, ranks, count * 2, cudaMemcpyHostToDevice));
            widen_ranks_kernel<<<(int)std::min<size_t>((count + 255) / 256, (size_t)s->num_sms * 32), 256>>>(
                d_ranks, count, d_calls);
            TCH_CK(e, cudaGetLastError());
        }
        cudaFree(d_ranks);
        d_ranks = nullptr;
    } else if (L) {
        if ((size_t)n * L) TCH_CK(e, cudaMemcpy(d_calls, calls, (size_t)n * L * 8, cudaMemcpyHostToDevice));
    } else {
        TCH_CK(e, cudaMemset(d_calls, 0, std::max<size_t>((size_t)n, 1) * 8));
    }
    if (encode_on_device(device, n, Le, dev_calls ? dev_calls : d_calls, tau, g_tau_model, verbose, max_chunk_bytes(),
                         rare_dense_default() ? ENC_DENSE : 0, &enc, e))
        goto fail;
    cudaFree(d_calls);
    d_calls = nullptr;
    if (enc.dense) {  // the solver takes the rare groups
        s->dense = true;
        s->gL = Le;
        s->gx = enc.x;
        s->gcnt_off = enc.cnt_off;
        s->ggoff = enc.goff;
        s->gmembers = enc.members;
        s->gmpos = enc.mpos;
        s->groff = enc.roff;
        s->grlo = enc.rlo;
        s->grpre = enc.rpre;
        s->grtot = enc.rtot;
        enc.roff = nullptr;
        enc.rlo = enc.rpre = enc.rtot = nullptr;
    } else {
        cudaFree(enc.x);
        enc.bytes -= (size_t)n * Le * 2;
    }
    enc.x = nullptr;
    s->X = enc.X;
    enc.X = Fp4Operands();
    s->kb = enc.kb;
    s->kp = Le;
    s->n_pad = enc.x_rows;
    s->K2 = (size_t)Le;
    s->K1 = (size_t)enc.kb * 2 - (size_t)Le;
    s->D = enc.D;
    s->tau = enc.tau;
    s->sub_rows = enc.sub_rows;
    s->tile_group = enc.tile_group;
    s->dStart = enc.start;
    s->dJs = enc.js;
    s->n_rare = enc.n_rare;
    s->sorted = true;
    s->bytes += enc.bytes;
    *out = s;
    return 0;
fail:
    if (d_calls) cudaFree(d_calls);
    if (d_ranks) cudaFree(d_ranks);
    solver_free(s);
    return 1;
}

int solver_from_calls(int device, int n, int L, const uint64_t* calls, int tau, int kernel, bool verbose,
                      tch_solver** out, Err& e) {
    return solver_from_input(device, n, L, calls, nullptr, tau, kernel, verbose, out, e);
}

int solver_from_device_calls(int device, int n, int L, const uint64_t* d_calls, int tau, bool verbose,
                             tch_solver** out, Err& e) {
    return solver_from_input(device, n, L, nullptr, nullptr, tau, TCH_KERNEL_AUTO, verbose, out, e, d_calls);
}

static RareGroups rare_groups(const tch_solver* s) {
    RareGroups g;
    g.x = s->gx;
    g.cnt_off = s->gcnt_off;
    g.goff = s->ggoff;
    g.members = s->gmembers;
    g.mpos = s->gmpos;
    g.roff = s->groff;
    g.rlo = s->grlo;
    g.rpre = s->grpre;
    g.rtot = s->grtot;
    g.n = s->n;
    g.L = s->gL;
    return g;
}

// The tile pass with the stripe's rare counts in R (nullptr: no rare term).
static cudaError_t launch_dense_stripe(tch_solver* s, const StripeArgs& a, const uint16_t* R, size_t ldr,
                                       cudaStream_t st) {
    return launch_tc_stripe(s->X, nullptr, R, ldr, a, s->num_sms, st);
}

int solver_stripe(tch_solver* s, int r0, int rows, uint16_t* d_out, size_t ldo, cudaStream_t st, Err& e,
                  bool lists_uploaded) {
    if (r0 < 0 || rows < 0 || r0 > s->n) return e.set("stripe out of range (r0=%d rows=%d n=%d)", r0, rows, s->n);
    if (s->defer_js && !lists_uploaded) return e.set("partner lists not uploaded (run the whole pipeline)");
    if (r0 + rows > s->n) rows = s->n - r0;
    if (rows == 0) return 0;
    if (ldo < (size_t)(s->n - r0)) return e.set("ldo %zu < stripe width %d", ldo, s->n - r0);
    if (((uintptr_t)d_out & 15) != 0) return e.set("output pointer must be 16-byte aligned");
    if (is_tc(s->kernel) && (ldo & 1)) return e.set("ldo must be even for the tensor-core kernels");
    StripeArgs a;
    a.n = s->n;
    a.r0 = r0;
    a.rows = rows;
    a.out = d_out;
    a.ldo = ldo;
    a.err = s->dErr;
    a.group = s->tile_group;
    cudaError_t ce;
    const bool lists = !s->dense && !s->rare_on_host && s->n_rare > 0;
    if (s->kernel == TCH_KERNEL_POPC) {
        RareCSR rare;
        if (lists) {
            rare.start = s->dStart;
            rare.js = s->dJs;
            rare.n_rare = s->n_rare;
            rare.sorted = s->sorted;
        }
        BitOperands ops;
        ops.P = s->dP;
        ops.O = s->dO;
        ops.wP = (int)(s->K2 / 32);
        ops.wO = (int)(s->K1 / 32);
        ce = launch_popc_stripe(ops, rare, a, st);
        if (ce != cudaSuccess) return e.set("stripe kernel: %s", cudaGetErrorString(ce));
        return 0;
    }
    if (!s->dense && !lists) {  // no rare term on the device
        ce = launch_dense_stripe(s, a, nullptr, 0, st);
        if (ce != cudaSuccess) return e.set("stripe kernel: %s", cudaGetErrorString(ce));
        return 0;
    }
    // in sub-stripes of sub_rows rows (the solver's schedule): each one's rare
    // counts (from the rare groups or the pair lists) into a block of the pool,
    // then the tile pass that subtracts them
    const int sub = (s->sub_rows > 0 && rows > s->sub_rows) ? s->sub_rows : rows;
    cudaMemPool_t pool;
    ce = stripe_pool(s->device, &pool);
    if (ce != cudaSuccess) return e.set("stripe pool: %s", cudaGetErrorString(ce));
    for (int q0 = r0; q0 < r0 + rows; q0 += sub) {
        const int qrows = std::min(sub, r0 + rows - q0);
        const size_t ldr = up((size_t)(s->n - q0), kRareDenseAlign);
        const size_t rbytes = (size_t)qrows * ldr * 2;
        uint16_t* R = nullptr;
        ce = cudaMallocFromPoolAsync((void**)&R, rbytes, pool, st);
        if (ce != cudaSuccess)
            return e.set("rare counts of the stripe (%zu bytes): %s", rbytes, cudaGetErrorString(ce));
        StripeArgs qa = a;
        qa.r0 = q0;
        qa.rows = qrows;
        qa.out = d_out + (size_t)(q0 - r0) * ldo + (size_t)(q0 - r0);  // a triangle's columns start at its first row
        ce = s->dense ? launch_rare_dense(rare_groups(s), q0, qrows, R, ldr, s->num_sms, st)
                      : launch_rare_from_lists(s->dStart, s->dJs, s->n, q0, qrows, R, ldr, s->dErr, s->num_sms, st);
        if (ce == cudaSuccess) ce = launch_dense_stripe(s, qa, R, ldr, st);
        const cudaError_t fe = cudaFreeAsync(R, st);
        if (ce == cudaSuccess) ce = fe;
        if (ce != cudaSuccess) return e.set("stripe kernel: %s", cudaGetErrorString(ce));
    }
    return 0;
}

int solver_check(tch_solver* s, Err& e) {
    int h = 0;
    TCH_CK(e, cudaSetDevice(s->device));
    TCH_CK(e, cudaDeviceSynchronize());
    TCH_CK(e, cudaMemcpy(&h, s->dErr, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        cudaMemset(s->dErr, 0, sizeof(int));
        return e.set("device reported error 0x%x (%s%s%s)", h, (h & DEVERR_RARE_PAIR) ? "invalid rare pair " : "",
                     (h & DEVERR_OVERFLOW) ? "distance overflow " : "", (h & DEVERR_TIMEOUT) ? "wait timeout" : "");
    }
    return 0;
fail:
    return 1;
}

// Stripe pipeline through pinned host memory, two streams (tch.cu:113-149).
// Page-locked stripe buffers cost far more to allocate than to use, so the
// pair of the previous run is kept for the next one (one pair per process;
// a run that finds it in use allocates its own).
struct PinnedPool {
    std::mutex mu;
    void* buf[2] = {nullptr, nullptr};
    size_t bytes = 0;
    bool busy = false;
};
static PinnedPool g_pinned;

static cudaError_t pinned_acquire(size_t bytes, uint16_t* out[2], bool* pooled) {
    {
        std::lock_guard<std::mutex> lk(g_pinned.mu);
        if (!g_pinned.busy) {
            if (g_pinned.bytes < bytes) {
                for (int b = 0; b < 2; b++) {
                    if (g_pinned.buf[b]) cudaFreeHost(g_pinned.buf[b]);
                    g_pinned.buf[b] = nullptr;
                }
                g_pinned.bytes = 0;
                for (int b = 0; b < 2; b++) {
                    const cudaError_t ce = cudaMallocHost(&g_pinned.buf[b], bytes);
                    if (ce != cudaSuccess) return ce;
                }
                g_pinned.bytes = bytes;
            }
            g_pinned.busy = true;
            out[0] = (uint16_t*)g_pinned.buf[0];
            out[1] = (uint16_t*)g_pinned.buf[1];
            *pooled = true;
            return cudaSuccess;
        }
    }
    *pooled = false;
    for (int b = 0; b < 2; b++) {
        const cudaError_t ce = cudaMallocHost((void**)&out[b], bytes);
        if (ce != cudaSuccess) return ce;
    }
    return cudaSuccess;
}

static void pinned_release(uint16_t* p[2], bool pooled) {
    if (pooled) {
        std::lock_guard<std::mutex> lk(g_pinned.mu);
        g_pinned.busy = false;
        return;
    }
    for (int b = 0; b < 2; b++)
        if (p[b]) cudaFreeHost(p[b]);
}

// Device-side copy from the caller's (pageable) host memory, for GPUs that
// reach host memory through the host's page tables (Grace-Blackwell: the
// NVLink-C2C link is coherent).  Runs asynchronously on the stripe's stream,
// unlike a cudaMemcpyAsync from pageable memory, which the host stages.
__global__ void pull_from_host_kernel(uint32_t* __restrict__ dst, const uint32_t* __restrict__ src, size_t count) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x)
        dst[k] = src[k];
}

static bool host_pages_visible(int device) {
    int a = 0, b = 0;
    if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess)
        return false;
    // opt-in: measured on GB300 the pull competes with the stripe kernel and
    // ends slower than the staged copy overlapped with it
    const char* on = getenv("TCH_HOST_PULL");
    return a == 1 && b == 1 && on && on[0] == '1';
}

static cudaError_t upload_u32(uint32_t* dst, const uint32_t* src, size_t count, bool pull, int sms,
                              cudaStream_t st) {
    if (!count) return cudaSuccess;
    if (!pull) return cudaMemcpyAsync(dst, src, count * 4, cudaMemcpyHostToDevice, st);
    const int blocks = (int)std::min<size_t>((count + 255) / 256, (size_t)sms * 2);
    pull_from_host_kernel<<<blocks, 256, 0, st>>>(dst, src, count);
    return cudaGetLastError();
}

// Row ranges whose partner lists are uploaded, checked and computed as one
// unit: the first stripe in sub-stripes of a quarter (multiples of 128 rows,
// so every sub-stripe's output starts 16-byte aligned), so that its tile pass
// starts after the first quarter's lists rather than the whole stripe's;
// every later stripe whole (its lists arrive while earlier stripes compute).
struct RowChunk {
    int r0, rows;
};

static std::vector<RowChunk> row_chunks(int n, int S) {
    std::vector<RowChunk> c;
    const int first = std::min(S, n);
    const int sub = S >= 1024 ? (int)up((size_t)S / 4, 128) : std::max(first, 1);
    for (int a = 0; a < first; a += sub) c.push_back({a, std::min(sub, first - a)});
    for (int r0 = S; r0 < n; r0 += S) c.push_back({r0, std::min(S, n - r0)});
    return c;
}

// Uploads every chunk's partner lists ahead of the pipeline, in row order, on
// a stream of its own, from a helper thread.  The device holds the whole
// partner array, so the copies reuse no buffer and only wait for the link; a
// copy from pageable host memory returns only once it has finished, so issued
// from the pipeline's own thread it would hold back the next stripe's launch
// and the previous stripe's callback.  A stripe stream waits for its chunks'
// events.
struct ListUploader {
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    int issued = 0;  // chunks whose copy is issued and whose event is recorded
    cudaError_t err = cudaSuccess;
    bool stop = false;
    cudaStream_t st = nullptr;
    std::vector<cudaEvent_t> ev;
    double seconds = 0;  // from the first copy issued to the last one returned

    cudaError_t start(const tch_solver* s, const std::vector<RowChunk>& chunks, bool pull);

    // chunk k's event once its copy is issued, or the uploader's error
    cudaError_t ready(int k, cudaEvent_t* out) {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return issued > k || err != cudaSuccess; });
        if (issued > k) {
            *out = ev[k];
            return cudaSuccess;
        }
        return err;
    }

    ~ListUploader() {
        if (th.joinable()) {
            {
                std::lock_guard<std::mutex> lk(mu);
                stop = true;
            }
            th.join();
        }
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
    }
};

cudaError_t ListUploader::start(const tch_solver* s, const std::vector<RowChunk>& chunks, bool pull) {
    const int ns = (int)chunks.size();
    cudaError_t ce = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (ce != cudaSuccess) return ce;
    ev.assign(ns, nullptr);
    for (cudaEvent_t& x : ev)
        if ((ce = cudaEventCreateWithFlags(&x, cudaEventDisableTiming)) != cudaSuccess) return ce;
    th = std::thread([this, s, chunks, ns, pull] {
        const auto t0 = std::chrono::steady_clock::now();
        cudaError_t ce = cudaSetDevice(s->device);
        for (int k = 0; k < ns && ce == cudaSuccess; k++) {
            {
                std::lock_guard<std::mutex> lk(mu);
                if (stop) return;
            }
            const size_t pa = s->defer_start[chunks[k].r0], pb = s->defer_start[chunks[k].r0 + chunks[k].rows];
            ce = upload_u32(s->dJs + pa, s->defer_js + pa, pb - pa, pull, s->num_sms, st);
            if (ce == cudaSuccess) ce = cudaEventRecord(ev[k], st);
            if (ce == cudaSuccess) {
                std::lock_guard<std::mutex> lk(mu);
                issued = k + 1;
                seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                cv.notify_all();
            }
        }
        if (ce != cudaSuccess) {
            std::lock_guard<std::mutex> lk(mu);
            err = ce;
            cv.notify_all();
        }
    });
    return cudaSuccess;
}

static double wall() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static bool verbose() {
    const char* v = getenv("TCH_VERBOSE");
    return v && v[0] == '1';
}

static int solver_run(tch_solver* s, int S, tch_cb cb, void* ctx, double* gpu_secs, Err& e) {
    const int n = s->n;
    const size_t ldo = up((size_t)std::max(n, 1), 8);
    uint16_t* dU[2] = {nullptr, nullptr};
    uint16_t* hU[2] = {nullptr, nullptr};
    bool pooled = false;
    std::vector<RowChunk> chunks;
    int ci = 0;             // next row chunk
    const bool pull = s->defer_js && host_pages_visible(s->device);
    ListUploader uploader;
    cudaStream_t st[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr}, t0 = nullptr, t1 = nullptr;
    int rc = 1, prev = -1;
    float ms = 0.f;
    double w0 = wall(), w_setup = 0, w_cb = 0;
    if (S <= 0) return e.set("stripe rows must be positive (got %d)", S);
    if (!cb) return e.set("null callback");
    S = std::min(S, std::max(n, 1));
    TCH_CK(e, cudaSetDevice(s->device));
    TCH_CK(e, pinned_acquire((size_t)S * ldo * 2, hU, &pooled));
    for (int b = 0; b < 2; b++) {
        TCH_CK(e, cudaMalloc(&dU[b], (size_t)S * ldo * 2));
        TCH_CK(e, cudaStreamCreateWithFlags(&st[b], cudaStreamNonBlocking));
        TCH_CK(e, cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming));
    }
    if (s->defer_js) {
        chunks = row_chunks(n, S);
        TCH_CK(e, uploader.start(s, chunks, pull));
    }
    w_setup = wall() - w0;
    TCH_CK(e, cudaEventCreate(&t0));
    TCH_CK(e, cudaEventCreate(&t1));
    TCH_CK(e, cudaEventRecord(t0, st[0]));
    TCH_CK(e, cudaStreamWaitEvent(st[1], t0, 0));
    for (int r0 = 0;; r0 += S) {
        if (r0 < n) {
            const int rows = std::min(S, n - r0), b = (r0 / S) & 1;
            const size_t w = (size_t)(n - r0);
            if (s->defer_js) {
                // each row chunk of this stripe, once the uploader has issued the
                // copy of its partner lists: rare counts (which check every
                // partner) and the tile pass, writing rows and columns from the
                // chunk's first row on (the stripe's cells below the diagonal are
                // not part of the output)
                for (; ci < (int)chunks.size() && chunks[ci].r0 < r0 + rows; ci++) {
                    cudaEvent_t uploaded = nullptr;
                    TCH_CK(e, uploader.ready(ci, &uploaded));
                    TCH_CK(e, cudaStreamWaitEvent(st[b], uploaded, 0));
                    const int ca = chunks[ci].r0, cr = chunks[ci].rows;
                    const size_t off = (size_t)(ca - r0);
                    if (solver_stripe(s, ca, cr, dU[b] + off * ldo + off, ldo, st[b], e, true)) goto fail;
                }
            } else if (solver_stripe(s, r0, rows, dU[b], ldo, st[b], e, false)) {
                goto fail;
            }
            // pitched: a stripe's rows are n - r0 wide; with two stripes in flight this ran
            // 37.1 ms per whole triangle, a device repack to packed rows plus one linear
            // copy 40.3 ms
            TCH_CK(e, cudaMemcpy2DAsync(hU[b], w * 2, dU[b], ldo * 2, w * 2, rows, cudaMemcpyDeviceToHost, st[b]));
            TCH_CK(e, cudaEventRecord(done[b], st[b]));
        }
        if (prev >= 0) {  // consume the previous stripe while this one runs
            const int rows = std::min(S, n - prev), b = (prev / S) & 1;
            const size_t w = (size_t)(n - prev);
            TCH_CK(e, cudaEventSynchronize(done[b]));
            if (s->rare_on_host && s->hStart)
                for (int r = 0; r < rows; r++) {
                    const int i = prev + r;
                    for (uint32_t p = s->hStart[i]; p < s->hStart[i + 1]; p++)
                        hU[b][(size_t)r * w + (s->hJs[p] - prev)] -= 1;
                }
            const double wc = wall();
            cb(ctx, prev, rows, w, hU[b]);
            w_cb += wall() - wc;
        }
        if (r0 >= n) break;
        prev = r0;
    }
    TCH_CK(e, cudaStreamWaitEvent(st[0], done[1], 0));
    TCH_CK(e, cudaEventRecord(t1, st[0]));
    TCH_CK(e, cudaEventSynchronize(t1));
    TCH_CK(e, cudaEventElapsedTime(&ms, t0, t1));
    if (gpu_secs) *gpu_secs = ms / 1e3;
    if (solver_check(s, e)) goto fail;
    if (verbose()) {
        double up_s;
        {
            std::lock_guard<std::mutex> lk(uploader.mu);
            up_s = uploader.seconds;
        }
        fprintf(stderr,
                "tch: stripes %d rows: setup %.1f ms, pipeline %.1f ms (device %.1f ms, callbacks %.1f ms, "
                "partner uploads %.1f ms)\n",
                S, w_setup * 1e3, (wall() - w0 - w_setup) * 1e3, ms, w_cb * 1e3, up_s * 1e3);
    }
    rc = 0;
fail:
    for (int b = 0; b < 2; b++) {
        if (st[b]) cudaStreamSynchronize(st[b]);
        if (dU[b]) cudaFree(dU[b]);
        if (st[b]) cudaStreamDestroy(st[b]);
        if (done[b]) cudaEventDestroy(done[b]);
    }
    pinned_release(hU, pooled);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    return rc;
}

// A stripe with the rare-count block in caller memory R (dense-rare solvers;
// others take the ordinary path): no allocation, so it can be captured.
int solver_stripe_counts(tch_solver* s, int r0, int rows, uint16_t* d_out, size_t ldo, uint16_t* R, size_t ldr,
                         cudaStream_t st, Err& e) {
    if (!s->dense) return solver_stripe(s, r0, rows, d_out, ldo, st, e);
    if (r0 < 0 || rows < 0 || r0 > s->n) return e.set("stripe out of range (r0=%d rows=%d n=%d)", r0, rows, s->n);
    if (r0 + rows > s->n) rows = s->n - r0;
    if (rows == 0) return 0;
    if (ldo < (size_t)(s->n - r0) || (ldo & 1) || ((uintptr_t)d_out & 15))
        return e.set("ldo must be even and >= n - r0, the output 16-byte aligned");
    if (ldr < up((size_t)(s->n - r0), kRareDenseAlign) || (ldr & 7) || ((uintptr_t)R & 15))
        return e.set("rare-count block too narrow or misaligned");
    StripeArgs a;
    a.n = s->n;
    a.r0 = r0;
    a.rows = rows;
    a.out = d_out;
    a.ldo = ldo;
    a.err = s->dErr;
    cudaError_t ce = launch_rare_dense(rare_groups(s), r0, rows, R, ldr, s->num_sms, st);
    if (ce == cudaSuccess) ce = launch_dense_stripe(s, a, R, ldr, st);
    if (ce != cudaSuccess) return e.set("stripe kernel: %s", cudaGetErrorString(ce));
    return 0;
}

// Work of one whole-triangle solve, for scheduling: pairs x operand bytes per row.
double solver_work(const tch_solver* s) { return (double)s->n * (double)(s->n - 1) / 2.0 * (double)s->kb; }

int solver_size(const tch_solver* s) { return s->n; }

const Fp4Operands* solver_operands(const tch_solver* s) { return is_tc(s->kernel) ? &s->X : nullptr; }

bool solver_rare_groups(const tch_solver* s, RareGroups* g) {
    if (!s->dense) return false;
    *g = rare_groups(s);
    return true;
}

}  // namespace tch

// ==================================================================================
// exported C ABI
// ==================================================================================

extern "C" {

int tch_device_count(void) {
    int c = 0;
    return cudaGetDeviceCount(&c) == cudaSuccess ? c : 0;
}

size_t tch_free_vram(int device) {
    size_t f = 0, t = 0;
    if (cudaSetDevice(device) != cudaSuccess || cudaMemGetInfo(&f, &t) != cudaSuccess) return 0;
    return f;
}

int tch_run(int device, int n, size_t n_pad, const uint8_t* O, size_t K1, const uint8_t* P, size_t K2,
            const uint32_t* start, const uint32_t* js, size_t n_rare, int S, tch_cb cb, void* ctx,
            double* gpu_secs, int* rare_on_gpu, char* err, int errlen) {
    Err e{err, errlen};
    tch_solver* s = nullptr;
    if (S <= 0) return e.set("stripe rows must be positive (got %d)", S);
    const double w0 = wall();
    if (solver_from_bits(device, n, n_pad, O, K1, P, K2, start, js, n_rare, default_kernel(), S, true, &s, e, true))
        return 1;
    if (verbose())
        fprintf(stderr, "tch: operands on the device in %.1f ms (%.2f GB uploaded)\n", (wall() - w0) * 1e3,
                (double)(n_pad * (K1 + K2) / 8 + (n_rare + (size_t)n + 1) * 4) / 1e9);
    if (rare_on_gpu) *rare_on_gpu = s->rare_on_host ? 0 : 1;
    const double w1 = wall();
    const int rc = solver_run(s, S, cb, ctx, gpu_secs, e);
    const double w2 = wall();
    solver_free(s);
    if (verbose())
        fprintf(stderr, "tch: tch_run %.1f ms: operands %.1f, stripes %.1f, release %.1f\n", (wall() - w0) * 1e3,
                (w1 - w0) * 1e3, (w2 - w1) * 1e3, (wall() - w2) * 1e3);
    return rc;
}

int tch_version(void) { return TCH_VERSION; }

const char* tch_kernel_name(int kernel) {
    return kernel >= 0 && kernel < TCH_KERNEL_COUNT ? kKernelNames[kernel] : "?";
}

int tch_kernel_available(int kernel) { return kernel == TCH_KERNEL_AUTO || kernel_compiled(kernel) ? 1 : 0; }

int tch_set_kernel(int kernel) {
    if (kernel < 0 || kernel >= TCH_KERNEL_COUNT || !tch_kernel_available(kernel)) return 1;
    g_kernel = kernel;
    return 0;
}

int tch_get_kernel(void) { return default_kernel(); }

int tch_solver_from_bits(int device, int n, size_t n_pad, const uint8_t* O, size_t K1, const uint8_t* P,
                         size_t K2, const uint32_t* start, const uint32_t* js, size_t n_rare, int kernel,
                         tch_solver** out, char* err, int errlen) {
    Err e{err, errlen};
    if (!out) return e.set("null output handle");
    return solver_from_bits(device, n, n_pad, O, K1, P, K2, start, js, n_rare, kernel, 0, false, out, e);
}

int tch_solver_from_calls(int device, int n, int L, const uint64_t* calls, int tau, int kernel, tch_solver** out,
                          char* err, int errlen) {
    Err e{err, errlen};
    if (!out) return e.set("null output handle");
    return solver_from_calls(device, n, L, calls, tau, kernel, false, out, e);
}

int tch_solver_from_ranks(int device, int n, int L, const uint16_t* ranks, int tau, int kernel, tch_solver** out,
                          char* err, int errlen) {
    Err e{err, errlen};
    if (!out) return e.set("null output handle");
    if ((size_t)n * L && !ranks) return e.set("null input buffer");
    return solver_from_input(device, n, L, nullptr, ranks, tau, kernel, false, out, e);
}

int tch_run_calls(int device, int n, int L, const uint64_t* calls, int tau, int S, tch_cb cb, void* ctx,
                  double* gpu_secs, int* tau_used, char* err, int errlen) {
    Err e{err, errlen};
    tch_solver* s = nullptr;
    if (S <= 0) return e.set("stripe rows must be positive (got %d)", S);
    const char* v = getenv("TCH_VERBOSE");
    if (solver_from_calls(device, n, L, calls, tau, TCH_KERNEL_AUTO, v && v[0] == '1', &s, e)) return 1;
    if (tau_used) *tau_used = s->tau;
    const int rc = n > 0 ? solver_run(s, S, cb, ctx, gpu_secs, e) : 0;
    solver_free(s);
    return rc;
}

int tch_tau_features(int device, int n, int L, const uint64_t* calls, int max_rows, int* taus, int* sub_rows,
                     int* groups, float* feats, double* est_s, int* rows, char* err, int errlen) {
    Err e{err, errlen};
    uint64_t* d_calls = nullptr;
    DeviceEncoding enc;
    TauTable table;
    if (n < 2 || L < 1) return e.set("need n >= 2 profiles and L >= 1 loci (got n=%d, L=%d)", n, L);
    if (L > 65535) return e.set("more than 65535 loci (u16 distances)");
    if (!calls || !taus || !feats || !rows || max_rows < 0) return e.set("null buffer");
    TCH_CK(e, cudaSetDevice(device));
    TCH_CK(e, cudaMalloc(&d_calls, (size_t)n * L * 8));
    TCH_CK(e, cudaMemcpy(d_calls, calls, (size_t)n * L * 8, cudaMemcpyHostToDevice));
    if (encode_on_device(device, n, L, d_calls, 0, g_tau_model, false, 0, rare_dense_default() ? ENC_DENSE : 0, &enc,
                         e, &table))
        goto fail;
    cudaFree(d_calls);
    *rows = (int)std::min<size_t>(table.taus.size(), (size_t)max_rows);
    for (int r = 0; r < *rows; r++) {
        taus[r] = table.taus[r];
        if (sub_rows) sub_rows[r] = table.subs[r];
        if (groups) groups[r] = table.groups[r];
        if (est_s) est_s[r] = table.est_s[r];
        for (int f = 0; f < TCH_TAU_FEATURES; f++) feats[(size_t)r * TCH_TAU_FEATURES + f] =
            table.feats[(size_t)r * TCH_TAU_FEATURES + f];
    }
    return 0;
fail:
    if (d_calls) cudaFree(d_calls);
    return 1;
}

int tch_set_max_chunk_bytes(size_t bytes) {
    g_max_chunk = (long long)bytes;
    return 0;
}

int tch_set_dense_rare_rate(double rate) {
    if (!(rate > 0)) return 1;
    g_tau_model.dense_rate = rate;
    return 0;
}

int tch_set_rare_term(int dense) {
    g_rare_dense = dense ? 1 : 0;
    return 0;
}

int tch_set_tau_model(double gemm_rate, double rare_rate) {
    if (!(gemm_rate > 0) || !(rare_rate > 0)) return 1;
    g_tau_model.gemm_rate = gemm_rate;
    g_tau_model.rare_rate = rare_rate;
    return 0;
}

int tch_solver_info(const tch_solver* s, tch_info* info) {
    if (!s || !info) return 1;
    memset(info, 0, sizeof(*info));
    info->n = s->n;
    info->L = s->L;
    info->tau = s->tau;
    info->kernel = s->kernel;
    info->n_pad = s->n_pad;
    info->k_presence = s->K2;
    info->k_onehot = s->K1;
    info->d_onehot = s->D;
    info->n_rare = s->n_rare;
    info->rare_sorted = s->sorted ? 1 : 0;
    info->device_bytes = s->bytes;
    info->k_chunks = is_tc(s->kernel) ? s->X.pos.n : 0;
    info->rare_dense = s->dense ? 1 : 0;
    info->sub_rows = s->sub_rows;
    info->tile_group = s->tile_group;
    return 0;
}

int tch_solver_set_schedule(tch_solver* s, int sub_rows, int tile_group) {
    if (!s || sub_rows < 0 || tile_group < 0 || tile_group > 256) return 1;
    s->sub_rows = sub_rows ? (int)up((size_t)sub_rows, 128) : 0;  // sub-stripe outputs stay 16-byte aligned
    s->tile_group = tile_group;
    return 0;
}

int tch_solver_stripe(tch_solver* s, int r0, int rows, uint16_t* d_out, size_t ldo, void* stream, char* err,
                      int errlen) {
    Err e{err, errlen};
    if (!s) return e.set("null solver");
    if (!d_out && rows > 0) return e.set("null output");
    if (cudaSetDevice(s->device) != cudaSuccess) return e.set("cudaSetDevice(%d) failed", s->device);
    return solver_stripe(s, r0, rows, d_out, ldo, (cudaStream_t)stream, e);
}

int tch_solver_rare_counts(tch_solver* s, int r0, int rows, uint16_t* d_R, size_t ldr, void* stream, char* err,
                           int errlen) {
    Err e{err, errlen};
    if (!s) return e.set("null solver");
    if (!s->dense) return e.set("the solver holds pair lists, not rare groups");
    if (r0 < 0 || rows < 0 || r0 > s->n) return e.set("stripe out of range (r0=%d rows=%d n=%d)", r0, rows, s->n);
    if (r0 + rows > s->n) rows = s->n - r0;
    if (rows == 0) return 0;
    const size_t width = up((size_t)(s->n - r0), kRareDenseAlign);
    if (!d_R || ldr < width || (ldr & 7) || ((uintptr_t)d_R & 15))
        return e.set("rare counts need a 16-byte aligned block with ldr >= %zu, a multiple of 8 (got %zu)", width, ldr);
    if (cudaSetDevice(s->device) != cudaSuccess) return e.set("cudaSetDevice(%d) failed", s->device);
    const cudaError_t ce = launch_rare_dense(rare_groups(s), r0, rows, d_R, ldr, s->num_sms, (cudaStream_t)stream);
    if (ce != cudaSuccess) return e.set("rare counts: %s", cudaGetErrorString(ce));
    return 0;
}

int tch_solver_stripe_counts(tch_solver* s, int r0, int rows, uint16_t* d_out, size_t ldo, const uint16_t* d_R,
                             size_t ldr, void* stream, char* err, int errlen) {
    Err e{err, errlen};
    if (!s) return e.set("null solver");
    if (!s->dense) return e.set("the solver holds pair lists, not rare groups");
    if (r0 < 0 || rows < 0 || r0 > s->n) return e.set("stripe out of range (r0=%d rows=%d n=%d)", r0, rows, s->n);
    if (r0 + rows > s->n) rows = s->n - r0;
    if (rows == 0) return 0;
    if (!d_out) return e.set("null output");
    if (ldo < (size_t)(s->n - r0) || (ldo & 1)) return e.set("ldo must be even and >= n - r0 (got %zu)", ldo);
    if (((uintptr_t)d_out & 15) != 0) return e.set("output pointer must be 16-byte aligned");
    const size_t width = up((size_t)(s->n - r0), kRareDenseAlign);
    if (!d_R || ldr < width || (ldr & 7) || ((uintptr_t)d_R & 15))
        return e.set("rare counts need a 16-byte aligned block with ldr >= %zu, a multiple of 8 (got %zu)", width, ldr);
    if (cudaSetDevice(s->device) != cudaSuccess) return e.set("cudaSetDevice(%d) failed", s->device);
    StripeArgs a;
    a.n = s->n;
    a.r0 = r0;
    a.rows = rows;
    a.out = d_out;
    a.ldo = ldo;
    a.err = s->dErr;
    const cudaError_t ce = launch_dense_stripe(s, a, d_R, ldr, (cudaStream_t)stream);
    if (ce != cudaSuccess) return e.set("stripe kernel: %s", cudaGetErrorString(ce));
    return 0;
}

int tch_solver_check(tch_solver* s, char* err, int errlen) {
    Err e{err, errlen};
    if (!s) return e.set("null solver");
    return solver_check(s, e);
}

int tch_solver_run(tch_solver* s, int S, tch_cb cb, void* ctx, double* gpu_secs, char* err, int errlen) {
    Err e{err, errlen};
    if (!s) return e.set("null solver");
    return solver_run(s, S, cb, ctx, gpu_secs, e);
}

void tch_solver_destroy(tch_solver* s) { solver_free(s); }

}  // extern "C"
