// tch_stripe_noalloc: one stripe of the distance matrix for callers that may
// not allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits — a host that
// hands this library memory it already owns and forbids further device
// allocations (a fixed-budget service, a framework whose allocator must see
// every byte), or code running while the caller holds a stream it must not
// synchronise through an allocation.  tch_solver_* allocate their operand
// expansion and error word with cudaMalloc; this entry point instead keeps
// that scratch in one file-scope device array, so a call allocates nothing.
//
// The scratch (g_noalloc_scratch, TCH_NOALLOC_SCRATCH_BYTES) holds
//   [0, 256)       the device error word of the call
//   [256, ...)     the two packed fp4 copies of the operand rows [presence |
//                  one-hot] of all n profiles (K2 + K1 columns, half a byte
//                  each, so both copies take one byte per bit column)
// It is a static device array: the module that holds it is loaded on the
// first call of this entry point (or at library load when CUDA loads modules
// eagerly), and a device that has loaded it keeps the memory until the
// process exits.  Every call shares the array and leaves its contents behind;
// the error word is cleared at the start of each call and the operand rows
// are rewritten in full.  Calls whose work overlaps on the GPU race on the
// array, so issue them one after another (this entry point synchronises the
// stream before it returns).
//
// Set-up, once per device: the first call on a device, with that device
// current, takes the array's device address with cudaGetSymbolAddress (in
// host code the symbol is only a host-side stand-in).  Make that first call
// before any stream capture.

#include <mutex>

#include "tch_internal.cuh"

namespace tch {
namespace {

static __device__ __align__(256) uint8_t g_noalloc_scratch[TCH_NOALLOC_SCRATCH_BYTES];

constexpr size_t kErrBytes = 256;

std::mutex g_mu;
uint8_t* g_addr[kMaxDevices];  // device address of g_noalloc_scratch, per device

int scratch_address(int device, uint8_t** out, Err& e) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (device < 0 || device >= kMaxDevices) return e.set("device %d out of range", device);
    if (!g_addr[device]) {
        void* p = nullptr;
        const cudaError_t ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (ce != cudaSuccess) return e.set("cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(ce));
        g_addr[device] = static_cast<uint8_t*>(p);
    }
    *out = g_addr[device];
    return 0;
}

// start[] must be ascending with start[n] <= n_rare before any kernel walks it.
__global__ void check_offsets_kernel(const uint32_t* __restrict__ start, int n, size_t n_rare, int* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t a = start[i], b = start[i + 1];
        if (a > b || (size_t)b > n_rare) atomicOr(err, DEVERR_RARE_PAIR);
    }
}

// Makes `device` current for the call and gives the caller's device back on
// every return.
struct DeviceScope {
    int prev = -1;
    cudaError_t set(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        return cudaSetDevice(device);
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// An error after work was queued: wait for that work first, so that no
// kernel of this call still uses the shared array when the caller retries.
int fail_queued(cudaStream_t st, Err& e, const char* what, cudaError_t ce) {
    cudaStreamSynchronize(st);
    return e.set("%s: %s", what, cudaGetErrorString(ce));
}

int read_error(int* d_err, cudaStream_t st, Err& e) {
    int h = 0;
    cudaError_t ce = cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return e.set("reading the device error word: %s", cudaGetErrorString(ce));
    if (h & DEVERR_RARE_PAIR) return e.set("rare CSR: offsets not ascending or a partner j not in (i, n)");
    if (h) return e.set("device reported error 0x%x", h);
    return 0;
}

}  // namespace
}  // namespace tch

using namespace tch;

extern "C" int tch_stripe_noalloc(int device, int n, const uint8_t* d_O, size_t K1, const uint8_t* d_P, size_t K2,
                                  const uint32_t* d_start, const uint32_t* d_js, size_t n_rare, int r0, int rows,
                                  uint16_t* d_out, size_t ldo, void* stream, char* err, int errlen) {
    Err e{err, errlen};
    const cudaStream_t st = (cudaStream_t)stream;
    if (n <= 0) return e.set("n must be positive (got %d)", n);
    if (K1 == 0 || K2 == 0 || (K1 % 1024) || (K2 % 1024))
        return e.set("K1 and K2 must be positive multiples of 1024 (got %zu, %zu)", K1, K2);
    if (r0 < 0 || rows <= 0 || r0 >= n) return e.set("stripe out of range (r0=%d rows=%d n=%d)", r0, rows, n);
    if (r0 + rows > n) rows = n - r0;
    if (ldo < (size_t)(n - r0) || (ldo & 1)) return e.set("ldo must be even and >= n - r0 (got %zu)", ldo);
    if (!d_O || !d_P || !d_out || (n_rare && (!d_start || !d_js)) || !d_start)
        return e.set("null device buffer");
    if (((uintptr_t)d_out & 15) != 0) return e.set("output pointer must be 16-byte aligned");
    // rows of K2 presence then K1 one-hot columns (multiples of 1024): kb
    // bytes per copy, two copies
    const size_t kb = (K2 + K1) / 2;
    const size_t x_rows = up((size_t)n, 256);
    const size_t need = kErrBytes + 2 * x_rows * kb;
    if (need > (size_t)TCH_NOALLOC_SCRATCH_BYTES)
        return e.set("needs %zu bytes of scratch (n=%d padded to %zu rows x 2 x %zu bytes); the limit is %zu bytes",
                     need, n, x_rows, kb, (size_t)TCH_NOALLOC_SCRATCH_BYTES);
    if (kb > (size_t)INT32_MAX) return e.set("rows too wide");

    DeviceScope scope;
    cudaError_t ce = scope.set(device);
    if (ce != cudaSuccess) return e.set("cudaSetDevice(%d): %s", device, cudaGetErrorString(ce));
    uint8_t* scratch = nullptr;
    if (scratch_address(device, &scratch, e)) return 1;
    int* d_err = reinterpret_cast<int*>(scratch);
    uint8_t* X = scratch + kErrBytes;
    int sms = 0;
    ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (ce != cudaSuccess) return e.set("cudaDeviceGetAttribute: %s", cudaGetErrorString(ce));

    // 1. clear the error word, check the CSR offsets before anything walks them
    ce = cudaMemsetAsync(d_err, 0, sizeof(int), st);
    if (ce != cudaSuccess) return fail_queued(st, e, "cudaMemsetAsync", ce);
    check_offsets_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_start, n, n_rare, d_err);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return fail_queued(st, e, "offset check", ce);
    if (read_error(d_err, st, e)) return 1;

    // 2. bits -> packed fp4 operand rows in the scratch array, 3. the tile
    // pass, 4. the partner lists (any order) subtracted with atomics
    BitOperands bits;
    bits.P = reinterpret_cast<const uint32_t*>(d_P);
    bits.O = reinterpret_cast<const uint32_t*>(d_O);
    bits.wP = (int)(K2 / 32);
    bits.wO = (int)(K1 / 32);
    Fp4Operands ops;
    ops.n_rows = x_rows;
    ops.kb = (int)kb;
    for (int side = 0; side < 2; side++) {
        KChunks& k = side ? ops.neg : ops.pos;
        k.p[0] = X + side * x_rows * kb;
        k.n = 1;
        k.width = (int)kb;
        k.kb = (int)kb;
    }
    ce = launch_expand_bits(bits, n, bits.wP, bits.wO, ops, st);
    if (ce != cudaSuccess) return fail_queued(st, e, "operand expansion", ce);
    RareCSR rare;
    rare.start = d_start;
    rare.js = d_js;
    rare.n_rare = n_rare;
    StripeArgs a;
    a.n = n;
    a.r0 = r0;
    a.rows = rows;
    a.out = d_out;
    a.ldo = ldo;
    a.err = d_err;
    ce = launch_tc_stripe(ops, nullptr, nullptr, 0, a, sms, st);
    if (ce == cudaSuccess && n_rare) ce = launch_rare_atomic(rare, a, st);
    if (ce != cudaSuccess) return fail_queued(st, e, "stripe kernel", ce);
    return read_error(d_err, st, e);
}
