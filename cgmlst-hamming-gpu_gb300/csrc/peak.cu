// tch-peak: measured instruction throughput of every arithmetic path a binary
// Hamming contraction could take on this GPU, so that the roofline of the
// contraction kernel is quoted against a number taken on the same part.
//
//   b1     mma.sync m16n8k256 b1 AND+popc -> s32   (legacy warp MMA)
//   s8     mma.sync m16n8k32 s8 -> s32             (legacy warp MMA)
//   e4m3   mma.sync m16n8k32 e4m3 -> f32           (legacy warp MMA)
//   popc   LOP3 AND + POPC + IADD on CUDA cores    (32 bit-MACs per instruction)
//   tc_f8  tcgen05.mma kind::f8f6f4, M128 N256 K32, shared memory -> TMEM
//   tc_f4  tcgen05.mma kind::mxf4 block-scaled (every scale 1.0), M128 N256
//          K64 packed e2m1 -> TMEM
//
// The warp-MMA and CUDA-core paths run a few independent dependency chains
// per thread over operands drawn from a seed passed at launch, and every
// thread writes the fold of its accumulators to its own word of a sink array.
// The tcgen05 paths keep one CTA per SM with a single issuing thread, and
// check every accumulator they read back against the exact expected integer
// (operands are +-1 everywhere), so a wrong encoding shows as a mismatch.
//
// Usage: tch-peak [path ...]   (default: every path).  Prints one JSON object;
// a MAC counts as 2 ops.

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "tc_ptx.cuh"

using namespace tch::ptx;

#define CK(x)                                                                \
    do {                                                                     \
        cudaError_t e_ = (x);                                                \
        if (e_ != cudaSuccess) {                                             \
            fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));         \
            return 1;                                                        \
        }                                                                    \
    } while (0)

// ------------------------------------------------------------ warp-level MMA
constexpr int CHAINS = 6;  // independent accumulator chains per thread

__device__ __forceinline__ uint32_t mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    return x ^ (x >> 16);
}

enum WarpPath { W_B1 = 0, W_S8 = 1, W_E4M3 = 2 };

template <int P>
__device__ __forceinline__ void warp_mma(uint32_t (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    if (P == W_B1)
        asm volatile("mma.sync.aligned.m16n8k256.row.col.s32.b1.b1.s32.and.popc "
                     "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                     : "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    else if (P == W_S8)
        asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 "
                     "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                     : "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    else  // fp32 accumulators carried in 32-bit registers
        asm volatile("mma.sync.aligned.m16n8k32.row.col.f32.e4m3.e4m3.f32 "
                     "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                     : "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <int P>
__global__ void warp_mma_rate(uint32_t seed, int rounds, uint32_t* sink) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    // e4m3 operands restricted to 0 and +1.0 (0x38) so sums stay exact integers
    const uint32_t mask = P == W_E4M3 ? 0x38383838u : 0xFFFFFFFFu;
    uint32_t a[4], b[CHAINS][2];
    uint32_t h = mix(seed ^ (tid * 0x9E3779B9u));
    for (int q = 0; q < 4; q++) a[q] = (h = mix(h + q)) & mask;
    for (int c = 0; c < CHAINS; c++) {
        b[c][0] = (h = mix(h ^ c)) & mask;
        b[c][1] = (h = mix(h + 0x51u)) & mask;
    }
    uint32_t acc[CHAINS][4] = {};
    for (int r = 0; r < rounds; r++) {
#pragma unroll
        for (int c = 0; c < CHAINS; c++) warp_mma<P>(acc[c], a, b[c][0], b[c][1]);
    }
    uint32_t f = 0;
    for (int c = 0; c < CHAINS; c++) f ^= acc[c][0] + 3 * acc[c][1] + 5 * acc[c][2] + 7 * acc[c][3];
    sink[tid] = f;
}

// CUDA cores: CHAINS x 2 popcount accumulators over seeded words that a
// linear congruential step keeps changing.
__global__ void popc_rate(uint32_t seed, int rounds, uint32_t* sink) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t x[CHAINS], y[2];
    uint32_t h = mix(seed + tid);
    for (int c = 0; c < CHAINS; c++) x[c] = h = mix(h ^ (c * 0x2545F491u));
    y[0] = mix(h + 1);
    y[1] = mix(h + 2);
    uint32_t acc[CHAINS][2] = {};
    for (int r = 0; r < rounds; r++) {
#pragma unroll
        for (int c = 0; c < CHAINS; c++) {
            acc[c][0] += __popc(x[c] & y[0]);
            acc[c][1] += __popc(x[c] & y[1]);
        }
        y[0] = y[0] * 1103515245u + 12345u;
        y[1] ^= y[0];
    }
    uint32_t f = 0;
    for (int c = 0; c < CHAINS; c++) f += acc[c][0] * 31u + acc[c][1];
    sink[tid] = f;
}

// ------------------------------------------------------------ tcgen05
enum TcPath { TC_F8 = 0, TC_F4 = 1, TC_NVF4_32 = 2, TC_NVF4_16 = 3 };
constexpr int TC_M = 128, TC_N_MAX = 256;
constexpr int TC_SF_COL = 256;          // scale factors (fp4) after the accumulator
constexpr int TC_SMEM = 120 * 1024;     // keeps one CTA per SM
constexpr int TC_A_BYTES = TC_M * 128, TC_B_BYTES = TC_N_MAX * 128;

// One stage of operands (A 128 rows, B TC_N rows of 128 bytes of K, every
// byte the same value) issued `iters` x 4 times into one accumulator of TC_N
// columns; then every warp reads back its lanes of the first and the last 32
// columns and compares them with `expect`.  err bit 1: a mismatch; bit 4: the
// completion wait timed out.
template <int P, int TC_N>
__global__ void __launch_bounds__(128, 1) tc_rate(int iters, uint32_t a_word, uint32_t b_word, float expect,
                                                  int* err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* A = smem;
    uint8_t* B = smem + TC_A_BYTES;
    uint64_t* bar = (uint64_t*)(smem + TC_A_BYTES + TC_B_BYTES);
    uint32_t* slot = (uint32_t*)(bar + 1);
    volatile int* abort_flag = (volatile int*)(slot + 1);
    const int warp = threadIdx.x / 32;
    for (int i = threadIdx.x; i < TC_A_BYTES / 4; i += blockDim.x) reinterpret_cast<uint32_t*>(A)[i] = a_word;
    for (int i = threadIdx.x; i < TC_B_BYTES / 4; i += blockDim.x) reinterpret_cast<uint32_t*>(B)[i] = b_word;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // operand writes -> tensor-core reads
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    const uint32_t lanes = (uint32_t)(warp * 32) << 16;
    if (P != TC_F8) {
        // every scale factor 1.0 (ue8m0 127, or ue4m3 0x38 for 16-element
        // blocks), wherever in these 32 columns the MMA reads it
        tmem_fill32(tmem + lanes + TC_SF_COL, 0x01010101u * (P == TC_NVF4_16 ? kUe4m3One : kUe8m0One));
        tmem_wait_st();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0) {
        const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
        if (P == TC_F8) {
            const uint32_t idesc = make_idesc(1, 0, 0, TC_M, TC_N);
            for (int i = 0; i < iters; i++)
#pragma unroll
                for (int k = 0; k < 4; k++)
                    tc_mma_f8(tmem, sw128_desc(a0 + 32 * k), sw128_desc(b0 + 32 * k), idesc, (i | k) ? 1u : 0u);
        } else {
            const uint32_t idesc = make_idesc_mx(kE2M1, P == TC_NVF4_16 ? 0 : 1, TC_M, TC_N);
            const uint32_t sf = tmem + TC_SF_COL;
            for (int i = 0; i < iters; i++)
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const uint64_t ad = sw128_desc(a0 + 32 * k), bd = sw128_desc(b0 + 32 * k);
                    const uint32_t acc = (i | k) ? 1u : 0u;
                    if (P == TC_F4) tc_mma_mxf4(tmem, ad, bd, idesc, sf, sf, acc);
                    else if (P == TC_NVF4_32) tc_mma_nvf4<32>(tmem, ad, bd, idesc, sf, sf, acc);
                    else tc_mma_nvf4<16>(tmem, ad, bd, idesc, sf, sf, acc);
                }
        }
        tc_commit(bar);
        mbar_wait(bar, 0, abort_flag, err);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (!*abort_flag) {
        int bad = 0;
        for (int c0 = 0; c0 < TC_N; c0 += TC_N - 32) {  // columns 0-31 and TC_N-32 .. TC_N-1
            uint32_t v[32];
            tmem_ld32(tmem + lanes + (uint32_t)c0, v);
            tmem_wait_ld();
            for (int c = 0; c < 32; c++) bad |= __uint_as_float(v[c]) != expect;
        }
        if (bad) atomicOr(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
}

// ------------------------------------------------------------ host
struct Probe {
    cudaDeviceProp prop;
    uint32_t* sink = nullptr;
    int* err = nullptr;
    bool first = true;
};

static void key(Probe& pr, const char* k) {
    printf("%s\"%s\": ", pr.first ? "" : ", ", k);
    pr.first = false;
}

template <class F>
static int time_ms(F launch, float* ms) {
    cudaEvent_t t0, t1;
    CK(cudaEventCreate(&t0));
    CK(cudaEventCreate(&t1));
    launch(true);  // short warm-up launch
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    CK(cudaEventRecord(t0));
    launch(false);
    CK(cudaEventRecord(t1));
    CK(cudaEventSynchronize(t1));
    CK(cudaGetLastError());
    CK(cudaEventElapsedTime(ms, t0, t1));
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    return 0;
}

template <int P>
static int run_warp(Probe& pr, const char* name, double macs_per_mma) {
    const int blocks = pr.prop.multiProcessorCount * 8, threads = 128, rounds = 3000;
    float ms = 0;
    if (time_ms([&](bool warm) { warp_mma_rate<P><<<blocks, threads>>>(0x1234567u, warm ? 8 : rounds, pr.sink); },
                &ms))
        return 1;
    const double warps = blocks * threads / 32.0;
    key(pr, name);
    printf("%.1f", 2.0 * warps * rounds * CHAINS * macs_per_mma / ms / 1e9);
    return 0;
}

static int run_popc(Probe& pr) {
    const int blocks = pr.prop.multiProcessorCount * 8, threads = 128, rounds = 12000;
    float ms = 0;
    if (time_ms([&](bool warm) { popc_rate<<<blocks, threads>>>(0xBEEFu, warm ? 8 : rounds, pr.sink); }, &ms))
        return 1;
    key(pr, "popc_bit_tops");
    printf("%.1f", 2.0 * blocks * threads * (double)rounds * CHAINS * 2 * 32 / ms / 1e9);
    return 0;
}

template <int P, int TC_N = 256>
static int run_tc(Probe& pr, const char* name, uint32_t a_word, uint32_t b_word, double per_mma_product) {
    CK(cudaFuncSetAttribute(tc_rate<P, TC_N>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    const int iters = 60000;  // 60000 x 4 x 64 < 2^24: exact in fp32
    const int kmma = P == TC_F8 ? 32 : 64;
    const int sms = pr.prop.multiProcessorCount;
    CK(cudaMemset(pr.err, 0, 4));
    float ms = 0;
    auto launch = [&](bool warm) {
        const int it = warm ? 100 : iters;
        tc_rate<P, TC_N><<<sms, 128, TC_SMEM>>>(it, a_word, b_word, (float)(per_mma_product * it * 4 * kmma), pr.err);
    };
    if (time_ms(launch, &ms)) return 1;
    int herr = 0;
    CK(cudaMemcpy(&herr, pr.err, 4, cudaMemcpyDeviceToHost));
    const double macs = (double)sms * iters * 4 * ((double)TC_M * TC_N * kmma);
    key(pr, name);
    printf("%.1f", 2 * macs / ms / 1e9);
    char ek[64];
    snprintf(ek, sizeof ek, "%s_check", name);
    key(pr, ek);
    printf("\"%s\"", herr == 0 ? "exact" : (herr & 4) ? "timeout" : "mismatch");
    return 0;
}

static bool want(int argc, char** argv, const char* name) {
    if (argc < 2) return true;
    for (int i = 1; i < argc; i++)
        if (!strcmp(argv[i], name)) return true;
    return false;
}

int main(int argc, char** argv) {
    Probe pr;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaGetDeviceProperties(&pr.prop, dev));
    CK(cudaMalloc(&pr.sink, (size_t)pr.prop.multiProcessorCount * 8 * 128 * 4));
    CK(cudaMalloc(&pr.err, 4));
    printf("{");
    key(pr, "gpu");
    printf("\"%s\"", pr.prop.name);
    key(pr, "sm");
    printf("%d%d", pr.prop.major, pr.prop.minor);
    key(pr, "sms");
    printf("%d", pr.prop.multiProcessorCount);
    int rc = 0;
    if (!rc && want(argc, argv, "b1")) rc = run_warp<W_B1>(pr, "b1_mma_sync_tops", 16.0 * 8 * 256);
    if (!rc && want(argc, argv, "s8")) rc = run_warp<W_S8>(pr, "s8_mma_sync_tops", 16.0 * 8 * 32);
    if (!rc && want(argc, argv, "e4m3")) rc = run_warp<W_E4M3>(pr, "e4m3_mma_sync_tflops", 16.0 * 8 * 32);
    if (!rc && want(argc, argv, "popc")) rc = run_popc(pr);
    // fp8: +1.0 (0x38) against -1.0 (0xB8); fp4: packed pairs of +1.0 (0x22)
    // against pairs of -1.0 (0xAA)
    if (!rc && want(argc, argv, "tc_f8")) rc = run_tc<TC_F8>(pr, "tc_f8_tflops", 0x38383838u, 0xB8B8B8B8u, -1.0);
    if (!rc && want(argc, argv, "tc_f4")) rc = run_tc<TC_F4>(pr, "tc_f4_tflops", 0x22222222u, 0xAAAAAAAAu, -1.0);
    // the tile shape of the contraction kernel (M128 N224); run alone: tch-peak tc_f4_n224
    if (!rc && argc > 1 && want(argc, argv, "tc_f4_n224"))
        rc = run_tc<TC_F4, 224>(pr, "tc_f4_n224_tflops", 0x22222222u, 0xAAAAAAAAu, -1.0);
    // kind::mxf4nvf4 (not in the default set: tch-peak tc_nvf4_32 / tc_nvf4_16)
    if (!rc && argc > 1 && want(argc, argv, "tc_nvf4_32"))
        rc = run_tc<TC_NVF4_32>(pr, "tc_nvf4_32_tflops", 0x22222222u, 0xAAAAAAAAu, -1.0);
    if (!rc && argc > 1 && want(argc, argv, "tc_nvf4_16"))
        rc = run_tc<TC_NVF4_16>(pr, "tc_nvf4_16_tflops", 0x22222222u, 0xAAAAAAAAu, -1.0);
    printf("}\n");
    return rc;
}
