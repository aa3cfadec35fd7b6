// tch-peak: throughput of the instruction paths the contraction kernels can
// use on this GPU, measured with register-only loops (the idea of the
// reference's tensorcore/peak.cu:8-37, extended to the paths GB300 offers).
//
//   b1    mma.sync m16n8k256 b1 AND+popc      (the reference's tensor path)
//   s8    mma.sync m16n8k32 s8 -> s32          (legacy int8 warp MMA)
//   e4m3  mma.sync m16n8k32 e4m3 -> f32        (legacy fp8 warp MMA)
//   popc  LOP3 AND + POPC + IADD on CUDA cores (32 bit-MACs per instruction)
//   tc_f8 tcgen05.mma kind::f8f6f4 M128 N256 K32 from shared memory into TMEM
//         (one CTA per SM, one issuing thread)
//
// Prints one JSON object; ops count 2 per bit/element MAC like peak.cu:36.

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "tc_ptx.cuh"

using namespace tch::ptx;

#define CK(x)                                                                                \
    do {                                                                                     \
        cudaError_t e_ = (x);                                                                \
        if (e_ != cudaSuccess) {                                                             \
            fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));                         \
            return 1;                                                                        \
        }                                                                                    \
    } while (0)

__global__ void k_b1(int iters, int* out) {
    uint32_t a0 = threadIdx.x * 2654435761u, a1 = a0 ^ 0x9e3779b9u, a2 = a0 * 3u, a3 = a0 + 7u;
    uint32_t b0 = a1 * 5u, b1 = a2 ^ 0x55555555u;
    int c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
            asm volatile("mma.sync.aligned.m16n8k256.row.col.s32.b1.b1.s32.and.popc "
                         "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                         : "+r"(c0), "+r"(c1), "+r"(c2), "+r"(c3)
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
    if (c0 + c1 + c2 + c3 == 42) out[0] = 1;
}

__global__ void k_s8(int iters, int* out) {
    uint32_t a0 = threadIdx.x * 2654435761u, a1 = a0 ^ 0x9e3779b9u, a2 = a0 * 3u, a3 = a0 + 7u;
    uint32_t b0 = a1 * 5u, b1 = a2 ^ 0x55555555u;
    int c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
            asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 "
                         "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                         : "+r"(c0), "+r"(c1), "+r"(c2), "+r"(c3)
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
    if (c0 + c1 + c2 + c3 == 42) out[0] = 1;
}

__global__ void k_e4m3(int iters, int* out) {
    // operands: bytes 0x38 (+1.0) / 0x00, so accumulators stay small integers
    uint32_t a0 = (threadIdx.x & 1) ? 0x38003800u : 0x00380038u, a1 = a0, a2 = a0 ^ 0x38383838u, a3 = a0;
    uint32_t b0 = 0x38383838u, b1 = a0;
    float c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
            asm volatile("mma.sync.aligned.m16n8k32.row.col.f32.e4m3.e4m3.f32 "
                         "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                         : "+f"(c0), "+f"(c1), "+f"(c2), "+f"(c3)
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
    if (c0 + c1 + c2 + c3 == 42.f) out[0] = 1;
}

__global__ void k_popc(int iters, int* out) {
    uint32_t a[4], b[4];
    for (int q = 0; q < 4; q++) {
        a[q] = (threadIdx.x + q) * 2654435761u;
        b[q] = (threadIdx.x ^ q) * 0x9e3779b9u;
    }
    int acc[4][4] = {};
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[p][q] += __popc(a[p] & b[q]);
#pragma unroll
        for (int q = 0; q < 4; q++) {  // keep the operands live and changing
            a[q] = a[q] * 1664525u + 1013904223u;
            b[q] ^= a[q];
        }
    }
    int s = 0;
    for (int p = 0; p < 4; p++)
        for (int q = 0; q < 4; q++) s += acc[p][q];
    if (s == 42) out[0] = 1;
}


// tcgen05 fp8 MMA issue rate: operands (zeros) in shared memory, one
// accumulator in TMEM, a bounded wait for completion at the end.
constexpr int TC_SMEM = 120 * 1024;  // keeps one CTA per SM
__global__ void __launch_bounds__(128, 1) k_tc_f8(int iters, int* err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* A = smem;                 // 128 rows x 128 B
    uint8_t* B = smem + 16384;         // 256 rows x 128 B
    uint64_t* bar = (uint64_t*)(smem + 49152);
    uint32_t* slot = (uint32_t*)(bar + 1);
    volatile int* abort_flag = (volatile int*)(slot + 1);
    for (int i = threadIdx.x; i < 49152 / 16; i += blockDim.x) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // operand writes -> tensor-core reads
    if (threadIdx.x / 32 == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    if (threadIdx.x == 0) {
        const uint32_t idesc = make_idesc(1, 0, 0, 128, 256);
        const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
        for (int i = 0; i < iters; i++)
#pragma unroll
            for (int k = 0; k < 4; k++)
                tc_mma_f8(tmem, sw128_desc(a0 + 32 * k), sw128_desc(b0 + 32 * k), idesc, (i | k) ? 1u : 0u);
        tc_commit(bar);
        mbar_wait(bar, 0, abort_flag, err);
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x / 32 == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
}

template <class K>
static int timed(K kern, int blocks, int threads, int iters, int* out, float* ms) {
    cudaEvent_t t0, t1;
    CK(cudaEventCreate(&t0));
    CK(cudaEventCreate(&t1));
    kern<<<blocks, threads>>>(16, out);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    CK(cudaEventRecord(t0));
    kern<<<blocks, threads>>>(iters, out);
    CK(cudaEventRecord(t1));
    CK(cudaEventSynchronize(t1));
    CK(cudaGetLastError());
    CK(cudaEventElapsedTime(ms, t0, t1));
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    return 0;
}

int main() {
    int dev = 0;
    cudaDeviceProp p;
    CK(cudaGetDevice(&dev));
    CK(cudaGetDeviceProperties(&p, dev));
    int* out;
    CK(cudaMalloc(&out, 4));
    const int blocks = p.multiProcessorCount * 8, threads = 128, iters = 4000;
    const double warps = blocks * threads / 32.0;
    float ms;
    printf("{\"gpu\": \"%s\", \"sm\": %d%d, \"sms\": %d", p.name, p.major, p.minor, p.multiProcessorCount);
    if (timed(k_b1, blocks, threads, iters, out, &ms)) return 1;
    printf(", \"b1_mma_sync_tops\": %.1f", warps * iters * 8 * (16.0 * 8 * 256) * 2 / ms / 1e9);
    if (timed(k_s8, blocks, threads, iters, out, &ms)) return 1;
    printf(", \"s8_mma_sync_tops\": %.1f", warps * iters * 8 * (16.0 * 8 * 32) * 2 / ms / 1e9);
    if (timed(k_e4m3, blocks, threads, iters, out, &ms)) return 1;
    printf(", \"e4m3_mma_sync_tflops\": %.1f", warps * iters * 8 * (16.0 * 8 * 32) * 2 / ms / 1e9);
    if (timed(k_popc, blocks, threads, iters, out, &ms)) return 1;
    printf(", \"popc_bit_tops\": %.1f", blocks * (double)threads * iters * 16 * 32.0 * 2 / ms / 1e9);
    {
        int* err;
        CK(cudaMalloc(&err, 4));
        CK(cudaMemset(err, 0, 4));
        CK(cudaFuncSetAttribute(k_tc_f8, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
        cudaEvent_t t0, t1;
        CK(cudaEventCreate(&t0));
        CK(cudaEventCreate(&t1));
        const int tc_iters = 60000;
        k_tc_f8<<<p.multiProcessorCount, 128, TC_SMEM>>>(100, err);
        CK(cudaGetLastError());
        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(t0));
        k_tc_f8<<<p.multiProcessorCount, 128, TC_SMEM>>>(tc_iters, err);
        CK(cudaEventRecord(t1));
        CK(cudaEventSynchronize(t1));
        CK(cudaGetLastError());
        CK(cudaEventElapsedTime(&ms, t0, t1));
        int herr = 0;
        CK(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost));
        const double macs = (double)p.multiProcessorCount * tc_iters * 4 * (128.0 * 256 * 32);
        printf(", \"tc_f8_tflops\": %.1f, \"tc_f8_err\": %d", 2 * macs / ms / 1e9, herr);
    }
    printf("}\n");
    return 0;
}
