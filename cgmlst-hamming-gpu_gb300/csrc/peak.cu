// tch-peak: throughput of the instruction paths the contraction kernels can
// use on this GPU, measured with register-only loops (the idea of the
// reference's tensorcore/peak.cu:8-37, extended to the paths GB300 offers).
//
//   b1    mma.sync m16n8k256 b1 AND+popc      (the reference's tensor path)
//   s8    mma.sync m16n8k32 s8 -> s32          (legacy int8 warp MMA)
//   e4m3  mma.sync m16n8k32 e4m3 -> f32        (legacy fp8 warp MMA)
//   popc  LOP3 AND + POPC + IADD on CUDA cores (32 bit-MACs per instruction)
//
// Prints one JSON object; ops count 2 per bit/element MAC like peak.cu:36.

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

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
    printf("}\n");
    return 0;
}
