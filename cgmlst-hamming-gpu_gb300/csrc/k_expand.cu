// The packed e2m1 operand rows of the tile pass: allocation (split along K),
// expansion from tch_run's bit rows, and the negated one-hot copy.
//
// Bits (reference layout, LSB first, u32 words) -> rows [presence | one-hot |
// zeros] of 4-bit elements: each 32-bit input word becomes 16 output bytes,
// bit k of the word the element at column 32 w + k.  HBM-bound: a thread
// reads one word and writes 16 bytes to each of the two copies.

#include "tch_internal.cuh"

namespace tch {
namespace {

// 32 bits -> 4 words of nibbles (0 or `v` per bit).
__device__ __forceinline__ uint4 nibbles(uint32_t bits, uint32_t v) {
    return make_uint4(spread_nibbles(bits) * v, spread_nibbles(bits >> 8) * v, spread_nibbles(bits >> 16) * v,
                      spread_nibbles(bits >> 24) * v);
}

__global__ void expand_bits_kernel(const uint32_t* __restrict__ P, int wP, const uint32_t* __restrict__ O, int wO,
                                   int n, int wp, int wo, KChunks pos, KChunks neg, size_t n_rows) {
    const size_t groups = (size_t)pos.kb / 16;  // 16-byte groups (32 columns) per row
    const size_t total = n_rows * groups;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t row = t / groups;
        const int g = (int)(t % groups);
        uint32_t bits = 0;
        bool onehot = false;
        if (row < (size_t)n) {
            if (g < wp) bits = P[row * wP + g];
            else if (g < wp + wo) bits = O[row * wO + (g - wp)], onehot = true;
        }
        // chunk widths are multiples of 128 bytes: a 16-byte group never straddles two
        *reinterpret_cast<uint4*>(pos.at(row, 16 * g)) = nibbles(bits, kFp4One);
        *reinterpret_cast<uint4*>(neg.at(row, 16 * g)) = nibbles(bits, onehot ? kFp4MinusOne : kFp4One);
    }
}

// Highest word index (+1) holding a set bit, over all rows, for P and O.
__global__ void used_words_kernel(const uint32_t* __restrict__ P, int wP, const uint32_t* __restrict__ O, int wO,
                                  size_t n_pad, int* out) {
    const size_t tp = n_pad * wP, to = n_pad * wO;
    int mp = 0, mo = 0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tp + to; t += (size_t)gridDim.x * blockDim.x) {
        if (t < tp) {
            if (P[t]) mp = max(mp, (int)(t % wP) + 1);
        } else if (O[t - tp]) {
            mo = max(mo, (int)((t - tp) % wO) + 1);
        }
    }
    for (int o = 16; o; o >>= 1) {
        mp = max(mp, __shfl_xor_sync(0xFFFFFFFFu, mp, o));
        mo = max(mo, __shfl_xor_sync(0xFFFFFFFFu, mo, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, mp);
        atomicMax(out + 1, mo);
    }
}

// neg = pos with every non-zero element at column >= kp turned to -1.0:
// +1.0 is 0x2 (bit 1 of the nibble), -1.0 adds the sign bit 3.
__global__ void negate_onehot_kernel(KChunks pos, KChunks neg, size_t n_rows, int kp) {
    const size_t groups = (size_t)pos.kb / 16;
    const size_t total = n_rows * groups;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t row = t / groups;
        const int g = (int)(t % groups);
        uint4 v = *reinterpret_cast<const uint4*>(pos.at(row, 16 * g));
        uint32_t* w = reinterpret_cast<uint32_t*>(&v);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int c0 = 32 * g + 8 * q;  // column of the word's first element
            // nibble positions at columns >= kp
            const uint32_t m = c0 >= kp ? 0xFFFFFFFFu : (c0 + 8 <= kp ? 0u : 0xFFFFFFFFu << (4 * (kp - c0)));
            w[q] |= (w[q] << 2) & 0x88888888u & m;
        }
        *reinterpret_cast<uint4*>(neg.at(row, 16 * g)) = v;
    }
}

int grid_of(size_t total) { return (int)std::min<size_t>((total + 255) / 256, (size_t)152 * 16); }

}  // namespace

cudaError_t alloc_fp4(Fp4Operands* X, size_t n_rows, int kb, size_t max_chunk, bool pos, bool neg, size_t* bytes) {
    const int w = chunk_width_for(kb, n_rows, max_chunk);
    if (!w || kb <= 0 || (kb % 128)) return cudaErrorInvalidValue;
    X->n_rows = n_rows;
    X->kb = kb;
    for (KChunks* k : {&X->pos, &X->neg}) {
        k->kb = kb;
        k->width = w;
        k->n = (kb + w - 1) / w;
    }
    for (int side = 0; side < 2; side++) {
        if (!(side ? neg : pos)) continue;
        KChunks& k = side ? X->neg : X->pos;
        for (int c = 0; c < k.n; c++) {
            const size_t b = n_rows * (size_t)k.width_of(c);
            const cudaError_t e = cudaMalloc(&k.p[c], std::max<size_t>(b, 16));
            if (e != cudaSuccess) return e;
            if (bytes) *bytes += b;
        }
    }
    return cudaSuccess;
}

void free_fp4(Fp4Operands* X) {
    for (KChunks* k : {&X->pos, &X->neg})
        for (int c = 0; c < kMaxKChunks; c++) {
            if (k->p[c]) cudaFree(k->p[c]);
            k->p[c] = nullptr;
        }
}

cudaError_t launch_expand_bits(const BitOperands& bits, int n, int wp, int wo, const Fp4Operands& X,
                               cudaStream_t st) {
    if (X.kb % 128 || wp < 0 || wo < 0 || (size_t)32 * (wp + wo) > (size_t)X.kb * 2) return cudaErrorInvalidValue;
    const size_t total = X.n_rows * (size_t)(X.kb / 16);
    if (!total) return cudaSuccess;
    expand_bits_kernel<<<grid_of(total), 256, 0, st>>>(bits.P, bits.wP, bits.O, bits.wO, n, wp, wo, X.pos, X.neg,
                                                       X.n_rows);
    return cudaGetLastError();
}

cudaError_t used_bit_words(const BitOperands& bits, size_t n_pad, int* wp, int* wo, cudaStream_t st) {
    int* d = nullptr;
    int h[2] = {0, 0};
    cudaError_t e = cudaMalloc(&d, 8);
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, 8, st);
    const size_t total = n_pad * (size_t)(bits.wP + bits.wO);
    if (e == cudaSuccess && total) {
        used_words_kernel<<<grid_of(total), 256, 0, st>>>(bits.P, bits.wP, bits.O, bits.wO, n_pad, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (d) cudaFree(d);
    *wp = h[0];
    *wo = h[1];
    return e;
}

cudaError_t launch_negate_onehot(const Fp4Operands& X, int kp, cudaStream_t st) {
    const size_t total = X.n_rows * (size_t)(X.kb / 16);
    if (!total) return cudaSuccess;
    negate_onehot_kernel<<<grid_of(total), 256, 0, st>>>(X.pos, X.neg, X.n_rows, kp);
    return cudaGetLastError();
}

}  // namespace tch
