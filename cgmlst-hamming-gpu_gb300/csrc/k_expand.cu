// Bit rows (reference layout, LSB first) -> byte rows for the tensor-core
// kernels: X[row] = [presence bytes (kp) | one-hot bytes (kb - kp)], each
// element 0 or the encoding of +1 (one) / -1 (one_neg, one-hot part only).
// The rows may be split along K into separate allocations (KChunks).
// HBM-bound: each thread reads 2 bytes of bits and writes 16 bytes.

#include "tch_internal.cuh"

namespace tch {
namespace {

__global__ void expand_bits_kernel(const uint8_t* __restrict__ Pb, int pbytes, const uint8_t* __restrict__ Ob,
                                   int obytes, int n, size_t n_rows, KChunks X, int kp, int kpres, int konehot,
                                   uint8_t one, uint8_t one_o) {
    const size_t chunks_per_row = (size_t)X.kb / 16;
    const size_t total = n_rows * chunks_per_row;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t row = t / chunks_per_row;
        const int c0 = (int)(t % chunks_per_row) * 16;  // first byte column of this 16-byte group
        uint32_t bits = 0;
        bool onehot = c0 >= kp;
        if (row < (size_t)n) {
            const int k = onehot ? c0 - kp : c0;  // bit index inside its part (multiple of 16)
            const int limit = onehot ? konehot : kpres;
            const uint8_t* src = onehot ? Ob + row * (size_t)obytes : Pb + row * (size_t)pbytes;
            if (k < limit) bits = (uint32_t)src[k >> 3] | ((uint32_t)src[(k >> 3) + 1] << 8);
        }
        const uint8_t v = onehot ? one_o : one;
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            uint32_t x = 0;
#pragma unroll
            for (int b = 0; b < 4; b++) x |= (uint32_t)(((bits >> (q * 4 + b)) & 1u) ? v : 0) << (8 * b);
            w[q] = x;
        }
        // chunk widths are multiples of 128 bytes, so a 16-byte group never straddles two
        *reinterpret_cast<uint4*>(X.at(row, c0)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

}  // namespace

cudaError_t launch_expand_bits_chunked(const BitOperands& bits, int n, size_t n_rows, const KChunks& X, int kp,
                                       int k_presence_bits, int k_onehot_bits, uint8_t one, uint8_t one_neg,
                                       cudaStream_t st) {
    if ((X.kb % 16) || (kp % 16) || (X.width % 16) || X.n < 1) return cudaErrorInvalidValue;
    const size_t total = n_rows * (size_t)(X.kb / 16);
    if (!total) return cudaSuccess;
    int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)152 * 16);
    expand_bits_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const uint8_t*>(bits.P), bits.wP * 4,
                                               reinterpret_cast<const uint8_t*>(bits.O), bits.wO * 4, n, n_rows, X, kp,
                                               k_presence_bits, k_onehot_bits, one, one_neg);
    return cudaGetLastError();
}

cudaError_t launch_expand_bits(const BitOperands& bits, int n, size_t n_rows, uint8_t* X, int kb, int kp,
                               int k_presence_bits, int k_onehot_bits, uint8_t one, uint8_t one_neg,
                               cudaStream_t st) {
    KChunks one_chunk;
    one_chunk.p[0] = X;
    one_chunk.n = 1;
    one_chunk.width = kb;
    one_chunk.kb = kb;
    return launch_expand_bits_chunked(bits, n, n_rows, one_chunk, kp, k_presence_bits, k_onehot_bits, one, one_neg,
                                      st);
}

}  // namespace tch
