/*
 * CPU oracle for the exact cgMLST Hamming distance path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library or CLI links or
 * calls this file; tests, the smoke check and the CPU-baseline leg of the
 * benchmark use it as the oracle.
 *
 * It restates the reference's brute-force count, which is the definition
 * every GPU result is compared with:
 *
 *   H[i][j] = sum_k [x_ik != x_jk] [x_ik != 0] [x_jk != 0]
 *
 *   - tensorcore/rs/check.py:39-44      (numpy `ref`, the end-to-end check)
 *   - tensorcore/tc_hamming.cu:244-247  (scalar C spot check of the prototype)
 *
 * x holds dense per-locus ranks (u16, 0 = missing).  Any injective map of the
 * allele ids that keeps 0 = missing gives the same H, so the rank order does
 * not matter here.
 *
 * The rolling checksum restates tensorcore/tc_hamming.cu:240-241 (and
 * cuda/bench.cu:14-19): h = h * 1000003 + H[i][j] over the upper triangle
 * (j > i) in row-major order, modulo 2^64.  The reference publishes
 * 85724a9d7d090f9f for its synthetic 30 000 x 5 000 profiles
 * (tensorcore/README.md:52).
 *
 * Portable C (no intrinsics): the inner loop is written so that gcc
 * vectorises it on x86-64 and on aarch64 alike.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Distance of one pair: the count of check.py:43 for a single (i, j). The u16
 * accumulator is exact because the result is at most L <= 65535. */
static inline uint16_t pair_dist(const uint16_t* restrict a, const uint16_t* restrict b, int64_t L) {
    uint16_t d = 0;
    for (int64_t k = 0; k < L; k++) d += (uint16_t)((a[k] != b[k]) & (a[k] != 0) & (b[k] != 0));
    return d;
}

static int pick_threads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

int orc_num_threads(void) { return pick_threads(0); }

/*
 * out[(i - i0) * ldo + (j - j0)] = H[i][j] for i in [i0, i1), j in [j0, j1).
 * Blocked over (row, column) tiles so a tile's profiles stay in cache.
 */
void orc_hamming_block(const uint16_t* x, int64_t n, int64_t L, int64_t i0, int64_t i1, int64_t j0,
                       int64_t j1, uint16_t* out, int64_t ldo, int threads) {
    (void)n;
    const int64_t TI = 16, TJ = 64;
    const int64_t nti = (i1 - i0 + TI - 1) / TI, ntj = (j1 - j0 + TJ - 1) / TJ;
    const int nt = pick_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t t = 0; t < nti * ntj; t++) {
        const int64_t bi = i0 + (t / ntj) * TI, bj = j0 + (t % ntj) * TJ;
        const int64_t ei = bi + TI < i1 ? bi + TI : i1, ej = bj + TJ < j1 ? bj + TJ : j1;
        for (int64_t i = bi; i < ei; i++) {
            const uint16_t* a = x + i * L;
            for (int64_t j = bj; j < ej; j++) out[(i - i0) * ldo + (j - j0)] = pair_dist(a, x + j * L, L);
        }
    }
}

/* The same count on raw allele ids (u64, 0 = missing): equality of ids is
 * what the ranks encode, so this equals orc_hamming_block on the ranks of x,
 * without ranking a large matrix first. */
static inline uint16_t pair_dist_u64(const uint64_t* restrict a, const uint64_t* restrict b, int64_t L) {
    uint16_t d = 0;
    for (int64_t k = 0; k < L; k++) d += (uint16_t)((a[k] != b[k]) & (a[k] != 0) & (b[k] != 0));
    return d;
}

void orc_hamming_block_u64(const uint64_t* x, int64_t n, int64_t L, int64_t i0, int64_t i1, int64_t j0,
                           int64_t j1, uint16_t* out, int64_t ldo, int threads) {
    (void)n;
    const int64_t TI = 8, TJ = 64;
    const int64_t nti = (i1 - i0 + TI - 1) / TI, ntj = (j1 - j0 + TJ - 1) / TJ;
    const int nt = pick_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t t = 0; t < nti * ntj; t++) {
        const int64_t bi = i0 + (t / ntj) * TI, bj = j0 + (t % ntj) * TJ;
        const int64_t ei = bi + TI < i1 ? bi + TI : i1, ej = bj + TJ < j1 ? bj + TJ : j1;
        for (int64_t i = bi; i < ei; i++) {
            const uint64_t* a = x + i * L;
            for (int64_t j = bj; j < ej; j++) out[(i - i0) * ldo + (j - j0)] = pair_dist_u64(a, x + j * L, L);
        }
    }
}

/* Upper-triangle pairs only: rows [i0, i1), columns j in (i, n). Returns the
 * number of pairs evaluated; the distances are folded into *sum so the work
 * cannot be optimised away. This is the CPU baseline's unit of work. */
int64_t orc_upper_rows(const uint16_t* x, int64_t n, int64_t L, int64_t i0, int64_t i1, uint64_t* sum,
                       int threads) {
    const int nt = pick_threads(threads);
    uint64_t total = 0;
    int64_t pairs = 0;
    const int64_t TJ = 256;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total, pairs) num_threads(nt)
    for (int64_t t = 0; t < (i1 - i0) * ((n + TJ - 1) / TJ); t++) {
        const int64_t ntj = (n + TJ - 1) / TJ;
        const int64_t i = i0 + t / ntj, bj = (t % ntj) * TJ;
        int64_t ej = bj + TJ < n ? bj + TJ : n;
        int64_t sj = bj > i + 1 ? bj : i + 1;
        const uint16_t* a = x + i * L;
        for (int64_t j = sj; j < ej; j++) {
            total += pair_dist(a, x + j * L, L);
            pairs++;
        }
    }
    if (sum) *sum = total;
    return pairs;
}

/* The same count over the rows i0, i0 + step, i0 + 2 step, ... below n: a
 * sample spread over the whole triangle (step consecutive offsets cover every
 * row once).  Returns the pairs evaluated; *sum as above. */
int64_t orc_upper_rows_step(const uint16_t* x, int64_t n, int64_t L, int64_t i0, int64_t step, uint64_t* sum,
                            int threads) {
    const int nt = pick_threads(threads);
    uint64_t total = 0;
    int64_t pairs = 0;
    const int64_t TJ = 256, ntj = (n + TJ - 1) / TJ;
    const int64_t rows = i0 < n && step > 0 ? (n - i0 + step - 1) / step : 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total, pairs) num_threads(nt)
    for (int64_t t = 0; t < rows * ntj; t++) {
        const int64_t i = i0 + (t / ntj) * step, bj = (t % ntj) * TJ;
        const int64_t ej = bj + TJ < n ? bj + TJ : n;
        const int64_t sj = bj > i + 1 ? bj : i + 1;
        const uint16_t* a = x + i * L;
        for (int64_t j = sj; j < ej; j++) {
            total += pair_dist(a, x + j * L, L);
            pairs++;
        }
    }
    if (sum) *sum = total;
    return pairs;
}

/* Rolling checksum of tc_hamming.cu:240-241 over one stripe buffer laid out
 * like the tch_run callback: rows x w, row stride ld, column c <-> j = r0 + c;
 * only c > r is part of the upper triangle. */
uint64_t orc_rollhash_stripe(uint64_t h, const uint16_t* s, int64_t rows, int64_t w, int64_t ld) {
    for (int64_t r = 0; r < rows; r++)
        for (int64_t c = r + 1; c < w; c++) h = h * 1000003ull + s[r * ld + c];
    return h;
}

/* Rolling checksum of the whole upper triangle straight from the ranks,
 * computing the distances block-row by block-row (parallel) and hashing them
 * in order (sequential). */
uint64_t orc_rollhash_ranks(const uint16_t* x, int64_t n, int64_t L, int threads) {
    const int64_t RB = 64;
    uint16_t* buf = (uint16_t*)malloc((size_t)RB * (size_t)(n > 0 ? n : 1) * sizeof(uint16_t));
    uint64_t h = 0;
    if (!buf) return 0;
    for (int64_t r0 = 0; r0 < n; r0 += RB) {
        const int64_t rows = r0 + RB < n ? RB : n - r0;
        orc_hamming_block(x, n, L, r0, r0 + rows, r0, n, buf, n - r0, threads);
        h = orc_rollhash_stripe(h, buf, rows, n - r0, n - r0);
    }
    free(buf);
    return h;
}
