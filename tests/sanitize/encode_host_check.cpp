// The host encoder (csrc/encode_host.cpp: tch_dense_ranks, tch_choose_tau,
// tch_encode_host) built with AddressSanitizer and UBSan, on random sets, with
// the rare-pair CSR checked against a direct count: n_rare equals the number
// of equal non-missing pairs of alleles seen fewer than tau times (at least
// twice), every partner j is in (i, n), and each row's partners do not
// decrease.  Prints "encode_host ok" and exits 0 when every check holds.
#include <cstdio>
#include <random>
#include <vector>

#include "tch.h"

int main() {
    std::mt19937_64 rng(5);
    for (int trial = 0; trial < 12; trial++) {
        const int n = 1 + (int)(rng() % 700), L = 1 + (int)(rng() % 90);
        std::vector<uint64_t> calls((size_t)n * L);
        for (auto& v : calls) v = (rng() % 7 == 0) ? 0 : (rng() % (trial % 3 == 0 ? 5 : 400)) + 1;
        std::vector<uint16_t> x((size_t)n * L);
        std::vector<uint32_t> nd(L);
        char err[256];
        for (int threads : {1, 5}) {
            if (tch_dense_ranks(calls.data(), n, L, x.data(), nd.data(), threads, err, sizeof err)) {
                printf("ranks: %s\n", err);
                return 1;
            }
            int tau = 0;
            if (tch_choose_tau(x.data(), nd.data(), n, L, 64, (size_t)1 << 34, 5.9e14, 3.5e9, 0, &tau, err,
                               sizeof err)) {
                printf("tau: %s\n", err);
                return 1;
            }
            for (int t : {tau, 1, 2, 1 << 20}) {
                tch_host_encoding e;
                if (tch_encode_host(x.data(), nd.data(), n, L, t, threads, &e, err, sizeof err)) {
                    printf("encode: %s\n", err);
                    return 1;
                }
                size_t want = 0;
                for (int k = 0; k < L; k++) {
                    std::vector<size_t> c(nd[k] + 1, 0);
                    for (int i = 0; i < n; i++) c[x[(size_t)i * L + k]]++;
                    for (uint32_t r = 1; r <= nd[k]; r++)
                        if ((int)c[r] < t && c[r] >= 2) want += c[r] * (c[r] - 1) / 2;
                }
                const size_t got = e.n_rare;
                bool ok = got == want && e.start[n] == want;
                for (int i = 0; ok && i < n; i++)
                    for (uint32_t p = e.start[i]; ok && p < e.start[i + 1]; p++)
                        ok = e.js[p] > (uint32_t)i && e.js[p] < (uint32_t)n && (p == e.start[i] || e.js[p - 1] <= e.js[p]);
                tch_host_encoding_free(&e);
                if (!ok) {
                    printf("trial %d tau %d threads %d: CSR wrong (n_rare %zu, want %zu)\n", trial, t, threads,
                           got, want);
                    return 1;
                }
            }
        }
    }
    printf("encode_host ok\n");
    return 0;
}
