// tch-ranks: the whole distance matrix of a ranks file, the binary input the
// reference prototype reads (tensorcore/tc_hamming.cu:12-13, 111-117; written
// by tensorcore/to_ranks.py): int32 n, int32 L, then n x L u16 dense per-locus
// ranks, row-major, 0 = missing.
//
//     tch-ranks <ranks file> [tau=0 auto] [stripe rows=512] [noverify]
//
// Same arguments and the same consumer as the prototype (tc_hamming.cu:
// 198-253): every stripe is folded into the rolling checksum
// h = h * 1000003 + H[i][j] over the upper triangle in row order, with 4 spot
// checks per stripe against a direct count; "noverify" leaves the consumer
// empty.  The device work goes through libtch (tch_solver_from_ranks: the
// device encoder, then the tcgen05 stripe pipeline of tch_solver_run).

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <random>
#include <string>
#include <vector>

#include "tch.h"

namespace {

double now() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

struct Consumer {
    const std::vector<uint16_t>* x = nullptr;
    int n = 0, L = 0;
    bool verify = true;
    uint64_t h = 0;
    double secs = 0;
    bool ok = true;
    std::mt19937 rng{7};
};

void on_stripe(void* ctx, int r0, int rows, size_t w, const uint16_t* H) {
    Consumer* c = static_cast<Consumer*>(ctx);
    const double t = now();
    if (c->verify && c->ok) {
        for (int r = 0; r < rows; r++)
            for (size_t j = (size_t)r + 1; j < w; j++) c->h = c->h * 1000003u + H[(size_t)r * w + j];
        for (int s = 0; s < 4 && w > 1; s++) {  // spot checks against a direct count
            const int r = (int)(c->rng() % (unsigned)rows);
            if ((size_t)r + 1 >= w) continue;
            const size_t j = (size_t)r + 1 + c->rng() % (w - r - 1);
            const int i = r0 + r, jj = r0 + (int)j;
            int d = 0;
            for (int k = 0; k < c->L; k++) {
                const int a = (*c->x)[(size_t)i * c->L + k], b = (*c->x)[(size_t)jj * c->L + k];
                d += (a && b && a != b);
            }
            if (d != H[(size_t)r * w + j]) {
                fprintf(stderr, "MISMATCH i=%d j=%d gpu=%d ref=%d\n", i, jj, H[(size_t)r * w + j], d);
                c->ok = false;
            }
        }
    }
    c->secs += now() - t;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <ranks> [tau] [stripe] [noverify]\n", argv[0]);
        return 1;
    }
    const int tau = argc > 2 ? atoi(argv[2]) : 0;
    const int S = argc > 3 ? atoi(argv[3]) : 512;
    const bool verify = !(argc > 4 && std::string(argv[4]) == "noverify");
    const double t_all = now();
    FILE* f = fopen(argv[1], "rb");
    int32_t nl[2];
    if (!f || fread(nl, 4, 2, f) != 2) {
        perror("read");
        return 1;
    }
    const int n = nl[0], L = nl[1];
    if (n < 0 || L < 0) {
        fprintf(stderr, "bad header: n=%d L=%d\n", n, L);
        return 1;
    }
    if (L > 65535) {
        fprintf(stderr, "L > 65535 not supported (u16 output)\n");
        return 1;
    }
    std::vector<uint16_t> x((size_t)n * L);
    if (fread(x.data(), 2, x.size(), f) != x.size()) {
        perror("read");
        return 1;
    }
    fclose(f);
    if (tch_device_count() <= 0) {
        fprintf(stderr, "no CUDA device\n");
        return 1;
    }
    char err[1024];
    double t_enc = now();
    tch_solver* s = nullptr;
    if (tch_solver_from_ranks(0, n, L, x.data(), tau, TCH_KERNEL_AUTO, &s, err, sizeof err)) {
        fprintf(stderr, "CUDA: %s\n", err);
        return 1;
    }
    t_enc = now() - t_enc;
    tch_info info;
    tch_solver_info(s, &info);
    fprintf(stderr, "n=%d L=%d tau=%d: dense one-hot cols=%zu, rare equal pairs=%zu, encode %.2fs\n", n, L, info.tau,
            info.d_onehot, info.n_rare, t_enc);
    fprintf(stderr, "stripe %d rows, %s\n", S,
            verify ? "verifying (full checksum + spot checks)" : "noverify (consumer does nothing)");
    Consumer c;
    c.x = &x;
    c.n = n;
    c.L = L;
    c.verify = verify;
    double gpu = 0, t_pipe = now();
    if (n > 1 && tch_solver_run(s, S, on_stripe, &c, &gpu, err, sizeof err)) {
        fprintf(stderr, "CUDA: %s\n", err);
        tch_solver_destroy(s);
        return 1;
    }
    t_pipe = now() - t_pipe;
    tch_solver_destroy(s);
    if (!c.ok) return 2;
    printf("tch-ranks tau=%d: pipeline (GPU + D2H u16 + consumer) %.3f s, of which consumer %.2f s, encode %.2f s, "
           "total %.2f s  checksum=%llx\n",
           info.tau, t_pipe, c.secs, t_enc, now() - t_all, (unsigned long long)c.h);
    return 0;
}
