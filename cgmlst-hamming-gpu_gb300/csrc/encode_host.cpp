// Host encoder: the reference host's encoding stage in multi-threaded C++.
//
//   tch_dense_ranks   tensorcore/rs/src/main.rs:134-165
//   tch_choose_tau    main.rs:167-198 (rates are parameters: the reference's
//                     L4 constants reproduce its choice; measured GB300 rates
//                     give this library's)
//   tch_encode_host   main.rs:366-444 (frequent column map, LSB-first bit
//                     packing of O and P, rare equal pairs as CSR)
//
// The partner list of each row comes out ascending (the reference fills it
// with atomics in an unspecified order); that order lets the device subtract
// the rare pairs inside each output tile.

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "tch.h"

namespace {

int set_err(char* err, int errlen, const char* fmt, ...) {
    if (err && errlen > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)errlen, fmt, ap);
        va_end(ap);
    }
    return 1;
}

size_t up(size_t x, size_t m) { return (x + m - 1) / m * m; }

int nthreads(int t) {
    if (t > 0) return t;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

// Dynamic parallel loop over [0, count) in chunks.
template <class F>
void parallel_for(int threads, size_t count, size_t chunk, F&& f) {
    threads = nthreads(threads);
    if (threads <= 1 || count <= chunk) {
        for (size_t b = 0; b < count; b += chunk) f(b, std::min(count, b + chunk));
        return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
        pool.emplace_back([&] {
            for (;;) {
                const size_t b = next.fetch_add(chunk);
                if (b >= count) break;
                f(b, std::min(count, b + chunk));
            }
        });
    for (auto& th : pool) th.join();
}

// counts per (locus, rank), flattened: cnt[off[k] + a], a in 0..k_distinct
struct Counts {
    std::vector<size_t> off;
    std::vector<uint32_t> cnt;
};

// The ranks x (n x L) and the distinct counts nd (L) come from the caller:
// every nd[k] must be at most 65 535 and every rank at most its locus's
// nd[k] (tch_dense_ranks gives both), else the counters of a locus would be
// indexed past their range.  A violation is an error, not a count.
int count_ranks(const uint16_t* x, const uint32_t* nd, int n, int L, int threads, Counts& c, char* err,
                int errlen) {
    if ((size_t)n * L != 0 && !x) return set_err(err, errlen, "null ranks");
    if (L > 0 && !nd) return set_err(err, errlen, "null distinct counts");
    c.off.assign((size_t)L + 1, 0);
    for (int k = 0; k < L; k++) {
        if (nd[k] > 65535) return set_err(err, errlen, "locus %d: %u distinct alleles (limit 65535)", k, nd[k]);
        c.off[k + 1] = c.off[k] + nd[k] + 1;
    }
    c.cnt.assign(c.off[L], 0);
    std::atomic<long long> bad{-1};  // a cell i * L + k whose rank is above nd[k]
    // loci in blocks: each worker owns whole loci and walks rows in tiles
    parallel_for(threads, (size_t)L, 16, [&](size_t k0, size_t k1) {
        for (int i = 0; i < n; i++) {
            const uint16_t* row = x + (size_t)i * L;
            for (size_t k = k0; k < k1; k++) {
                if (row[k] > nd[k]) {
                    long long expect = -1;
                    bad.compare_exchange_strong(expect, (long long)i * L + (long long)k);
                    continue;
                }
                c.cnt[c.off[k] + row[k]]++;
            }
        }
    });
    const long long b = bad.load();
    if (b >= 0)
        return set_err(err, errlen, "row %lld, locus %lld: rank %u is above the locus's %u distinct alleles", b / L,
                       b % L, (unsigned)x[b], nd[b % L]);
    return 0;
}

}  // namespace

extern "C" {

int tch_dense_ranks(const uint64_t* calls, int n, int L, uint16_t* x, uint32_t* n_distinct, int threads,
                    char* err, int errlen) {
    if (n < 0 || L < 0) return set_err(err, errlen, "negative size");
    if ((size_t)n * L != 0 && (!calls || !x || !n_distinct)) return set_err(err, errlen, "null buffer");
    std::atomic<int> bad_locus{-1};
    std::atomic<size_t> bad_count{0};
    parallel_for(threads, (size_t)L, 1, [&](size_t kb, size_t ke) {
        std::vector<uint64_t> col((size_t)n), uniq;
        for (size_t k = kb; k < ke; k++) {
            uniq.clear();
            for (int i = 0; i < n; i++) {
                col[i] = calls[(size_t)i * L + k];
                if (col[i]) uniq.push_back(col[i]);
            }
            std::sort(uniq.begin(), uniq.end());
            uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
            if (uniq.size() > 65535) {
                int expect = -1;
                if (bad_locus.compare_exchange_strong(expect, (int)k)) bad_count = uniq.size();
                continue;
            }
            n_distinct[k] = (uint32_t)uniq.size();
            for (int i = 0; i < n; i++) {
                const uint64_t v = col[i];
                x[(size_t)i * L + k] =
                    v ? (uint16_t)(std::lower_bound(uniq.begin(), uniq.end(), v) - uniq.begin() + 1) : 0;
            }
        }
    });
    if (bad_locus >= 0)
        return set_err(err, errlen, "locus %d has %zu distinct alleles (limit 65535)", bad_locus.load(),
                       bad_count.load());
    return 0;
}

int tch_choose_tau(const uint16_t* x, const uint32_t* nd, int n, int L, int stripe, size_t free_bytes,
                   double gemm_rate, double rare_rate, int verbose, int* tau_out, char* err, int errlen) {
    if (!tau_out) return set_err(err, errlen, "null output");
    if (n < 0 || L < 0) return set_err(err, errlen, "negative size");
    Counts c;
    if (count_ranks(x, nd, n, L, 0, c, err, errlen)) return 1;
    std::vector<double> cs;
    cs.reserve(c.cnt.size());
    for (int k = 0; k < L; k++)
        for (size_t a = 1; a <= nd[k]; a++)
            if (c.cnt[c.off[k] + a]) cs.push_back((double)c.cnt[c.off[k] + a]);
    const size_t n_pad = up((size_t)n, 256);
    const double bufs = (double)((size_t)stripe * n_pad * 12 + ((size_t)64 << 20));
    int best = 0;
    double best_t = 1e300;
    for (int tau = 2; tau <= 4096; tau *= 2) {
        size_t d = 0;
        double r = 0;
        for (double v : cs) {
            if (v >= tau) d++;
            else r += v * (v - 1.0) / 2.0;
        }
        const size_t k1 = up(std::max<size_t>(d, 1), 1024);
        const double mem = (double)(n_pad * k1 / 8) + 4.0 * (r + n + 1.0) + bufs;
        const double t = (double)n * (double)n / 2.0 * (double)k1 / gemm_rate + r / rare_rate;
        const bool fits = mem <= (double)free_bytes && r < 4.0e9;
        if (verbose)
            fprintf(stderr, "  tau=%5d  one-hot=%8zu  rare=%14.0f  est %.3fs  vram %.2f GB%s\n", tau, d, r, t,
                    mem / 1e9, fits ? "" : "  (does not fit)");
        if (fits && t < best_t) {
            best = tau;
            best_t = t;
        }
    }
    if (!best) return set_err(err, errlen, "no tau fits in %.2f GB of free VRAM", (double)free_bytes / 1e9);
    *tau_out = best;
    return 0;
}

int tch_encode_host(const uint16_t* x, const uint32_t* nd, int n, int L, int tau, int threads,
                    tch_host_encoding* out, char* err, int errlen) {
    if (!out) return set_err(err, errlen, "null output");
    memset(out, 0, sizeof(*out));
    if (n < 0 || L < 0) return set_err(err, errlen, "negative size");
    if (tau < 1) return set_err(err, errlen, "tau must be >= 1");
    Counts c;
    if (count_ranks(x, nd, n, L, threads, c, err, errlen)) return 1;
    // frequent column of (locus, rank), -1 otherwise (main.rs:367-385)
    std::vector<int32_t> col(c.cnt.size(), -1);
    std::vector<size_t> base((size_t)L + 1, 0);
    for (int k = 0; k < L; k++) {
        size_t d = 0;
        for (size_t a = 1; a <= nd[k]; a++)
            if (c.cnt[c.off[k] + a] >= (uint32_t)tau) col[c.off[k] + a] = (int32_t)d++;
        base[k + 1] = base[k] + d;
    }
    const size_t D = base[L];
    const size_t n_pad = up((size_t)n, 256), K1 = up(std::max<size_t>(D, 1), 1024), K2 = up((size_t)L, 1024);
    out->n = n;
    out->L = L;
    out->tau = tau;
    out->D = D;
    out->n_pad = n_pad;
    out->K1 = K1;
    out->K2 = K2;
    out->O = (uint8_t*)calloc(std::max<size_t>(n_pad * K1 / 8, 1), 1);
    out->P = (uint8_t*)calloc(std::max<size_t>(n_pad * K2 / 8, 1), 1);
    out->start = (uint32_t*)calloc((size_t)n + 1, 4);
    if (!out->O || !out->P || !out->start) {
        tch_host_encoding_free(out);
        return set_err(err, errlen, "out of host memory");
    }
    // bit-pack (main.rs:389-403)
    parallel_for(threads, (size_t)n, 64, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; i++) {
            uint8_t* orow = out->O + i * (K1 / 8);
            uint8_t* prow = out->P + i * (K2 / 8);
            for (int k = 0; k < L; k++) {
                const int a = x[i * L + k];
                if (!a) continue;
                prow[k >> 3] |= (uint8_t)(1u << (k & 7));
                const int32_t cc = col[c.off[k] + a];
                if (cc >= 0) {
                    const size_t b = base[k] + (size_t)cc;
                    orow[b >> 3] |= (uint8_t)(1u << (b & 7));
                }
            }
        }
    });
    // rare groups per locus: rows sharing a rare allele with count >= 2 (main.rs:405-417)
    // group members are listed by (locus, rank) in ascending row order
    std::vector<size_t> goff(c.cnt.size() + 1, 0);
    for (int k = 0; k < L; k++)
        for (size_t a = 0; a <= nd[k]; a++) {  // slots q run over off[k] .. off[k+1]-1 in order
            const size_t q = c.off[k] + a;
            const bool rare = a > 0 && col[q] < 0 && c.cnt[q] >= 2;
            goff[q + 1] = goff[q] + (rare ? c.cnt[q] : 0);
        }
    std::vector<uint32_t> members(goff[c.cnt.size()]);
    {
        std::vector<size_t> fill(goff.begin(), goff.end() - 1);
        // locus-parallel, rows ascending inside each locus
        parallel_for(threads, (size_t)L, 8, [&](size_t k0, size_t k1) {
            for (int i = 0; i < n; i++)
                for (size_t k = k0; k < k1; k++) {
                    const int a = x[(size_t)i * L + k];
                    const size_t q = c.off[k] + a;
                    if (a && goff[q + 1] > goff[q]) members[fill[q]++] = (uint32_t)i;
                }
        });
    }
    // partners per row (main.rs:418-433): row i's partners at locus k are the
    // members of its group after its own entry (groups list rows ascending);
    // its place in a group is found by binary search
    auto own_place = [&](size_t g0, size_t g1, uint32_t i) {
        return (size_t)(std::lower_bound(members.begin() + g0, members.begin() + g1, i) - members.begin());
    };
    std::vector<uint64_t> rowcnt((size_t)n, 0);
    parallel_for(threads, (size_t)n, 64, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; i++) {
            uint64_t sum = 0;
            for (int k = 0; k < L; k++) {
                const int a = x[i * L + k];
                const size_t q = c.off[k] + a, g0 = goff[q], g1 = goff[q + 1];
                if (a && g1 > g0) sum += g1 - 1 - own_place(g0, g1, (uint32_t)i);
            }
            rowcnt[i] = sum;
        }
    });
    uint64_t n_rare = 0;
    for (int i = 0; i < n; i++) {
        out->start[i] = (uint32_t)n_rare;
        n_rare += rowcnt[i];
        if (n_rare >= (1ull << 32)) {
            tch_host_encoding_free(out);
            return set_err(err, errlen, "too many rare pairs: raise --tau");
        }
    }
    out->start[n] = (uint32_t)n_rare;
    out->n_rare = n_rare;
    out->js = (uint32_t*)malloc(std::max<size_t>(n_rare, 1) * 4);
    if (!out->js) {
        tch_host_encoding_free(out);
        return set_err(err, errlen, "out of host memory");
    }
    // each row's list, ascending, a partner repeated once per shared rare
    // allele: the row's partners are counted in a per-thread array over the
    // columns, then emitted in column order — by sorting the distinct partners
    // when the row has few partners against its width, by a scan of the width
    // otherwise (the row's partner count decides, before any is counted)
    std::atomic<bool> mismatch{false};
    parallel_for(threads, (size_t)n, 64, [&](size_t i0, size_t i1) {
        // one counter array per worker thread, sized once: emission resets
        // every entry it touched to 0, so it is clean for the next chunk
        thread_local std::vector<uint32_t> cnt;
        thread_local std::vector<uint32_t> touched;
        if (cnt.size() < (size_t)n) cnt.assign((size_t)n, 0);
        for (size_t i = i0; i < i1; i++) {
            const bool few = rowcnt[i] * 16 < (uint64_t)n - i;
            touched.clear();
            for (int k = 0; k < L; k++) {
                const int a = x[i * L + k];
                const size_t q = c.off[k] + a, g0 = goff[q], g1 = goff[q + 1];
                if (!a || g1 == g0) continue;
                const size_t b0 = own_place(g0, g1, (uint32_t)i) + 1;
                if (few) {
                    for (size_t b = b0; b < g1; b++)
                        if (cnt[members[b]]++ == 0) touched.push_back(members[b]);
                } else {
                    for (size_t b = b0; b < g1; b++) cnt[members[b]]++;
                }
            }
            uint32_t* w = out->js + out->start[i];
            auto emit = [&](uint32_t j) {
                for (uint32_t r = cnt[j]; r; r--) *w++ = j;
                cnt[j] = 0;
            };
            if (few) {
                std::sort(touched.begin(), touched.end());
                for (uint32_t j : touched) emit(j);
            } else {
                // branch-free for counts 0 and 1: the column is always stored
                // and the end advances by the count (a store at the end of the
                // row's slice lands in a scratch word instead)
                uint32_t* const end = out->js + out->start[i + 1];
                uint32_t scratch;
                for (size_t j = i + 1; j < (size_t)n; j++) {
                    const uint32_t cj = cnt[j];
                    if (cj <= 1) {
                        *(w < end ? w : &scratch) = (uint32_t)j;
                        w += cj;
                        cnt[j] = 0;
                    } else {
                        emit((uint32_t)j);
                    }
                }
            }
            if (w != out->js + out->start[i + 1]) mismatch = true;
        }
    });
    if (mismatch) {
        tch_host_encoding_free(out);
        return set_err(err, errlen, "internal error: rare partner lists do not match their counts");
    }
    return 0;
}

void tch_host_encoding_free(tch_host_encoding* e) {
    if (!e) return;
    free(e->O);
    free(e->P);
    free(e->start);
    free(e->js);
    e->O = e->P = nullptr;
    e->start = e->js = nullptr;
}

}  // extern "C"
