// The CLI's row parser (parse_row: a fused fast path for plain digit cells)
// against the per-cell loop it replaces (find the separator, parse_allele),
// built with AddressSanitizer and UBSan, on random rows of adversarial cells:
// 1-25 digit ids (overflow past 20), INF- prefixes, ASCII and Unicode
// whitespace, missing tokens (also all-digit ones, which turn the fast path
// off), empty cells, too few and too many cells, two separators.  Prints
// "parse_row ok" and exits 0 when every row agrees in values, verdict and
// the first bad cell.
#define main cli_main
#include "cgmlst_hamming_gpu.cpp"
#undef main

#include <random>

static bool reference_row(std::string_view text, size_t f, size_t e, char sep, bool skip, const std::string& missing,
                          size_t L, uint64_t* out, size_t* bb, size_t* be) {
    bool ok = true;
    size_t k = 0;
    while (f < e) {
        const size_t cb = f + 1;
        size_t ce = text.find(sep, cb);
        if (ce == std::string_view::npos || ce > e) ce = e;
        uint64_t v;
        if (!parse_allele(text, cb, ce, skip, missing, &v)) {
            if (ok) {
                *bb = cb;
                *be = ce;
            }
            ok = false;
            v = 0;
        }
        if (k < L) out[k] = v;
        k++;
        f = ce;
    }
    for (; k < L; k++) out[k] = 0;
    return ok;
}

int main() {
    std::mt19937_64 rng(12);
    const char* pieces[] = {"-", "", " ", "INF-", "INF-INF-", "a", "NA", "7", "\xe3\x80\x80", "\xc2\xa0", "0", "x1"};
    size_t rows = 0, fast_cells = 0;
    for (char sep : {'\t', ','})
        for (const std::string missing : {std::string("-"), std::string("NA"), std::string("7")})
            for (bool skip : {false, true}) {
                const RowFormat rf = row_format(sep, skip, missing);
                for (int t = 0; t < 3000; t++) {
                    const size_t L = rng() % 40;
                    const size_t extra = rng() % 7;  // L - 3 .. L + 3 cells
                    const size_t cells = L + extra >= 3 ? L + extra - 3 : 0;
                    std::string row = "id";
                    for (size_t c = 0; c < cells; c++) {
                        row += sep;
                        const int kind = (int)(rng() % 10);
                        if (kind < 5) {  // digits, sometimes long enough to overflow
                            const int nd = 1 + (int)(rng() % (rng() % 8 == 0 ? 25 : 12));
                            for (int d = 0; d < nd; d++) row += (char)('0' + rng() % 10);
                            fast_cells++;
                        } else {
                            const int np = 1 + (int)(rng() % 3);
                            for (int q = 0; q < np; q++) {
                                row += pieces[rng() % (sizeof pieces / sizeof *pieces)];
                                if (rng() % 2) row += std::to_string(rng() % 100000);
                            }
                        }
                    }
                    const std::string_view text(row);
                    size_t f = text.find(sep);
                    if (f == std::string_view::npos) f = text.size();
                    std::vector<uint64_t> a(L + 1, 0xAAAAu), b(L + 1, 0xBBBBu);
                    size_t ab = 0, ae = 0, bb = 0, be = 0;
                    const bool ra = parse_row(text, f, text.size(), rf, L, a.data(), &ab, &ae);
                    const bool rb = reference_row(text, f, text.size(), sep, skip, missing, L, b.data(), &bb, &be);
                    a[L] = b[L] = 0;  // past L: untouched by both
                    if (ra != rb || a != b || (!ra && (ab != bb || ae != be))) {
                        printf("mismatch: sep %d missing '%s' skip %d row '%s'\n", sep, missing.c_str(), skip,
                               row.c_str());
                        return 1;
                    }
                    rows++;
                }
            }
    printf("parse_row ok (%zu rows, %zu digit cells)\n", rows, fast_cells);
    return 0;
}
