// The CLI's CPU TSV writer (write_matrix, the --host-format path) built with
// AddressSanitizer and UBSan.  Arguments: output separator, index name,
// layout (full | lower-tri | upper-tri), cap, threads.  Standard input: n,
// then the n x n symmetric distance matrix, row by row.  The rows are named
// s0 .. s{n-1}; the text goes to standard output.  The CLI's main is renamed
// away.
#define main cli_main
#include "cgmlst_hamming_gpu.cpp"
#undef main

int main(int argc, char** argv) {
    if (argc < 6) return 2;
    const std::string osep = argv[1], index_name = argv[2], lay = argv[3];
    const int cap = atoi(argv[4]);
    const size_t threads = (size_t)atoi(argv[5]);
    size_t n = 0;
    if (scanf("%zu", &n) != 1) return 2;
    std::vector<std::vector<uint16_t>> upper(n);
    for (size_t i = 0; i < n; i++)
        for (size_t j = 0; j < n; j++) {
            unsigned v;
            if (scanf("%u", &v) != 1) return 2;
            if (j > i) upper[i].push_back((uint16_t)v);
        }
    std::vector<std::string> ids(n);
    for (size_t i = 0; i < n; i++) ids[i] = "s" + std::to_string(i);
    const Layout layout = lay == "lower-tri" ? Layout::LowerTri : lay == "upper-tri" ? Layout::UpperTri : Layout::Full;
    FileOut out{stdout};
    write_matrix(out, ids, upper, osep, index_name, layout, cap, threads);
    fflush(stdout);
    return 0;
}
