// The CLI's input path (host/cgmlst_hamming_gpu.cpp: read_all with parallel
// preads, rust_lines, parse_allele) built with AddressSanitizer and UBSan.
// For each file argument and each thread count it prints one line:
// "<bytes> <lines> <cells> <sum of parsed ids>"; the caller checks that every
// thread count gives the same line.  The CLI's main is renamed away.
#define main cli_main
#include "cgmlst_hamming_gpu.cpp"
#undef main

int main(int argc, char** argv) {
    for (int a = 1; a < argc; a++) {
        for (size_t threads : {1, 3, 7, 16}) {
            InputText in;
            std::string err;
            if (!read_all(argv[a], in, err, threads)) {
                printf("error %s\n", err.c_str());
                continue;
            }
            const auto lines = rust_lines(in.view, threads);
            size_t cells = 0;
            unsigned long long sum = 0;
            for (const auto& l : lines) {
                size_t p = l.first;
                while (p < l.second) {
                    size_t f = in.view.find('\t', p);
                    if (f == std::string_view::npos || f > l.second) f = l.second;
                    uint64_t v = 0;
                    if (parse_allele(in.view, p, f, false, "-", &v)) sum += v;
                    cells++;
                    p = f + 1;
                }
            }
            printf("%zu %zu %zu %llu\n", in.view.size(), lines.size(), cells, sum);
        }
    }
    return 0;
}
