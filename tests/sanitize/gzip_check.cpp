// The CLI's gzip writer (host/gzip_writer.h) built with AddressSanitizer and
// UBSan: the bytes read from standard input are written through it in chunks
// of varying size (empty ones, and ones past its 1 MiB block), and the gzip
// member goes to standard output.  Deflate through zlib when built with
// TCH_HAVE_ZLIB, stored blocks otherwise.
#include <cstdio>
#include <random>
#include <string>

#include "gzip_writer.h"

struct StringOut {
    std::string s;
    void write(const char* p, size_t n) { s.append(p, n); }
};

int main() {
    std::string in;
    char tmp[1 << 16];
    size_t r;
    while ((r = fread(tmp, 1, sizeof tmp, stdin)) > 0) in.append(tmp, r);
    StringOut out;
    {
        tch_host::GzipWriter<StringOut> z(out, 3);
        std::mt19937 rng(9);
        size_t off = 0;
        while (off < in.size()) {
            size_t n = rng() % 5 == 0 ? 0 : rng() % 3 == 0 ? (1u << 20) + rng() % 70000 : rng() % 5000;
            n = std::min(n, in.size() - off);
            z.write(in.data() + off, n);
            off += n;
        }
        z.finish();
    }
    fwrite(out.s.data(), 1, out.s.size(), stdout);
    return 0;
}
