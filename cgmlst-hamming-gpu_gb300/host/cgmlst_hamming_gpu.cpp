// cgmlst-hamming-gpu — the command-line host of libtch.
//
// Restates the reference's Rust host (tensorcore/rs/src/main.rs) in C++, with
// the same flags, the same cell semantics, filters and limits, the same
// stderr log lines and the same TSV output, over the same C ABI:
//
//   flags          main.rs:19-73        layouts        main.rs:75-82
//   parse_allele   main.rs:95-113       read_input     main.rs:115-123
//   load           main.rs:286-311      filters        main.rs:313-351
//   encode         main.rs:353-445 (tch_dense_ranks / tch_choose_tau /
//                  tch_encode_host in libtch)
//   GPU            main.rs:447-465 (tch_run + on_stripe, main.rs:200-211)
//   write          main.rs:213-265, 472-490 (gzip: level 3, also for *.gz)
//
// Differences that do not change any output byte: the automatic tau uses rates
// measured on GB300 instead of the L4 constants of main.rs:170-171, the table is
// parsed and filtered on the GPU (tch_tsv_parse / tch_tsv_filter, feeding the
// device encoder; --host-parse or --host-encode: a thread pool on the CPU), and
// the writer formats on the GPU (tch_solver_write_tsv; --host-format: a thread
// pool on the CPU) instead of with rayon.

#include <dlfcn.h>
#include <errno.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <fcntl.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <memory>
#include <new>
#include <string>
#include <string_view>
#include <thread>
#include <utility>
#include <vector>

#include "tch.h"
#include "gzip_writer.h"

namespace {

// GB300 rates for the analytic tau of the host-encoder path (--host-encode):
// pair-columns/s of the tcgen05 fp4 tile pass, and rare pairs/s including
// their 4-byte upload through tch_run (about 190 GB/s of host link; the
// device-encoder path builds the rare groups on the GPU and uses the
// library's own model).
constexpr double kGemmRateGB300 = 2.9e15;
constexpr double kRareRateGB300 = 4.5e10;

// Set while a helper thread creates the CUDA context (during the input's
// load): an error exit then skips the runtime's teardown, which must not run
// while another thread is inside its initialisation.
std::atomic<bool> g_cuda_starting{false};

[[noreturn]] void die(const std::string& msg) {
    fprintf(stderr, "error: %s\n", msg.c_str());
    if (g_cuda_starting) {
        fflush(nullptr);
        _exit(1);
    }
    exit(1);
}

std::string fmt(const char* f, ...) {
    char buf[4096];
    va_list ap;
    va_start(ap, f);
    vsnprintf(buf, sizeof buf, f, ap);
    va_end(ap);
    return buf;
}

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// An allocator whose value-less construct leaves trivial elements
// uninitialised: a vector of n elements is allocated without being zero-filled
// on one core, and its pages are first touched by the threads that fill them.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <class U>
    NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <class U>
    void construct(U* p) noexcept {
        ::new ((void*)p) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a) {
        ::new ((void*)p) U(std::forward<A>(a)...);
    }
};
using CallMatrix = std::vector<uint64_t, NoInitAlloc<uint64_t>>;

enum class Layout { Full, LowerTri, UpperTri };

struct Args {
    std::string input;
    bool has_output = false;
    std::string output;
    size_t threads = 0;
    Layout layout = Layout::Full;
    std::string input_sep = "\t";
    std::string output_sep = "\t";
    std::string index_name = "cgmlst-hamming-gpu";
    std::string missing = "-";
    bool skip_repl = false;
    bool has_locus = false, has_sample = false;
    double locus_pct = 0, sample_pct = 0;
    bool gzip = false;
    int max_dist = 0;
    size_t tau = 0;
    size_t stripe = 512;
    size_t device = 0;
    bool silent = false;
    bool host_encode = false;
    bool host_format = false;
    bool host_parse = false;
};

const char* kUsage =
    "Exact cgMLST Hamming distance matrix on GB300 tensor cores\n\n"
    "Usage: cgmlst-hamming-gpu [OPTIONS] --input <INPUT>\n\n"
    "Options:\n"
    "  -i, --input <INPUT>                      Input allele-call TSV (chewBBACA format). Use '-' for stdin\n"
    "  -o, --output <OUTPUT>                    Output file [default: stdout]\n"
    "  -t, --threads <THREADS>                  Number of CPU threads [default: all cores] [default: 0]\n"
    "  -m, --matrix-format <MATRIX_FORMAT>      Output matrix layout [default: full] [possible values: full, "
    "lower-tri, upper-tri]\n"
    "  -d, --input-sep <INPUT_SEP>              Input field separator [default: \"\\t\"]\n"
    "  -D, --output-sep <OUTPUT_SEP>            Output field separator [default: \"\\t\"]\n"
    "  -x, --index-name <INDEX_NAME>            Name for the top-left index cell [default: cgmlst-hamming-gpu]\n"
    "  -n, --missing-char <MISSING_CHAR>        Character used for missing data [default: -]\n"
    "  -r, --skip-input-replacements            Do not strip the chewBBACA `INF-` prefix\n"
    "  -L, --locus-completeness <PCT>           Keep only loci with at least this % of non-missing calls (0-100)\n"
    "  -S, --sample-completeness <PCT>          Keep only samples with at least this % of non-missing calls (0-100)\n"
    "  -z, --gzip                               gzip-compress the output (also enabled when -o ends with .gz)\n"
    "  -X, --max-dist <MAX_DIST>                Cap distances at this value (0 = no cap) [default: 0]\n"
    "      --tau <TAU>                          Frequency threshold: alleles seen >= tau times go to the "
    "tensor-core GEMM [0 = auto] [default: 0]\n"
    "      --stripe <STRIPE>                    Rows per GPU stripe [default: 512]\n"
    "      --device <DEVICE>                    CUDA device [default: 0]\n"
    "  -s, --silent                             Suppress progress/log messages on stderr\n"
    "      --host-encode                        Encode on the host and call tch_run (the reference's path)\n"
    "      --host-format                        Format the matrix text on the CPU (default: on the GPU)\n"
    "      --host-parse                         Parse the input table on the CPU (default: on the GPU)\n"
    "  -h, --help                               Print help\n"
    "  -V, --version                            Print version\n";

[[noreturn]] void usage_error(const std::string& msg) {
    fprintf(stderr, "error: %s\n\nUsage: cgmlst-hamming-gpu [OPTIONS] --input <INPUT>\n\nFor more information, try "
            "'--help'.\n", msg.c_str());
    exit(2);
}

template <class T>
T parse_num(const std::string& flag, const std::string& v, bool allow_neg, bool is_float) {
    errno = 0;
    char* end = nullptr;
    if (v.empty()) usage_error(fmt("invalid value '' for '%s'", flag.c_str()));
    if (is_float) {
        double d = strtod(v.c_str(), &end);
        if (*end || errno) usage_error(fmt("invalid value '%s' for '%s': invalid float literal", v.c_str(), flag.c_str()));
        return (T)d;
    }
    if (!allow_neg && v[0] == '-') usage_error(fmt("invalid value '%s' for '%s': invalid digit found in string",
                                                   v.c_str(), flag.c_str()));
    long long x = strtoll(v.c_str(), &end, 10);
    if (*end || errno) usage_error(fmt("invalid value '%s' for '%s': invalid digit found in string", v.c_str(),
                                       flag.c_str()));
    return (T)x;
}

Args parse_args(int argc, char** argv) {
    Args a;
    bool have_input = false;
    struct Opt {
        const char* shrt;
        const char* lng;
        bool takes;
    };
    static const Opt opts[] = {{"i", "input", true},         {"o", "output", true},
                               {"t", "threads", true},       {"m", "matrix-format", true},
                               {"d", "input-sep", true},     {"D", "output-sep", true},
                               {"x", "index-name", true},    {"n", "missing-char", true},
                               {"r", "skip-input-replacements", false},
                               {"L", "locus-completeness", true}, {"S", "sample-completeness", true},
                               {"z", "gzip", false},         {"X", "max-dist", true},
                               {nullptr, "tau", true},       {nullptr, "stripe", true},
                               {nullptr, "device", true},    {"s", "silent", false},
                               {nullptr, "host-encode", false},     {nullptr, "host-format", false},
                               {nullptr, "host-parse", false},
                               {"h", "help", false},         {"V", "version", false}};
    for (int k = 1; k < argc; k++) {
        std::string arg = argv[k];
        const Opt* o = nullptr;
        std::string val;
        bool has_val = false;
        if (arg.rfind("--", 0) == 0 && arg.size() > 2) {
            std::string name = arg.substr(2);
            size_t eq = name.find('=');
            if (eq != std::string::npos) {
                val = name.substr(eq + 1);
                name = name.substr(0, eq);
                has_val = true;
            }
            for (auto& c : opts)
                if (name == c.lng) o = &c;
            if (!o) usage_error(fmt("unexpected argument '%s' found", arg.c_str()));
        } else if (arg.size() >= 2 && arg[0] == '-' && arg[1] != '-') {
            std::string s(1, arg[1]);
            for (auto& c : opts)
                if (c.shrt && s == c.shrt) o = &c;
            if (!o) usage_error(fmt("unexpected argument '%s' found", arg.c_str()));
            if (arg.size() > 2) {
                if (!o->takes) usage_error(fmt("unexpected argument '%s' found", arg.c_str()));
                val = arg.substr(2);
                has_val = true;
            }
        } else {
            usage_error(fmt("unexpected argument '%s' found", arg.c_str()));
        }
        const std::string flag = o->lng ? std::string("--") + o->lng : arg;
        if (o->takes && !has_val) {
            if (k + 1 >= argc) usage_error(fmt("a value is required for '%s <VALUE>' but none was supplied",
                                               flag.c_str()));
            val = argv[++k];
        }
        const std::string name = o->lng;
        if (name == "help") {
            fputs(kUsage, stdout);
            exit(0);
        } else if (name == "version") {
            printf("cgmlst-hamming-gpu %d.0.0 (GB300)\n", tch_version());
            exit(0);
        } else if (name == "input") {
            a.input = val;
            have_input = true;
        } else if (name == "output") {
            a.output = val;
            a.has_output = true;
        } else if (name == "threads") {
            a.threads = parse_num<size_t>(flag, val, false, false);
        } else if (name == "matrix-format") {
            if (val == "full") a.layout = Layout::Full;
            else if (val == "lower-tri") a.layout = Layout::LowerTri;
            else if (val == "upper-tri") a.layout = Layout::UpperTri;
            else usage_error(fmt("invalid value '%s' for '--matrix-format <MATRIX_FORMAT>'\n  [possible values: "
                                 "full, lower-tri, upper-tri]", val.c_str()));
        } else if (name == "input-sep") {
            a.input_sep = val;
        } else if (name == "output-sep") {
            a.output_sep = val;
        } else if (name == "index-name") {
            a.index_name = val;
        } else if (name == "missing-char") {
            a.missing = val;
        } else if (name == "skip-input-replacements") {
            a.skip_repl = true;
        } else if (name == "locus-completeness") {
            a.locus_pct = parse_num<double>(flag, val, true, true);
            a.has_locus = true;
        } else if (name == "sample-completeness") {
            a.sample_pct = parse_num<double>(flag, val, true, true);
            a.has_sample = true;
        } else if (name == "gzip") {
            a.gzip = true;
        } else if (name == "max-dist") {
            a.max_dist = parse_num<int>(flag, val, true, false);
        } else if (name == "tau") {
            a.tau = parse_num<size_t>(flag, val, false, false);
        } else if (name == "stripe") {
            a.stripe = parse_num<size_t>(flag, val, false, false);
        } else if (name == "device") {
            a.device = parse_num<size_t>(flag, val, false, false);
        } else if (name == "silent") {
            a.silent = true;
        } else if (name == "host-encode") {
            a.host_encode = true;
        } else if (name == "host-format") {
            a.host_format = true;
        } else if (name == "host-parse") {
            a.host_parse = true;
        }
    }
    if (!have_input) usage_error("the following required arguments were not provided:\n  --input <INPUT>");
    return a;
}

template <class F>
void parallel_for(size_t threads, size_t count, size_t chunk, F&& f) {
    if (threads <= 1 || count <= chunk) {
        for (size_t b = 0; b < count; b += chunk) f(b, std::min(count, b + chunk));
        return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (size_t t = 0; t < threads; t++)
        pool.emplace_back([&] {
            for (;;) {
                const size_t b = next.fetch_add(chunk);
                if (b >= count) break;
                f(b, std::min(count, b + chunk));
            }
        });
    for (auto& th : pool) th.join();
}

// ---- text semantics ---------------------------------------------------------------

// Decodes the UTF-8 code point starting at s[i] (input already validated).
uint32_t cp_at(std::string_view s, size_t i, size_t* len) {
    const unsigned char c = (unsigned char)s[i];
    if (c < 0x80) { *len = 1; return c; }
    if ((c >> 5) == 6) { *len = 2; return ((c & 0x1F) << 6) | (s[i + 1] & 0x3F); }
    if ((c >> 4) == 14) { *len = 3; return ((c & 0x0F) << 12) | ((s[i + 1] & 0x3F) << 6) | (s[i + 2] & 0x3F); }
    *len = 4;
    return ((c & 0x07) << 18) | ((s[i + 1] & 0x3F) << 12) | ((s[i + 2] & 0x3F) << 6) | (s[i + 3] & 0x3F);
}

// Unicode White_Space, the set Rust's str::trim removes.
bool is_ws(uint32_t c) {
    return (c >= 0x09 && c <= 0x0D) || c == 0x20 || c == 0x85 || c == 0xA0 || c == 0x1680 ||
           (c >= 0x2000 && c <= 0x200A) || c == 0x2028 || c == 0x2029 || c == 0x202F || c == 0x205F || c == 0x3000;
}

// [b, e) of the trimmed cell inside s.
void trim(std::string_view s, size_t& b, size_t& e) {
    while (b < e) {
        size_t len;
        const uint32_t c = cp_at(s, b, &len);
        if (!is_ws(c)) break;
        b += len;
    }
    while (e > b) {
        size_t p = e - 1;
        while (p > b && ((unsigned char)s[p] & 0xC0) == 0x80) p--;
        size_t len;
        const uint32_t c = cp_at(s, p, &len);
        if (!is_ws(c)) break;
        e = p;
    }
}

// parse_allele (main.rs:98-113): 0 = missing; returns false on u64 overflow.
bool parse_allele(std::string_view s, size_t b, size_t e, bool skip_repl, const std::string& missing,
                  uint64_t* out) {
    trim(s, b, e);
    if (!skip_repl && e - b >= 4 && s.compare(b, 4, "INF-") == 0) b += 4;
    if (b == e || (e - b == missing.size() && s.compare(b, e - b, missing) == 0)) {
        *out = 0;
        return true;
    }
    uint64_t v = 0;
    for (size_t p = b; p < e; p++) {
        const char c = s[p];
        if (c < '0' || c > '9') {
            *out = 0;
            return true;
        }
    }
    for (size_t p = b; p < e; p++) {
        const uint64_t d = (uint64_t)(s[p] - '0');
        if (v > (UINT64_MAX - d) / 10) return false;
        v = v * 10 + d;
    }
    *out = v;
    return true;
}

// The cells of one data row (main.rs:295-311): the row is text[f, e), f at the
// separator after the sample id (or e).  Cell k goes to out[k] for k < L;
// cells past L are read and dropped, cells missing at the row's end are 0.
// A cell of 1-19 ASCII digits running up to the separator is parsed in the
// same pass that finds its end (such a value cannot overflow, trimming and the
// INF- prefix do not apply, and the missing token is not all digits when the
// fast path is on); any other cell is found with memchr and read by
// parse_allele.  Returns false with [*bad_b, *bad_e) at the first cell whose
// id overflows u64 (that cell reads 0).
struct RowFormat {
    char sep;
    bool skip_repl;
    const std::string* missing;
    bool fast;  // the separator is not a digit and the missing token is not all digits
};

RowFormat row_format(char sep, bool skip_repl, const std::string& missing) {
    bool digits = !missing.empty();
    for (char c : missing) digits = digits && c >= '0' && c <= '9';
    return RowFormat{sep, skip_repl, &missing, !(sep >= '0' && sep <= '9') && !digits};
}

bool parse_row(std::string_view text, size_t f, size_t e, const RowFormat& rf, size_t L, uint64_t* out,
               size_t* bad_b, size_t* bad_e) {
    const char* s = text.data();
    bool ok = true;
    size_t k = 0;
    while (f < e) {
        const size_t cb = f + 1;
        size_t q = cb;
        uint64_t v = 0;
        if (rf.fast)
            while (q < e && q - cb < 19) {
                const unsigned d = (unsigned)(unsigned char)s[q] - (unsigned)'0';
                if (d > 9) break;
                v = v * 10 + d;
                q++;
            }
        size_t ce;
        if (rf.fast && q > cb && (q == e || s[q] == rf.sep)) {
            ce = q;
        } else {
            const void* hit = cb < e ? memchr(s + cb, rf.sep, e - cb) : nullptr;
            ce = hit ? (size_t)((const char*)hit - s) : e;
            if (!parse_allele(text, cb, ce, rf.skip_repl, *rf.missing, &v)) {
                if (ok) {
                    *bad_b = cb;
                    *bad_e = ce;
                }
                ok = false;
                v = 0;
            }
        }
        if (k < L) out[k] = v;
        k++;
        f = ce;
    }
    for (; k < L; k++) out[k] = 0;
    return ok;
}

// UTF-8 check of s[b, e): every sequence that starts there is complete and
// well formed (it may read up to 3 bytes past e to finish one).
bool valid_utf8_range(std::string_view s, size_t b, size_t e) {
    size_t i = b;
    const size_t n = s.size();
    while (i < e) {
        // a run of ASCII, eight bytes at a time (no byte with its high bit set)
        while (i + 8 <= e) {
            uint64_t w;
            memcpy(&w, s.data() + i, 8);
            if (w & 0x8080808080808080ull) break;
            i += 8;
        }
        if (i >= e) break;
        const unsigned char c = (unsigned char)s[i];
        size_t len;
        uint32_t cp;
        if (c < 0x80) { i++; continue; }
        if ((c >> 5) == 6) { len = 2; cp = c & 0x1F; }
        else if ((c >> 4) == 14) { len = 3; cp = c & 0x0F; }
        else if ((c >> 3) == 30) { len = 4; cp = c & 0x07; }
        else return false;
        if (i + len > n) return false;
        for (size_t k = 1; k < len; k++) {
            const unsigned char d = (unsigned char)s[i + k];
            if ((d & 0xC0) != 0x80) return false;
            cp = (cp << 6) | (d & 0x3F);
        }
        if ((len == 2 && cp < 0x80) || (len == 3 && cp < 0x800) || (len == 4 && (cp < 0x10000 || cp > 0x10FFFF)) ||
            (cp >= 0xD800 && cp <= 0xDFFF))
            return false;
        i += len;
    }
    return true;
}

// The whole buffer, in parallel chunks; a chunk starts at a byte that begins a
// sequence (continuation bytes at a chunk's start belong to the previous one).
bool valid_utf8(std::string_view s, size_t threads) {
    const size_t n = s.size(), parts = std::max<size_t>(1, std::min<size_t>(threads * 4, n / (1 << 20) + 1));
    std::vector<size_t> cut(parts + 1, n);
    cut[0] = 0;
    for (size_t k = 1; k < parts; k++) {
        size_t c = n * k / parts;
        for (int back = 0; back < 3 && c > 0 && ((unsigned char)s[c] & 0xC0) == 0x80; back++) c--;
        cut[k] = std::max(c, cut[k - 1]);
    }
    std::atomic<bool> ok{true};
    parallel_for(threads, parts, 1, [&](size_t a, size_t b) {
        for (size_t k = a; k < b; k++)
            if (!valid_utf8_range(s, cut[k], cut[k + 1])) ok = false;
    });
    return ok;
}

// The input's bytes.  A regular file is read into one allocation that is not
// zero-filled, by parallel preads: each thread faults in and fills its own
// range, so neither the page faults nor the copy out of the page cache run on
// one core.  A pipe (or "-") is read sequentially.
struct InputText {
    std::unique_ptr<char[]> raw;
    std::string piped;
    std::string_view view;
};

bool read_all(const std::string& path, InputText& in, std::string& err, size_t threads) {
    bool bad = false;
    int fd = -1;
    struct stat st;
    if (path != "-" && (fd = open(path.c_str(), O_RDONLY)) < 0) {
        err = strerror(errno);
        return false;
    }
    if (fd >= 0 && fstat(fd, &st) == 0 && S_ISREG(st.st_mode)) {
        const size_t size = (size_t)st.st_size;
        in.raw.reset(new char[std::max<size_t>(size, 1)]);
        char* base = in.raw.get();
        const size_t parts = std::max<size_t>(1, std::min<size_t>(threads, size >> 22));
        std::atomic<bool> short_read{false};
        parallel_for(threads, parts, 1, [&](size_t a, size_t b) {
            for (size_t k = a; k < b; k++) {
                size_t off = size * k / parts;
                const size_t end = size * (k + 1) / parts;
                while (off < end) {
                    const ssize_t r = pread(fd, base + off, end - off, (off_t)off);
                    if (r <= 0) {
                        short_read = true;
                        break;
                    }
                    off += (size_t)r;
                }
            }
        });
        bad = short_read;
        char extra;
        if (!bad && pread(fd, &extra, 1, (off_t)size) == 1) {  // grew meanwhile: read the rest
            in.piped.assign(base, size);
            in.raw.reset();
            char tmp[1 << 16];
            ssize_t r;
            off_t off = (off_t)size;
            while ((r = pread(fd, tmp, sizeof tmp, off)) > 0) {
                in.piped.append(tmp, (size_t)r);
                off += r;
            }
            if (r < 0) bad = true;
            in.view = in.piped;
        } else {
            in.view = std::string_view(base, size);
        }
    } else {
        FILE* f = fd >= 0 ? fdopen(fd, "rb") : stdin;
        if (!f) {
            err = strerror(errno);
            close(fd);
            return false;
        }
        char tmp[1 << 16];
        size_t r;
        while ((r = fread(tmp, 1, sizeof tmp, f)) > 0) in.piped.append(tmp, r);
        bad = ferror(f) != 0;
        if (f != stdin) fclose(f);
        fd = -1;
        in.view = in.piped;
    }
    if (fd >= 0) close(fd);
    if (bad) {
        err = "read error";
        return false;
    }
    if (!valid_utf8(in.view, threads)) {
        err = "stream did not contain valid UTF-8";
        return false;
    }
    return true;
}

// str::lines: (begin, end) of every line, '\n' and one '\r' before it removed;
// the newlines are found in parallel chunks.
std::vector<std::pair<size_t, size_t>> rust_lines(std::string_view t, size_t threads) {
    const size_t n = t.size(), parts = std::max<size_t>(1, std::min<size_t>(threads * 4, n / (1 << 20) + 1));
    std::vector<std::vector<size_t>> nl(parts);
    parallel_for(threads, parts, 1, [&](size_t a, size_t b) {
        for (size_t k = a; k < b; k++) {
            const size_t lo = n * k / parts, hi = n * (k + 1) / parts;
            const char* p = t.data() + lo;
            const char* e = t.data() + hi;
            while (p < e) {
                const char* q = (const char*)memchr(p, '\n', (size_t)(e - p));
                if (!q) break;
                nl[k].push_back((size_t)(q - t.data()));
                p = q + 1;
            }
        }
    });
    std::vector<std::pair<size_t, size_t>> out;
    size_t b = 0;
    for (auto& v : nl)
        for (size_t q : v) {
            size_t e = q;
            if (e > b && t[e - 1] == '\r') e--;
            out.push_back({b, e});
            b = q + 1;
        }
    if (b < n) out.push_back({b, n});
    return out;
}

// ---- output ----------------------------------------------------------------------

struct Sink {
    std::vector<std::vector<uint16_t>>* upper;
    size_t threads;
};

void on_stripe(void* ctx, int r0, int rows, size_t w, const uint16_t* stripe) {
    Sink* s = (Sink*)ctx;
    parallel_for(s->threads, (size_t)rows, 16, [&](size_t a, size_t b) {
        for (size_t r = a; r < b; r++)
            (*s->upper)[r0 + r].assign(stripe + r * w + r + 1, stripe + (r + 1) * w);
    });
}

// A distance (0-65 535) in decimal at p, two digits per table lookup; returns
// the end.
inline char* put_u16(char* p, unsigned v) {
    static const char d2[] =
        "00010203040506070809101112131415161718192021222324252627282930313233343536373839"
        "40414243444546474849505152535455565758596061626364656667686970717273747576777879"
        "8081828384858687888990919293949596979899";
    if (v < 10) {
        *p = (char)('0' + v);
        return p + 1;
    }
    if (v < 100) {
        memcpy(p, d2 + 2 * v, 2);
        return p + 2;
    }
    if (v >= 10000) {
        *p++ = (char)('0' + v / 10000);
        v %= 10000;
        memcpy(p, d2 + 2 * (v / 100), 2);
        memcpy(p + 2, d2 + 2 * (v % 100), 2);
        return p + 4;
    }
    if (v >= 1000) {
        memcpy(p, d2 + 2 * (v / 100), 2);
        memcpy(p + 2, d2 + 2 * (v % 100), 2);
        return p + 4;
    }
    *p = (char)('0' + v / 100);
    memcpy(p + 1, d2 + 2 * (v % 100), 2);
    return p + 3;
}

// write_matrix (main.rs:225-265): header, then rows formatted in parallel
// chunks of 1024 and written in order.  A row is written through a pointer
// into a buffer sized for its longest text (id, then per cell the separator
// and at most five digits), reused for every chunk: cells left of the
// diagonal come from the earlier rows' upper parts, cells right of it from the
// row's own, and cells the layout blanks are 0.
template <class W>
void write_matrix(W& out, const std::vector<std::string>& ids, const std::vector<std::vector<uint16_t>>& upper,
                  const std::string& osep, const std::string& index_name, Layout lay, int cap, size_t threads) {
    const size_t n = ids.size();
    std::string head = index_name;
    for (auto& id : ids) {
        head += osep;
        head += id;
    }
    head += '\n';
    out.write(head.data(), head.size());
    const size_t CHUNK = 1024, sl = osep.size();
    size_t maxid = 0;
    for (auto& id : ids) maxid = std::max(maxid, id.size());
    const size_t cap_row = maxid + n * (sl + 5) + 1;
    const size_t rows_buf = std::min(n, CHUNK);
    std::unique_ptr<char[]> text(new char[std::max<size_t>(rows_buf * cap_row, 1)]);
    std::vector<size_t> len(rows_buf);
    const unsigned vcap = cap > 0 ? (unsigned)cap : 65535u;
    for (size_t start = 0; start < n; start += CHUNK) {
        const size_t end = std::min(n, start + CHUNK);
        parallel_for(threads, end - start, 8, [&](size_t a, size_t b) {
            for (size_t q = a; q < b; q++) {
                const size_t i = start + q;
                char* const row = text.get() + q * cap_row;
                char* p = row;
                memcpy(p, ids[i].data(), ids[i].size());
                p += ids[i].size();
                auto sep = [&]() {
                    if (sl == 1) *p++ = osep[0];
                    else {
                        memcpy(p, osep.data(), sl);
                        p += sl;
                    }
                };
                // columns j < i (blank in the upper-tri layout)
                for (size_t j = 0; j < i; j++) {
                    sep();
                    const unsigned v = lay == Layout::UpperTri ? 0u : upper[j][i - j - 1];
                    p = put_u16(p, std::min(v, vcap));
                }
                sep();  // the diagonal
                *p++ = '0';
                // columns j > i (blank in the lower-tri layout)
                const uint16_t* u = upper[i].data();
                for (size_t j = i + 1; j < n; j++) {
                    sep();
                    const unsigned v = lay == Layout::LowerTri ? 0u : u[j - i - 1];
                    p = put_u16(p, std::min(v, vcap));
                }
                *p++ = '\n';
                len[q] = (size_t)(p - row);
            }
        });
        for (size_t q = 0; q < end - start; q++) out.write(text.get() + q * cap_row, len[q]);
    }
}

struct FileOut {
    FILE* f;
    void write(const char* p, size_t n) {
        if (n && fwrite(p, 1, n, f) != n) die(fmt("writing output: %s", strerror(errno)));
    }
};

// tch_text_cb into a writer.
template <class W>
void text_to(void* ctx, const char* text, size_t len) {
    static_cast<W*>(ctx)->write(text, len);
}

}  // namespace

int main(int argc, char** argv) {
    Args args = parse_args(argc, argv);
    const double t_start = now();
    auto log = [&](const std::string& m) {
        if (!args.silent) fprintf(stderr, "%s\n", m.c_str());
    };
    size_t threads = args.threads ? args.threads : std::max(1u, std::thread::hardware_concurrency());
    if (args.input_sep.size() != 1) die("input separator must be a single character");
    const char sep = args.input_sep[0];
    if ((size_t)tch_device_count() <= args.device) die(fmt("CUDA device %zu not available", args.device));

    // the CUDA context (~0.1 s) is created while the input is read and parsed
    g_cuda_starting = true;
    std::thread cuda_start([&] { tch_free_vram((int)args.device); });

    // ---- load (main.rs:286-311)
    double t = now();
    InputText in;
    std::string rerr;
    if (!read_all(args.input, in, rerr, threads)) die(fmt("reading %s: %s", args.input.c_str(), rerr.c_str()));
    const std::string_view text = in.view;
    if (text.empty()) die("empty input");
    // the table parsed on the GPU (the calls stay there for the device encoder),
    // or on the host cores (--host-parse, and the reference's path)
    const bool gpu_parse = !args.host_parse && !args.host_encode;
    tch_tsv* tsv = nullptr;
    size_t n = 0, L = 0;
    std::vector<std::string> ids;
    CallMatrix calls;
    auto tsv_ids = [&]() {
        int nn = 0, ll = 0;
        tch_tsv_shape(tsv, &nn, &ll);
        n = (size_t)nn;
        L = (size_t)ll;
        std::vector<size_t> b(n), e(n);
        tch_tsv_ids(tsv, b.data(), e.data());
        ids.assign(n, std::string());
        for (size_t i = 0; i < n; i++) ids[i] = std::string(text.substr(b[i], e[i] - b[i]));
    };
    if (gpu_parse) {
        if (cuda_start.joinable()) cuda_start.join();
        g_cuda_starting = false;
        char perr[512] = {0};
        if (tch_tsv_parse((int)args.device, text.data(), text.size(), sep, args.skip_repl ? 1 : 0,
                          args.missing.c_str(), &tsv, perr, sizeof perr))
            die(perr);
        tsv_ids();
    } else {
    auto lines = rust_lines(text, threads);
    L = 1;
    for (size_t p = lines[0].first; p < lines[0].second; p++) L += text[p] == sep;
    L -= 1;
    std::vector<std::pair<size_t, size_t>> data;
    for (size_t k = 1; k < lines.size(); k++)
        if (lines[k].second > lines[k].first) data.push_back(lines[k]);
    n = data.size();
    ids.assign(n, std::string());
    CallMatrix(n * L).swap(calls);  // every cell written by the parse below
    std::atomic<long> bad_row{-1};
    std::vector<std::string> bad_cell(1);
    std::atomic<bool> bad_taken{false};
    const RowFormat rf = row_format(sep, args.skip_repl, args.missing);
    parallel_for(threads, n, 64, [&](size_t a, size_t b) {
        for (size_t i = a; i < b; i++) {
            const size_t p = data[i].first, e = data[i].second;
            size_t f = text.find(sep, p);
            if (f == std::string_view::npos || f > e) f = e;
            ids[i] = std::string(text.substr(p, f - p));
            size_t cb = 0, ce = 0;
            if (!parse_row(text, f, e, rf, L, calls.data() + i * L, &cb, &ce)) {
                bool expect = false;
                if (bad_taken.compare_exchange_strong(expect, true)) {
                    trim(text, cb, ce);
                    bad_cell[0] = std::string(text.substr(cb, ce - cb));
                    bad_row = (long)i;
                }
            }
        }
    });
    if (bad_row >= 0) die(fmt("sample %s: allele '%s' too large", ids[bad_row].c_str(), bad_cell[0].c_str()));
    }
    log(fmt("Loaded %zu samples x %zu loci in %.2fs", n, L, now() - t));

    // ---- completeness filters (main.rs:313-348), counted and compacted in parallel
    if (args.has_locus && tsv) {
        char ferr[512] = {0};
        if (tch_tsv_filter(tsv, args.locus_pct, -1.0, ferr, sizeof ferr)) die(ferr);
        tsv_ids();
        log(fmt("Locus completeness >= %s%%: kept %zu loci", fmt("%g", args.locus_pct).c_str(), L));
    } else if (args.has_locus) {
        // non-missing calls per locus: blocks of rows counted apart, then summed
        const size_t parts = std::max<size_t>(1, std::min<size_t>(threads, n / 256 + 1));
        std::vector<std::vector<size_t>> part(parts, std::vector<size_t>(L, 0));
        parallel_for(threads, parts, 1, [&](size_t a, size_t b) {
            for (size_t p = a; p < b; p++) {
                std::vector<size_t>& c = part[p];
                for (size_t i = n * p / parts; i < n * (p + 1) / parts; i++) {
                    const uint64_t* row = calls.data() + i * L;
                    for (size_t k = 0; k < L; k++) c[k] += row[k] != 0;
                }
            }
        });
        std::vector<size_t> keep;
        for (size_t k = 0; k < L; k++) {
            size_t c = 0;
            for (size_t p = 0; p < parts; p++) c += part[p][k];
            if (((double)c / (double)n) * 100.0 >= args.locus_pct) keep.push_back(k);
        }
        if (keep.size() != L) {
            const size_t lk = keep.size();
            CallMatrix nc(n * lk);
            parallel_for(threads, n, 256, [&](size_t a, size_t b) {
                for (size_t i = a; i < b; i++)
                    for (size_t d = 0; d < lk; d++) nc[i * lk + d] = calls[i * L + keep[d]];
            });
            calls.swap(nc);
            L = lk;
        }
        log(fmt("Locus completeness >= %s%%: kept %zu loci", fmt("%g", args.locus_pct).c_str(), L));
    }
    if (args.has_sample && tsv) {
        char ferr[512] = {0};
        if (tch_tsv_filter(tsv, -1.0, args.sample_pct, ferr, sizeof ferr)) die(ferr);
        tsv_ids();
        log(fmt("Sample completeness >= %s%%: kept %zu samples", fmt("%g", args.sample_pct).c_str(), n));
    } else if (args.has_sample) {
        std::vector<char> ok(n, 0);
        parallel_for(threads, n, 256, [&](size_t a, size_t b) {
            for (size_t i = a; i < b; i++) {
                size_t c = 0;
                const uint64_t* row = calls.data() + i * L;
                for (size_t k = 0; k < L; k++) c += row[k] != 0;
                ok[i] = ((double)c / (double)L) * 100.0 >= args.sample_pct;
            }
        });
        std::vector<size_t> keep;
        for (size_t i = 0; i < n; i++)
            if (ok[i]) keep.push_back(i);
        if (keep.size() != n) {
            CallMatrix nc(keep.size() * L);
            parallel_for(threads, keep.size(), 256, [&](size_t a, size_t b) {
                for (size_t d = a; d < b; d++)
                    std::copy(calls.begin() + keep[d] * L, calls.begin() + (keep[d] + 1) * L, nc.begin() + d * L);
            });
            std::vector<std::string> nids(keep.size());
            for (size_t d = 0; d < keep.size(); d++) nids[d] = std::move(ids[keep[d]]);
            calls.swap(nc);
            ids.swap(nids);
            n = keep.size();
        }
        log(fmt("Sample completeness >= %s%%: kept %zu samples", fmt("%g", args.sample_pct).c_str(), n));
    }
    in = InputText();  // the ids are copied out
    if (L > 65535) die("more than 65535 loci (u16 distances)");

    // ---- output (main.rs:472-490): a file or stdout, gzip level 3 with -z or *.gz
    const bool gz = args.gzip || (args.has_output && args.output.size() >= 3 &&
                                  args.output.compare(args.output.size() - 3, 3, ".gz") == 0);
    auto open_out = [&]() {
        FILE* f = stdout;
        if (args.has_output) {
            f = fopen(args.output.c_str(), "wb");
            if (!f) die(fmt("creating %s: %s", args.output.c_str(), strerror(errno)));
        }
        setvbuf(f, nullptr, _IOFBF, 16 << 20);
        return f;
    };
    auto close_out = [&](FILE* f) {
        if (fflush(f) != 0) die(fmt("writing output: %s", strerror(errno)));
        if (f != stdout) fclose(f);
    };

    // ---- encode (main.rs:353-445) and GPU (main.rs:447-465)
    if (cuda_start.joinable()) cuda_start.join();
    g_cuda_starting = false;
    t = now();
    char err[512] = {0};
    std::vector<std::vector<uint16_t>> upper(n);
    double gpu_secs = 0;
    if (n >= 2 && L > 0 && !args.host_encode) {
        // device encoder: ranks, one-hot, presence and rare pairs on the GPU
        const size_t stripe = std::max<size_t>(args.stripe, 8) / 8 * 8;
        if (!args.silent) setenv("TCH_VERBOSE", "1", 1);
        tch_solver* solver = nullptr;
        if (tsv ? tch_solver_from_tsv(tsv, (int)args.tau, &solver, err, sizeof err)
                : tch_solver_from_calls((int)args.device, (int)n, (int)L, calls.data(), (int)args.tau,
                                        TCH_KERNEL_AUTO, &solver, err, sizeof err))
            die(err);
        CallMatrix().swap(calls);
        tch_tsv_free(tsv);
        tsv = nullptr;
        tch_info info;
        tch_solver_info(solver, &info);
        log(fmt("Encoded in %.2fs: tau=%d, one-hot cols=%zu, rare equal pairs=%zu", now() - t, info.tau,
                info.d_onehot, info.n_rare));
        t = now();
        if (!args.host_format) {
            // the matrix stays in HBM and is formatted there; text blocks come back in order
            std::vector<const char*> idp(n);
            for (size_t i = 0; i < n; i++) idp[i] = ids[i].c_str();
            const int lay = args.layout == Layout::Full ? 0 : args.layout == Layout::LowerTri ? 1 : 2;
            FILE* f = open_out();
            FileOut fo{f};
            int rc;
            if (gz) {
                tch_host::GzipWriter<FileOut> z(fo, 3);
                rc = tch_solver_write_tsv(solver, idp.data(), args.output_sep.c_str(), args.index_name.c_str(), lay,
                                          args.max_dist, 0, text_to<tch_host::GzipWriter<FileOut>>, &z, err,
                                          sizeof err);
                if (!rc) z.finish();
            } else {
                rc = tch_solver_write_tsv(solver, idp.data(), args.output_sep.c_str(), args.index_name.c_str(), lay,
                                          args.max_dist, 0, text_to<FileOut>, &fo, err, sizeof err);
            }
            tch_solver_destroy(solver);
            if (rc) die(fmt("CUDA: %s", err));
            close_out(f);
            log(fmt("Computed and wrote the %zu x %zu matrix (tensor cores, text formatted on the GPU) in %.2fs. "
                    "Total %.2fs", n, n, now() - t, now() - t_start));
            return 0;
        }
        Sink sink{&upper, threads};
        const int rc = tch_solver_run(solver, (int)stripe, on_stripe, &sink, &gpu_secs, err, sizeof err);
        tch_solver_destroy(solver);
        if (rc) die(fmt("CUDA: %s", err));
        log(fmt("Computed %zu x %zu matrix on tensor cores in %.2fs (GPU pipeline %.2fs, rare pairs on GPU)", n, n,
                now() - t, gpu_secs));
    } else if (n >= 2 && L > 0) {
        // the reference's path: host encoder + tch_run
        std::vector<uint16_t> x(n * L);
        std::vector<uint32_t> nd(L);
        if (tch_dense_ranks(calls.data(), (int)n, (int)L, x.data(), nd.data(), (int)threads, err, sizeof err))
            die(err);
        CallMatrix().swap(calls);
        const size_t stripe = std::max<size_t>(args.stripe, 8) / 8 * 8;
        int tau = (int)args.tau;
        if (tau <= 0 &&
            tch_choose_tau(x.data(), nd.data(), (int)n, (int)L, (int)stripe, tch_free_vram((int)args.device),
                           kGemmRateGB300, kRareRateGB300, args.silent ? 0 : 1, &tau, err, sizeof err))
            die(err);
        tch_host_encoding enc;
        if (tch_encode_host(x.data(), nd.data(), (int)n, (int)L, tau, (int)threads, &enc, err, sizeof err)) die(err);
        log(fmt("Encoded in %.2fs: tau=%d, one-hot cols=%zu, rare equal pairs=%zu", now() - t, tau, enc.D,
                enc.n_rare));
        t = now();
        Sink sink{&upper, threads};
        int rare_gpu = 0;
        const int rc = tch_run((int)args.device, (int)n, enc.n_pad, enc.O, enc.K1, enc.P, enc.K2, enc.start, enc.js,
                               enc.n_rare, (int)stripe, on_stripe, &sink, &gpu_secs, &rare_gpu, err, sizeof err);
        tch_host_encoding_free(&enc);
        if (rc) die(fmt("CUDA: %s", err));
        log(fmt("Computed %zu x %zu matrix on tensor cores in %.2fs (GPU pipeline %.2fs, rare pairs on %s)", n, n,
                now() - t, gpu_secs, rare_gpu ? "GPU" : "host"));
    } else {
        // n < 2 or no loci: every distance is 0 and the GPU is not used (main.rs:466-470);
        // the reference still ranks the calls, which enforces its 65535-allele limit
        if (tsv) {
            CallMatrix(n * L).swap(calls);
            if (tch_tsv_calls(tsv, calls.data())) die("copying the parsed calls failed");
            tch_tsv_free(tsv);
            tsv = nullptr;
        }
        std::vector<uint16_t> x(n * L);
        std::vector<uint32_t> nd(L);
        if (tch_dense_ranks(calls.data(), (int)n, (int)L, x.data(), nd.data(), (int)threads, err, sizeof err))
            die(err);
        for (size_t i = 0; i < n; i++) upper[i].assign(n - 1 - i, 0);
    }

    // ---- write (main.rs:472-490)
    t = now();
    FILE* f = open_out();
    FileOut fo{f};
    if (gz) {
        tch_host::GzipWriter<FileOut> z(fo, 3);
        write_matrix(z, ids, upper, args.output_sep, args.index_name, args.layout, args.max_dist, threads);
        z.finish();
    } else {
        write_matrix(fo, ids, upper, args.output_sep, args.index_name, args.layout, args.max_dist, threads);
    }
    close_out(f);
    log(fmt("Wrote output in %.2fs. Total %.2fs", now() - t, now() - t_start));
    return 0;
}
