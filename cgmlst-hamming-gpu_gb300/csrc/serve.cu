// Serving: a profile database resident in HBM and query batches of new
// profiles against it (no reference counterpart; the reference computes one
// matrix per run).
//
// tch_db holds the database encoded on the device (operand rows, rare groups
// including single-row groups, and the maps that encode new profiles like the
// database's own: ids in rank order per locus, frequent column per allele).
// A query batch of m new profiles runs on the caller's stream, allocating only
// from a stream-ordered pool:
//   ranks      each id looked up in its locus's sorted ids (new ids -> novel)
//   operand    packed fp4 rows in the database's column layout (presence +
//              frequent one-hot, the A side of the tile pass; a novel id is
//              present but matches nothing); the database keeps only its
//              B-side copy (one-hot columns negated)
//   rare       u16 counts of rare equal alleles against every database row
//   tile pass  the tcgen05 kernel over the m x n rectangle, subtracting them
//   q x q      the batch's own upper triangle by a direct count on the calls
//              (ids compared as given; 0 = missing)
// Every distance is exact; the database's tau only decides which alleles go
// through the one-hot columns and which through the rare counts.
//
// tch_server runs query batches from many callers: a FIFO of requests, a set
// of worker threads with one stream each (the slots), and admission by device
// memory: a request starts when its estimated bytes fit in the budget next to
// the requests already running, so batches that arrive while others are on the
// GPU overlap with them.

#include <math.h>
#include <string.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "tch_internal.cuh"

namespace tch {
namespace {

__global__ void query_rank_kernel(const uint64_t* __restrict__ q, int m, int L, const uint64_t* __restrict__ cnt_off,
                                  const uint64_t* __restrict__ slot_ids, uint32_t* xq) {
    const size_t total = (size_t)m * L;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t % L);
        const uint64_t v = q[t];
        uint32_t r = 0;
        if (v) {
            // ids of locus k ascend at slots cnt_off[k] + 1 .. cnt_off[k + 1] - 1
            uint64_t lo = cnt_off[k] + 1, hi = cnt_off[k + 1];
            while (lo < hi) {
                const uint64_t mid = lo + (hi - lo) / 2;
                if (slot_ids[mid] < v) lo = mid + 1; else hi = mid;
            }
            r = (lo < cnt_off[k + 1] && slot_ids[lo] == v) ? (uint32_t)(lo - cnt_off[k]) : kNovelRank;
        }
        xq[t] = r;
    }
}

// +1.0 at column col of row `row` (zeroed before); two columns of one byte
// belong to different cells, hence the atomic OR on the word.
__device__ __forceinline__ void set_fp4_one(const KChunks& X, size_t row, size_t col) {
    uint32_t* w = reinterpret_cast<uint32_t*>(X.at(row, (int)((col >> 1) & ~(size_t)3)));
    atomicOr(w, kFp4One << (4 * (col & 7)));
}

__global__ void query_pack_kernel(const uint32_t* __restrict__ xq, int m, int L, const uint64_t* __restrict__ cnt_off,
                                  const int32_t* __restrict__ col, const uint32_t* __restrict__ base, KChunks X) {
    const size_t total = (size_t)m * L;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t a = xq[t];
        if (!a) continue;
        const size_t i = t / L;
        const int k = (int)(t % L);
        set_fp4_one(X, i, (size_t)k);
        if (a == kNovelRank) continue;
        const int32_t c = col[cnt_off[k] + a];
        if (c >= 0) set_fp4_one(X, i, (size_t)L + base[k] + (size_t)c);
    }
}

// Direct count of the batch's own pairs: 16 x 16 pairs per block, the calls of
// the two row groups staged in shared memory 64 loci at a time.
constexpr int QQ_T = 16, QQ_K = 64;
__global__ void qq_kernel(const uint64_t* __restrict__ q, int m, int L, uint16_t* out, size_t ldo) {
    const int a0 = blockIdx.y * QQ_T, b0 = blockIdx.x * QQ_T;
    if (b0 + QQ_T - 1 < a0) return;  // entirely below the diagonal
    __shared__ uint64_t A[QQ_T][QQ_K + 1], B[QQ_T][QQ_K + 1];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * QQ_T + tx;
    uint32_t d = 0;
    for (int k0 = 0; k0 < L; k0 += QQ_K) {
        const int kn = min(QQ_K, L - k0);
        for (int e = tid; e < QQ_T * QQ_K; e += QQ_T * QQ_T) {
            const int r = e / QQ_K, k = e % QQ_K;
            A[r][k] = (a0 + r < m && k < kn) ? q[(size_t)(a0 + r) * L + k0 + k] : 0;
            B[r][k] = (b0 + r < m && k < kn) ? q[(size_t)(b0 + r) * L + k0 + k] : 0;
        }
        __syncthreads();
        for (int k = 0; k < kn; k++) {
            const uint64_t x = A[ty][k], y = B[tx][k];
            d += (x != 0) & (y != 0) & (x != y);
        }
        __syncthreads();
    }
    const int a = a0 + ty, b = b0 + tx;
    if (a < m && b < m && b > a) out[(size_t)a * ldo + b] = (uint16_t)d;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace
}  // namespace tch

using namespace tch;

struct tch_db {
    int device = 0, n = 0, L = 0, sms = 0;
    DeviceEncoding enc;
    cudaMemPool_t pool = nullptr;
};

namespace tch {
namespace {

size_t query_bytes(const tch_db* db, int m) {
    const size_t mr = up((size_t)std::max(m, 1), 256);
    return (size_t)m * db->L * 12 + mr * (size_t)db->enc.kb + (size_t)m * up((size_t)db->n, kRareDenseAlign) * 2 +
           (size_t)m * up((size_t)db->n, 8) * 2 + (size_t)m * up((size_t)m, 8) * 2 + (1u << 20);
}

int db_query(tch_db* db, int m, const uint64_t* qcalls, uint16_t* h_qdb, uint16_t* h_qq, cudaStream_t st, Err& e) {
    const int n = db->n, L = db->L;
    const DeviceEncoding& enc = db->enc;
    const size_t mr = up((size_t)std::max(m, 1), 256);
    const size_t ldr = up((size_t)n, kRareDenseAlign), ldo = up((size_t)n, 8), ldq = up((size_t)m, 8);
    uint64_t* dq = nullptr;
    uint32_t* xq = nullptr;
    uint16_t *R = nullptr, *out = nullptr, *qq = nullptr;
    int* derr = nullptr;
    Fp4Operands QX;  // the batch's A-side rows: the database's K layout, m rows
    QX.pos = enc.X.neg;
    for (int c = 0; c < kMaxKChunks; c++) QX.pos.p[c] = nullptr;
    QX.n_rows = mr;
    QX.kb = enc.kb;
    KChunks& X = QX.pos;
    cudaError_t ce = cudaSuccess;
    // TCH_VERBOSE=1: device time of each phase on stderr
    const char* vb = getenv("TCH_VERBOSE");
    const bool verbose = vb && vb[0] == '1';
    cudaEvent_t ev[8] = {};
    int nev = 0;
    auto mark = [&]() {
        if (verbose && nev < 8 && cudaEventCreate(&ev[nev]) == cudaSuccess) cudaEventRecord(ev[nev++], st);
    };
    auto alloc = [&](void** p, size_t bytes) {
        if (ce == cudaSuccess) ce = cudaMallocFromPoolAsync(p, std::max<size_t>(bytes, 16), db->pool, st);
    };
    if (m <= 0) return e.set("empty query batch");
    if (!qcalls) return e.set("null query calls");
    if (cudaSetDevice(db->device) != cudaSuccess) return e.set("cudaSetDevice(%d) failed", db->device);
    alloc((void**)&dq, (size_t)m * L * 8);
    alloc((void**)&xq, (size_t)m * L * 4);
    alloc((void**)&derr, 4);
    for (int c = 0; c < X.n; c++) alloc((void**)&X.p[c], mr * (size_t)X.width_of(c));
    if (h_qdb) {
        alloc((void**)&R, (size_t)m * ldr * 2);
        alloc((void**)&out, (size_t)m * ldo * 2);
    }
    if (h_qq && m > 1) alloc((void**)&qq, (size_t)m * ldq * 2);
    if (ce != cudaSuccess) goto done;
    mark();
    ce = cudaMemcpyAsync(dq, qcalls, (size_t)m * L * 8, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(derr, 0, 4, st);
    if (ce != cudaSuccess) goto done;
    {
        const int grid = (int)std::min<size_t>(((size_t)m * L + 255) / 256, (size_t)db->sms * 16);
        if (h_qdb) {
            for (int c = 0; c < X.n && ce == cudaSuccess; c++)
                ce = cudaMemsetAsync(X.p[c], 0, mr * (size_t)X.width_of(c), st);
            if (ce != cudaSuccess) goto done;
            mark();
            query_rank_kernel<<<grid, 256, 0, st>>>(dq, m, L, enc.cnt_off, enc.slot_ids, xq);
            query_pack_kernel<<<grid, 256, 0, st>>>(xq, m, L, enc.cnt_off, enc.col, enc.base, X);
            ce = cudaGetLastError();
            if (ce != cudaSuccess) goto done;
            RareGroups g;
            g.x = enc.x;
            g.cnt_off = enc.cnt_off;
            g.goff = enc.goff;
            g.members = enc.members;
            g.mpos = enc.mpos;
            g.n = n;
            g.L = L;
            mark();
            ce = launch_rare_query(g, xq, m, R, ldr, db->sms, st);
            mark();
            if (ce != cudaSuccess) goto done;
            StripeArgs a;
            a.n = n;
            a.r0 = 0;
            a.rows = m;
            a.out = out;
            a.ldo = ldo;
            a.err = derr;
            a.rect = true;
            ce = launch_tc_stripe(QX, &enc.X, R, ldr, a, db->sms, st);
            if (ce != cudaSuccess) goto done;
            mark();
            // one linear copy when the rows are packed (ldo == n), a pitched one otherwise
            ce = ldo == (size_t)n ? cudaMemcpyAsync(h_qdb, out, (size_t)m * n * 2, cudaMemcpyDeviceToHost, st)
                                  : cudaMemcpy2DAsync(h_qdb, (size_t)n * 2, out, ldo * 2, (size_t)n * 2, m,
                                                      cudaMemcpyDeviceToHost, st);
            if (ce != cudaSuccess) goto done;
        }
        if (qq) {
            mark();
            const dim3 blk(QQ_T, QQ_T), grd((m + QQ_T - 1) / QQ_T, (m + QQ_T - 1) / QQ_T);
            qq_kernel<<<grd, blk, 0, st>>>(dq, m, L, qq, ldq);
            ce = cudaGetLastError();
            if (ce == cudaSuccess)
                ce = ldq == (size_t)m ? cudaMemcpyAsync(h_qq, qq, (size_t)m * m * 2, cudaMemcpyDeviceToHost, st)
                                      : cudaMemcpy2DAsync(h_qq, (size_t)m * 2, qq, ldq * 2, (size_t)m * 2, m,
                                                          cudaMemcpyDeviceToHost, st);
            if (ce != cudaSuccess) goto done;
        }
    }
done:
    {
        int herr = 0;
        if (derr && ce == cudaSuccess) ce = cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st);
        for (void* p : {(void*)dq, (void*)xq, (void*)R, (void*)out, (void*)qq, (void*)derr})
            if (p) cudaFreeAsync(p, st);
        for (int c = 0; c < X.n; c++)
            if (X.p[c]) cudaFreeAsync(X.p[c], st);
        mark();
        const cudaError_t se = cudaStreamSynchronize(st);
        if (ce == cudaSuccess) ce = se;
        if (nev > 1) {
            static const char* names[] = {"h2d", "rank+pack", "rare counts", "tile pass", "d2h", "q x q + d2h", "",
                                          ""};
            fprintf(stderr, "tch query m=%d:", m);
            for (int k = 0; k + 1 < nev; k++) {
                float ms = 0;
                cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
                fprintf(stderr, " %s %.2f ms", names[k], ms);
            }
            fprintf(stderr, "\n");
        }
        for (int k = 0; k < nev; k++) cudaEventDestroy(ev[k]);
        if (ce != cudaSuccess) return e.set("query batch: %s", cudaGetErrorString(ce));
        if (herr) return e.set("query batch: device reported error 0x%x", herr);
    }
    return 0;
}

struct Request {
    int64_t id = 0;
    int m = 0;
    const uint64_t* q = nullptr;
    uint16_t* h_qdb = nullptr;
    uint16_t* h_qq = nullptr;
    size_t bytes = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    bool done = false;
    int rc = 0;
    char err[256] = {0};
};

}  // namespace
}  // namespace tch

struct tch_server {
    tch_db* db = nullptr;
    size_t budget = 0, in_use = 0;
    int running = 0;
    bool stop = false;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> queue;
    std::map<int64_t, Request*> reqs;
    int64_t next_id = 1;
    std::vector<std::thread> workers;
};

namespace tch {
namespace {

void worker_loop(tch_server* sv) {
    cudaSetDevice(sv->db->device);
    cudaStream_t st = nullptr;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            // FIFO; the head starts when it fits next to the running requests
            // (or alone, whatever its size)
            sv->cv.wait(lk, [&] {
                return sv->stop ||
                       (!sv->queue.empty() && (sv->running == 0 || sv->in_use + sv->queue.front()->bytes <= sv->budget));
            });
            if (sv->stop && sv->queue.empty()) break;
            r = sv->queue.front();
            sv->queue.pop_front();
            sv->in_use += r->bytes;
            sv->running++;
            r->t_start = now_s();
        }
        Err e{r->err, (int)sizeof(r->err)};
        const int rc = db_query(sv->db, r->m, r->q, r->h_qdb, r->h_qq, st, e);
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->in_use -= r->bytes;
            sv->running--;
            r->rc = rc;
            r->t_done = now_s();
            r->done = true;
        }
        sv->cv.notify_all();
    }
    if (st) cudaStreamDestroy(st);
}

}  // namespace
}  // namespace tch

extern "C" {

int tch_db_create(int device, int n, int L, const uint64_t* calls, int tau, tch_db** out, char* err, int errlen) {
    Err e{err, errlen};
    uint64_t* d_calls = nullptr;
    tch_db* db = nullptr;
    if (!out) return e.set("null output handle");
    *out = nullptr;
    if (n < 1 || L < 1) return e.set("the database needs n >= 1 profiles and L >= 1 loci (got n=%d, L=%d)", n, L);
    if (L > 65535) return e.set("more than 65535 loci (u16 distances)");
    if (!calls) return e.set("null input buffer");
    db = new tch_db();
    db->device = device;
    db->n = n;
    db->L = L;
    {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        uint64_t keep = ~0ull;
        TCH_CK(e, cudaSetDevice(device));
        TCH_CK(e, cudaDeviceGetAttribute(&db->sms, cudaDevAttrMultiProcessorCount, device));
        TCH_CK(e, cudaMemPoolCreate(&db->pool, &props));
        TCH_CK(e, cudaMemPoolSetAttribute(db->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    TCH_CK(e, cudaMalloc(&d_calls, (size_t)n * L * 8));
    TCH_CK(e, cudaMemcpy(d_calls, calls, (size_t)n * L * 8, cudaMemcpyHostToDevice));
    {
        TauModel model;
        if (encode_on_device(device, n, L, d_calls, tau, model, false, max_chunk_bytes(), ENC_QUERY, &db->enc, e))
            goto fail;
    }
    cudaFree(d_calls);
    // the database's own triangle is not served: drop its ranks and positions,
    // and its A-side operand copy (queries are the A side)
    cudaFree(db->enc.x);
    cudaFree(db->enc.mpos);
    db->enc.bytes -= (size_t)n * L * 6;
    db->enc.x = nullptr;
    db->enc.mpos = nullptr;
    for (int c = 0; c < kMaxKChunks; c++)
        if (db->enc.X.pos.p[c]) {
            cudaFree(db->enc.X.pos.p[c]);
            db->enc.X.pos.p[c] = nullptr;
            db->enc.bytes -= db->enc.x_rows * (size_t)db->enc.X.pos.width_of(c);
        }
    *out = db;
    return 0;
fail:
    if (d_calls) cudaFree(d_calls);
    if (db) {
        if (db->pool) cudaMemPoolDestroy(db->pool);
        delete db;
    }
    return 1;
}

void* tch_host_alloc(size_t bytes) {
    void* p = nullptr;
    return cudaMallocHost(&p, std::max<size_t>(bytes, 16)) == cudaSuccess ? p : nullptr;
}

void tch_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

void tch_db_destroy(tch_db* db) {
    if (!db) return;
    cudaSetDevice(db->device);
    cudaDeviceSynchronize();
    free_device_encoding(&db->enc);
    if (db->pool) cudaMemPoolDestroy(db->pool);
    delete db;
}

int tch_db_info(const tch_db* db, int* n, int* L, int* tau, size_t* d_onehot, size_t* device_bytes, int* k_chunks) {
    if (!db) return 1;
    if (k_chunks) *k_chunks = db->enc.X.neg.n;
    if (n) *n = db->n;
    if (L) *L = db->L;
    if (tau) *tau = db->enc.tau;
    if (d_onehot) *d_onehot = db->enc.D;
    if (device_bytes) *device_bytes = db->enc.bytes;
    return 0;
}

size_t tch_db_query_bytes(const tch_db* db, int m) { return db && m > 0 ? query_bytes(db, m) : 0; }

int tch_db_query(tch_db* db, int m, const uint64_t* qcalls, uint16_t* qdb, uint16_t* qq, void* stream, char* err,
                 int errlen) {
    Err e{err, errlen};
    if (!db) return e.set("null database");
    return db_query(db, m, qcalls, qdb, qq, (cudaStream_t)stream, e);
}

int tch_server_create(tch_db* db, int slots, size_t budget, tch_server** out, char* err, int errlen) {
    Err e{err, errlen};
    if (!db || !out) return e.set("null argument");
    if (slots < 1 || slots > 64) return e.set("slots must be in [1, 64] (got %d)", slots);
    tch_server* sv = new tch_server();
    sv->db = db;
    if (!budget) {
        size_t f = 0, t = 0;
        cudaSetDevice(db->device);
        cudaMemGetInfo(&f, &t);
        budget = f / 2;
    }
    sv->budget = budget;
    for (int s = 0; s < slots; s++) sv->workers.emplace_back(worker_loop, sv);
    *out = sv;
    return 0;
}

int64_t tch_server_submit(tch_server* sv, int m, const uint64_t* qcalls, uint16_t* qdb, uint16_t* qq) {
    if (!sv || m <= 0 || !qcalls) return -1;
    Request* r = new Request();
    r->m = m;
    r->q = qcalls;
    r->h_qdb = qdb;
    r->h_qq = qq;
    r->bytes = query_bytes(sv->db, m);
    r->t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        r->id = sv->next_id++;
        sv->reqs[r->id] = r;
        sv->queue.push_back(r);
    }
    sv->cv.notify_all();
    return r->id;
}

int tch_server_wait(tch_server* sv, int64_t id, double* queued_s, double* latency_s, char* err, int errlen) {
    Err e{err, errlen};
    if (!sv) return e.set("null server");
    Request* r = nullptr;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        auto it = sv->reqs.find(id);
        if (it == sv->reqs.end()) return e.set("unknown request %lld", (long long)id);
        r = it->second;
        // claimed before the wait releases the lock: a second wait on the
        // same id finds it unknown instead of sharing (and deleting) it
        sv->reqs.erase(it);
        sv->cv.wait(lk, [&] { return r->done; });
    }
    if (queued_s) *queued_s = r->t_start - r->t_submit;
    if (latency_s) *latency_s = r->t_done - r->t_submit;
    const int rc = r->rc;
    if (rc) e.set("%s", r->err);
    delete r;
    return rc;
}

void tch_server_destroy(tch_server* sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv.notify_all();
    for (auto& t : sv->workers) t.join();
    for (auto& kv : sv->reqs) delete kv.second;
    delete sv;
}

}  // extern "C"
