// Batched solves: many independent profile sets of uneven size, each set's
// whole upper triangle into its own region of one device buffer (no reference
// counterpart; the reference solves one matrix per run).
//
// Every set is encoded on the device once (tch_solver_from_calls; a tau of 0
// lets the learned model, when set, or the analytic model pick it per set).
// Two schedules, each captured once as a CUDA graph (per output buffer) and
// replayed on every later run; nothing is allocated inside the graph:
//
// * branches >= 1: every set's rare counts + tile pass (into one preallocated
//   rare-count block per stream) spread over `branches` streams forked from
//   the caller's stream (largest sets first, each to the branch with the least
//   work so far), so the small sets' kernels, which fill only a few SMs each,
//   run side by side;
// * branches == 0 (persistent): two launches for the whole batch, the rare
//   counts of every row of every set (one CTA per row, a row -> set table) into
//   one rare-count buffer, then one tile pass over every set's tiles (one CTA
//   per SM walking a tile -> set table, each set with its own tensor maps and
//   output).  Needs dense rare counts and sets of at most 65 536 rows.
//
// tch_batch_tune is the autotuner of that schedule: it times the graph for
// every schedule and keeps the fastest.

#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "tch_internal.cuh"

using namespace tch;

struct tch_batch {
    int device = 0;
    std::vector<tch_solver*> sets;
    std::vector<size_t> off;  // u16 elements: set s at off[s], n_s x ld_s; off.back() = total
    std::vector<size_t> ld;
    int branches = 8;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;  // branches + 1
    cudaStream_t origin = nullptr;  // the stream the fork / join is captured on
    std::vector<uint16_t*> rbuf;    // per branch: rare-count block of its largest set
    std::vector<size_t> rbytes;
    // persistent schedule: every set's rare-count block in one buffer, the
    // job tables of the two launches, the tile pass's error word
    uint16_t* pbuf = nullptr;
    size_t pbytes = 0;
    RareBatchPlan rplan;
    TcBatchPlan tplan;
    int* dErr = nullptr;
    int num_sms = 0;
    cudaGraphExec_t exec = nullptr;
    uint16_t* exec_out = nullptr;
    bool warmed = false;
};

namespace tch {
namespace {

void drop_graph(tch_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->exec_out = nullptr;
}

int ensure_streams(tch_batch* b, int branches, Err& e) {
    if (!b->origin) TCH_CK(e, cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
    while ((int)b->streams.size() < branches) {
        cudaStream_t st;
        TCH_CK(e, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        b->streams.push_back(st);
    }
    while ((int)b->events.size() < branches + 1) {
        cudaEvent_t ev;
        TCH_CK(e, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        b->events.push_back(ev);
    }
    return 0;
fail:
    return 1;
}

// Rare-count block of set s: n x up(n, 256) u16.
size_t rare_ld(int n) { return up((size_t)std::max(n, 1), kRareDenseAlign); }

int ensure_rbuf(tch_batch* b, int k, size_t bytes, Err& e) {
    while ((int)b->rbuf.size() <= k) b->rbuf.push_back(nullptr), b->rbytes.push_back(0);
    if (b->rbytes[k] >= bytes) return 0;
    cudaFree(b->rbuf[k]);
    b->rbuf[k] = nullptr;
    b->rbytes[k] = 0;
    TCH_CK(e, cudaMalloc(&b->rbuf[k], bytes));
    b->rbytes[k] = bytes;
    return 0;
fail:
    return 1;
}

// Largest rare-count buffer of the persistent schedule.
constexpr size_t kPersistentRareBytes = size_t(8) << 30;

// Whether the persistent schedule can run this batch (why not in *why).
bool persistent_ready(const tch_batch* b, const char** why) {
    size_t bytes = 0;
    for (tch_solver* sv : b->sets) {
        const int n = solver_size(sv);
        if (n < 2) continue;
        RareGroups g;
        if (!solver_operands(sv) || !solver_rare_groups(sv, &g)) {
            *why = "a set holds pair lists, not rare groups";
            return false;
        }
        if (rare_ld(n) > 65536) {
            *why = "a set has more than 65 536 rows";
            return false;
        }
        bytes += (size_t)n * rare_ld(n) * 2;
    }
    if (bytes > kPersistentRareBytes) {
        *why = "the rare counts of all sets exceed 8 GiB";
        return false;
    }
    return true;
}

// Job tables of the two persistent launches of the whole batch into d_out
// (device memory written here, before the capture).
int prepare_persistent(tch_batch* b, uint16_t* d_out, Err& e) {
    std::vector<int> order(b->sets.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(),
              [&](int x, int y) { return solver_work(b->sets[x]) > solver_work(b->sets[y]); });
    std::vector<size_t> roff(b->sets.size(), 0);
    size_t total = 0;
    for (int s : order) {
        const int n = solver_size(b->sets[s]);
        if (n < 2) continue;
        roff[s] = total;
        total += (size_t)n * rare_ld(n);
    }
    if (b->pbytes < total * 2) {
        cudaFree(b->pbuf);
        b->pbuf = nullptr;
        b->pbytes = 0;
        TCH_CK(e, cudaMalloc(&b->pbuf, total * 2));
        b->pbytes = total * 2;
    }
    if (!b->dErr) {
        TCH_CK(e, cudaMalloc(&b->dErr, sizeof(int)));
        TCH_CK(e, cudaMemset(b->dErr, 0, sizeof(int)));
    }
    {
        std::vector<RareBatchItem> ri;
        std::vector<TcBatchItem> ti;
        for (int s : order) {
            const int n = solver_size(b->sets[s]);
            if (n < 2) continue;
            RareBatchItem r;
            solver_rare_groups(b->sets[s], &r.g);
            r.R = b->pbuf + roff[s];
            r.ldr = rare_ld(n);
            ri.push_back(r);
            TcBatchItem t;
            t.ops = solver_operands(b->sets[s]);
            t.n = n;
            t.R = r.R;
            t.ldr = r.ldr;
            t.out = d_out + b->off[s];
            t.ldo = b->ld[s];
            ti.push_back(t);
        }
        TCH_CK(e, rare_batch_prepare(ri, &b->rplan));
        TCH_CK(e, tc_batch_prepare(ti, b->num_sms, &b->tplan, b->dErr));
    }
    return 0;
fail:
    return 1;
}

// One eager solve before the first capture, so one-time set-up (kernel
// attributes) never runs inside it.
int warm_up(tch_batch* b, uint16_t* d_out, Err& e) {
    int best = -1;
    for (size_t s = 0; s < b->sets.size(); s++)
        if (solver_size(b->sets[s]) > 1 && (best < 0 || solver_work(b->sets[s]) < solver_work(b->sets[best])))
            best = (int)s;
    if (best >= 0) {
            const int n = solver_size(b->sets[best]);
            if (ensure_rbuf(b, 0, (size_t)n * rare_ld(n) * 2, e)) return 1;
            if (solver_stripe_counts(b->sets[best], 0, n, d_out + b->off[best], b->ld[best], b->rbuf[0], rare_ld(n),
                                     b->origin, e))
                return 1;
        }
    TCH_CK(e, cudaStreamSynchronize(b->origin));
    b->warmed = true;
    return 0;
fail:
    return 1;
}

// Fork, every set's solve on its branch, join: captured into a graph.
int build_graph(tch_batch* b, uint16_t* d_out, Err& e) {
    cudaGraph_t graph = nullptr;
    cudaStream_t st = nullptr;
    const int nb = b->branches;
    std::vector<int> order(b->sets.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(),
              [&](int x, int y) { return solver_work(b->sets[x]) > solver_work(b->sets[y]); });
    std::vector<double> load(nb, 0.0);
    std::vector<int> branch(b->sets.size());
    std::vector<size_t> need(nb, 0);
    drop_graph(b);
    if (ensure_streams(b, std::max(nb, 1), e)) return 1;
    if (!b->warmed && warm_up(b, d_out, e)) return 1;
    st = b->origin;
    if (nb == 0) {
        const char* why = "";
        if (!persistent_ready(b, &why)) return e.set("persistent schedule unavailable: %s", why);
        if (!b->num_sms) TCH_CK(e, cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device));
        if (prepare_persistent(b, d_out, e)) return 1;
        TCH_CK(e, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        TCH_CK(e, launch_rare_batch(b->rplan, b->num_sms, st));
        TCH_CK(e, launch_tc_batch(b->tplan, st));
        TCH_CK(e, cudaStreamEndCapture(st, &graph));
        TCH_CK(e, cudaGraphInstantiate(&b->exec, graph, 0));
        cudaGraphDestroy(graph);
        b->exec_out = d_out;
        return 0;
    }
    // largest sets first, each to the least-loaded branch; one rare-count block
    // per branch, sized for its largest set (a branch runs its sets in order)
    for (int s : order) {
        const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[k] += solver_work(b->sets[s]);
        branch[s] = k;
        const int n = solver_size(b->sets[s]);
        need[k] = std::max(need[k], (size_t)n * rare_ld(n) * 2);
    }
    for (int k = 0; k < nb; k++)
        if (ensure_rbuf(b, k, need[k], e)) return 1;
    TCH_CK(e, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    TCH_CK(e, cudaEventRecord(b->events[nb], st));
    for (int k = 0; k < nb; k++) TCH_CK(e, cudaStreamWaitEvent(b->streams[k], b->events[nb], 0));
    for (int s : order) {
        const int k = branch[s], n = solver_size(b->sets[s]);
        if (n > 1 && solver_stripe_counts(b->sets[s], 0, n, d_out + b->off[s], b->ld[s], b->rbuf[k], rare_ld(n),
                                          b->streams[k], e))
            goto fail;
    }
    for (int k = 0; k < nb; k++) {
        TCH_CK(e, cudaEventRecord(b->events[k], b->streams[k]));
        TCH_CK(e, cudaStreamWaitEvent(st, b->events[k], 0));
    }
    TCH_CK(e, cudaStreamEndCapture(st, &graph));
    TCH_CK(e, cudaGraphInstantiate(&b->exec, graph, 0));
    cudaGraphDestroy(graph);
    b->exec_out = d_out;
    return 0;
fail:
    if (st) {
        cudaStreamCaptureStatus cs;
        if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
        }
    }
    if (graph) cudaGraphDestroy(graph);
    return 1;
}

int run(tch_batch* b, uint16_t* d_out, cudaStream_t st, Err& e) {
    if (!b->exec || b->exec_out != d_out)
        if (build_graph(b, d_out, e)) return 1;
    TCH_CK(e, cudaGraphLaunch(b->exec, st));
    return 0;
fail:
    return 1;
}

}  // namespace
}  // namespace tch

extern "C" {

int tch_batch_add(tch_batch* b, int n, int L, const uint64_t* calls, int tau, char* err, int errlen) {
    Err e{err, errlen};
    tch_solver* sv = nullptr;
    if (!b) return e.set("null batch");
    if (n < 1 || L < 1 || !calls) return e.set("need n >= 1, L >= 1 and calls (got n=%d, L=%d)", n, L);
    if (solver_from_calls(b->device, n, L, calls, tau, TCH_KERNEL_AUTO, false, &sv, e)) return 1;
    drop_graph(b);
    const size_t acc = b->off.back();
    b->sets.push_back(sv);
    b->ld.push_back(up((size_t)n, 8));
    b->off.push_back(acc + (size_t)n * up((size_t)n, 8));
    return 0;
}

int tch_batch_create(int device, int count, const int* n, const int* L, const uint64_t* const* calls, const int* tau,
                     tch_batch** out, char* err, int errlen) {
    Err e{err, errlen};
    if (!out || count < 0 || (count && (!n || !L || !calls))) return e.set("null argument");
    *out = nullptr;
    tch_batch* b = new tch_batch();
    b->device = device;
    b->off.push_back(0);
    for (int s = 0; s < count; s++)
        if (tch_batch_add(b, n[s], L[s], calls[s], tau ? tau[s] : 0, err, errlen)) {
            char msg[512];
            snprintf(msg, sizeof msg, "set %d: %s", s, err ? err : "");
            e.set("%s", msg);
            tch_batch_destroy(b);
            return 1;
        }
    *out = b;
    return 0;
}

int tch_batch_layout(const tch_batch* b, size_t* offsets, size_t* ld) {
    if (!b) return 1;
    for (size_t s = 0; s < b->sets.size(); s++) {
        if (offsets) offsets[s] = b->off[s];
        if (ld) ld[s] = b->ld[s];
    }
    if (offsets) offsets[b->sets.size()] = b->off.back();
    return 0;
}

int tch_batch_run(tch_batch* b, uint16_t* d_out, void* stream, char* err, int errlen) {
    Err e{err, errlen};
    if (!b || !d_out) return e.set("null argument");
    if (((uintptr_t)d_out & 15) != 0) return e.set("output pointer must be 16-byte aligned");
    if (cudaSetDevice(b->device) != cudaSuccess) return e.set("cudaSetDevice(%d) failed", b->device);
    return run(b, d_out, (cudaStream_t)stream, e);
}

int tch_batch_check(tch_batch* b, char* err, int errlen) {
    Err e{err, errlen};
    if (!b) return e.set("null batch");
    for (size_t s = 0; s < b->sets.size(); s++)
        if (solver_check(b->sets[s], e)) return 1;
    if (b->dErr) {  // the persistent tile pass
        int h = 0;
        TCH_CK(e, cudaSetDevice(b->device));
        TCH_CK(e, cudaMemcpy(&h, b->dErr, sizeof(int), cudaMemcpyDeviceToHost));
        if (h) {
            cudaMemset(b->dErr, 0, sizeof(int));
            return e.set("device reported error 0x%x in the batch's tile pass (%s%s)", h,
                         (h & DEVERR_OVERFLOW) ? "distance overflow " : "", (h & DEVERR_TIMEOUT) ? "wait timeout" : "");
        }
    }
    return 0;
fail:
    return 1;
}

int tch_batch_tune(tch_batch* b, uint16_t* d_out, void* stream, int reps, double* best_ms, int* best_branches,
                   char* err, int errlen) {
    Err e{err, errlen};
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    double best = 1e300;
    int bb = b ? b->branches : 8;
    const char* why = "";
    if (!b || !d_out) return e.set("null argument");
    if (cudaSetDevice(b->device) != cudaSuccess) return e.set("cudaSetDevice(%d) failed", b->device);
    const bool persistent = persistent_ready(b, &why);
    reps = std::max(reps, 1);
    TCH_CK(e, cudaEventCreate(&t0));
    TCH_CK(e, cudaEventCreate(&t1));
    for (int nb : {0, 1, 4, 8, 16, 32}) {
        if (nb == 0 && !persistent) continue;
        b->branches = nb;
        if (build_graph(b, d_out, e)) goto fail;
        TCH_CK(e, cudaGraphLaunch(b->exec, st));  // warm
        TCH_CK(e, cudaEventRecord(t0, st));
        for (int r = 0; r < reps; r++) TCH_CK(e, cudaGraphLaunch(b->exec, st));
        TCH_CK(e, cudaEventRecord(t1, st));
        TCH_CK(e, cudaEventSynchronize(t1));
        float ms = 0;
        TCH_CK(e, cudaEventElapsedTime(&ms, t0, t1));
        if (ms / reps < best) best = ms / reps, bb = nb;
    }
    b->branches = bb;
    if (build_graph(b, d_out, e)) goto fail;
    if (best_ms) *best_ms = best;
    if (best_branches) *best_branches = bb;
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    return 0;
fail:
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    return 1;
}

int tch_batch_set_schedule(tch_batch* b, int branches) {
    const char* why = "";
    if (!b || branches < 0 || branches > 64 || (branches == 0 && !persistent_ready(b, &why))) return 1;
    b->branches = branches;
    drop_graph(b);
    return 0;
}

int tch_batch_info(const tch_batch* b, int* count, int* taus, int* branches) {
    if (!b) return 1;
    if (count) *count = (int)b->sets.size();
    if (taus)
        for (size_t s = 0; s < b->sets.size(); s++) {
            tch_info info;
            tch_solver_info(b->sets[s], &info);
            taus[s] = info.tau;
        }
    if (branches) *branches = b->branches;
    return 0;
}

void tch_batch_destroy(tch_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    drop_graph(b);
    for (auto st : b->streams) cudaStreamDestroy(st);
    if (b->origin) cudaStreamDestroy(b->origin);
    for (auto p : b->rbuf) cudaFree(p);
    rare_batch_release(&b->rplan);
    tc_batch_release(&b->tplan);
    cudaFree(b->pbuf);
    cudaFree(b->dErr);
    for (auto ev : b->events) cudaEventDestroy(ev);
    for (auto s : b->sets) solver_free(s);
    delete b;
}

}  // extern "C"
