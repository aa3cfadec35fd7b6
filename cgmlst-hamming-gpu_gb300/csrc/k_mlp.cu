// The learned tau model: a small MLP, trained and evaluated by this file's
// kernels on the GPU.
//
// It predicts ln(milliseconds) of one whole-triangle solve (rare counts + tile
// pass) for a candidate tau from TCH_TAU_FEATURES features (dataset shape,
// allele-frequency quantiles, missing fraction, and the candidate's one-hot
// width, rare pairs, rare cells, GEMM work and analytic estimate).  The solver
// takes the candidate with the smallest prediction; tau only moves work
// between the contraction and the rare term, so exactness never depends on it.
//
// Shape F -> H -> H -> 1 with ReLU, fp32, parameters packed as
//   W1[F][H] | b1[H] | W2[H][H] | b2[H] | w3[H] | b3
// Training: full-batch mean squared error, Adam; one step = forward of every
// sample (one thread per sample, keeping what the backward pass needs), the
// gradient (one thread per parameter summing over the samples in order, so it
// is deterministic), Adam update.  The step is captured once as a CUDA graph
// and replayed.

#include <math.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "tch_internal.cuh"

namespace tch {
namespace {

constexpr int F = kMlpIn, H = kMlpHidden, NP = kMlpParams;
constexpr int OW1 = 0, OB1 = F * H, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + H;
static_assert(OB3 + 1 == NP, "parameter layout");
constexpr int MLP_THREADS = 128;

// Forward of one sample; z1, z2 keep the pre-activations for the backward pass.
__device__ __forceinline__ float mlp_forward(const float* w, const float* x, float (&z1)[H], float (&z2)[H]) {
#pragma unroll
    for (int j = 0; j < H; j++) {
        float a = w[OB1 + j];
#pragma unroll
        for (int k = 0; k < F; k++) a = fmaf(x[k], w[OW1 + k * H + j], a);
        z1[j] = a;
    }
#pragma unroll 4
    for (int j = 0; j < H; j++) {
        float a = w[OB2 + j];
#pragma unroll
        for (int k = 0; k < H; k++) a = fmaf(fmaxf(z1[k], 0.f), w[OW2 + k * H + j], a);
        z2[j] = a;
    }
    float p = w[OB3];
#pragma unroll
    for (int j = 0; j < H; j++) p = fmaf(fmaxf(z2[j], 0.f), w[OW3 + j], p);
    return p;
}

// Per-sample scratch of the backward pass: relu(z1), relu(z2), dL/dz2, dL/dz1,
// dL/dp and the squared error.
constexpr int SW = 4 * H + 2;
constexpr int SA1 = 0, SA2 = H, SD2 = 2 * H, SDZ1 = 3 * H, SGP = 4 * H, SE2 = 4 * H + 1;

// Forward of every sample (pred optional); with targets y, the per-sample
// quantities the gradient needs go to scratch.
__global__ void __launch_bounds__(MLP_THREADS)
    mlp_forward_kernel(const float* __restrict__ wg, const float* __restrict__ X, const float* __restrict__ y, int n,
                       float* pred, float* scratch) {
    __shared__ float w[NP];
    for (int q = threadIdx.x; q < NP; q += blockDim.x) w[q] = wg[q];
    __syncthreads();
    const float inv_n = 1.f / (float)max(n, 1);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        float x[F];
#pragma unroll
        for (int k = 0; k < F; k++) x[k] = X[(size_t)s * F + k];
        float z1[H], z2[H];
        const float p = mlp_forward(w, x, z1, z2);
        if (pred) pred[s] = p;
        if (!y) continue;
        float* sc = scratch + (size_t)s * SW;
        const float err = p - y[s];
        const float gp = 2.f * err * inv_n;  // d loss / d p
        sc[SGP] = gp;
        sc[SE2] = err * err;
        float d2[H];
#pragma unroll
        for (int j = 0; j < H; j++) {
            d2[j] = z2[j] > 0.f ? gp * w[OW3 + j] : 0.f;
            sc[SA2 + j] = fmaxf(z2[j], 0.f);
            sc[SD2 + j] = d2[j];
        }
#pragma unroll 4
        for (int k = 0; k < H; k++) {
            float d1 = 0.f;
#pragma unroll
            for (int j = 0; j < H; j++) d1 = fmaf(w[OW2 + k * H + j], d2[j], d1);
            sc[SA1 + k] = fmaxf(z1[k], 0.f);
            sc[SDZ1 + k] = z1[k] > 0.f ? d1 : 0.f;
        }
    }
}

// One thread per parameter (and one for the loss): the sum over samples, in
// sample order, so the gradient is deterministic.
__global__ void mlp_grad_kernel(const float* __restrict__ X, const float* __restrict__ scratch, int n, float* grad,
                                float* loss) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q > NP) return;
    float acc = 0.f;
    if (q < OB1) {  // W1[i][k]
        const int i = q / H, k = q % H;
        for (int s = 0; s < n; s++) acc = fmaf(X[(size_t)s * F + i], scratch[(size_t)s * SW + SDZ1 + k], acc);
    } else if (q < OW2) {  // b1[k]
        const int k = q - OB1;
        for (int s = 0; s < n; s++) acc += scratch[(size_t)s * SW + SDZ1 + k];
    } else if (q < OB2) {  // W2[k][j]
        const int k = (q - OW2) / H, j = (q - OW2) % H;
        for (int s = 0; s < n; s++)
            acc = fmaf(scratch[(size_t)s * SW + SA1 + k], scratch[(size_t)s * SW + SD2 + j], acc);
    } else if (q < OW3) {  // b2[j]
        const int j = q - OB2;
        for (int s = 0; s < n; s++) acc += scratch[(size_t)s * SW + SD2 + j];
    } else if (q < OB3) {  // w3[j]
        const int j = q - OW3;
        for (int s = 0; s < n; s++) acc = fmaf(scratch[(size_t)s * SW + SGP], scratch[(size_t)s * SW + SA2 + j], acc);
    } else if (q == OB3) {  // b3
        for (int s = 0; s < n; s++) acc += scratch[(size_t)s * SW + SGP];
    } else {  // the loss
        for (int s = 0; s < n; s++) acc += scratch[(size_t)s * SW + SE2];
        *loss = acc / (float)max(n, 1);
        return;
    }
    grad[q] = acc;
}

// Adam; *step counts the updates done so far (bias correction of update step+1).
__global__ void adam_kernel(float* w, const float* g, float* m, float* v, const int* step, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const int t = *step + 1;
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < NP; q += gridDim.x * blockDim.x) {
        const float gq = g[q];
        const float mq = b1 * m[q] + (1.f - b1) * gq;
        const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
        m[q] = mq;
        v[q] = vq;
        w[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
    }
}

__global__ void step_kernel(int* step) { *step += 1; }

int grid_for(int n) { return std::max(1, std::min((n + MLP_THREADS - 1) / MLP_THREADS, 1024)); }

std::mutex g_mlp_mu;
bool g_mlp_set = false;
float g_mlp_w[NP];

}  // namespace

int mlp_run(int device, const float* w, const float* X, const float* y, int n, float* pred, float* loss,
            float* grad, Err& e) {
    float *dw = nullptr, *dX = nullptr, *dy = nullptr, *dp = nullptr, *dl = nullptr, *dg = nullptr, *ds = nullptr;
    if (n < 0 || !w || (n > 0 && !X)) return e.set("mlp: bad arguments");
    TCH_CK(e, cudaSetDevice(device));
    TCH_CK(e, cudaMalloc(&dw, NP * 4));
    TCH_CK(e, cudaMalloc(&dX, std::max(n, 1) * (size_t)F * 4));
    TCH_CK(e, cudaMalloc(&dp, std::max(n, 1) * (size_t)4));
    TCH_CK(e, cudaMalloc(&dl, 4));
    TCH_CK(e, cudaMalloc(&dg, NP * 4));
    TCH_CK(e, cudaMemcpy(dw, w, NP * 4, cudaMemcpyHostToDevice));
    if (n) TCH_CK(e, cudaMemcpy(dX, X, (size_t)n * F * 4, cudaMemcpyHostToDevice));
    if (y) {
        TCH_CK(e, cudaMalloc(&dy, std::max(n, 1) * (size_t)4));
        TCH_CK(e, cudaMalloc(&ds, std::max(n, 1) * (size_t)SW * 4));
        if (n) TCH_CK(e, cudaMemcpy(dy, y, (size_t)n * 4, cudaMemcpyHostToDevice));
    }
    if (n) {
        mlp_forward_kernel<<<grid_for(n), MLP_THREADS>>>(dw, dX, dy, n, dp, ds);
        TCH_CK(e, cudaGetLastError());
    }
    if (y) {
        mlp_grad_kernel<<<(NP + 1 + 127) / 128, 128>>>(dX, ds, n, dg, dl);
        TCH_CK(e, cudaGetLastError());
    }
    TCH_CK(e, cudaDeviceSynchronize());
    if (pred && n) TCH_CK(e, cudaMemcpy(pred, dp, (size_t)n * 4, cudaMemcpyDeviceToHost));
    if (loss && y) TCH_CK(e, cudaMemcpy(loss, dl, 4, cudaMemcpyDeviceToHost));
    if (grad && y) TCH_CK(e, cudaMemcpy(grad, dg, NP * 4, cudaMemcpyDeviceToHost));
    cudaFree(dw); cudaFree(dX); cudaFree(dy); cudaFree(dp); cudaFree(dl); cudaFree(dg); cudaFree(ds);
    return 0;
fail:
    cudaFree(dw); cudaFree(dX); cudaFree(dy); cudaFree(dp); cudaFree(dl); cudaFree(dg); cudaFree(ds);
    return 1;
}

int mlp_train(int device, float* w, const float* X, const float* y, int n, int steps, float lr, float* loss_out,
              Err& e) {
    float *dw = nullptr, *dX = nullptr, *dy = nullptr, *dl = nullptr, *dg = nullptr, *dm = nullptr, *dv = nullptr;
    float* ds = nullptr;
    int* dstep = nullptr;
    cudaStream_t st = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (n <= 0 || steps < 0 || !w || !X || !y || !(lr > 0)) return e.set("mlp: bad training arguments");
    TCH_CK(e, cudaSetDevice(device));
    TCH_CK(e, cudaMalloc(&dw, NP * 4));
    TCH_CK(e, cudaMalloc(&dg, NP * 4));
    TCH_CK(e, cudaMalloc(&dm, NP * 4));
    TCH_CK(e, cudaMalloc(&dv, NP * 4));
    TCH_CK(e, cudaMalloc(&dX, (size_t)n * F * 4));
    TCH_CK(e, cudaMalloc(&dy, (size_t)n * 4));
    TCH_CK(e, cudaMalloc(&ds, (size_t)n * SW * 4));
    TCH_CK(e, cudaMalloc(&dl, 4));
    TCH_CK(e, cudaMalloc(&dstep, 4));
    TCH_CK(e, cudaMemcpy(dw, w, NP * 4, cudaMemcpyHostToDevice));
    TCH_CK(e, cudaMemcpy(dX, X, (size_t)n * F * 4, cudaMemcpyHostToDevice));
    TCH_CK(e, cudaMemcpy(dy, y, (size_t)n * 4, cudaMemcpyHostToDevice));
    TCH_CK(e, cudaMemset(dm, 0, NP * 4));
    TCH_CK(e, cudaMemset(dv, 0, NP * 4));
    TCH_CK(e, cudaMemset(dstep, 0, 4));
    TCH_CK(e, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    // one optimisation step as a graph: forward, gradient, Adam, count
    TCH_CK(e, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    mlp_forward_kernel<<<grid_for(n), MLP_THREADS, 0, st>>>(dw, dX, dy, n, nullptr, ds);
    mlp_grad_kernel<<<(NP + 1 + 127) / 128, 128, 0, st>>>(dX, ds, n, dg, dl);
    adam_kernel<<<(NP + 255) / 256, 256, 0, st>>>(dw, dg, dm, dv, dstep, lr);
    step_kernel<<<1, 1, 0, st>>>(dstep);
    TCH_CK(e, cudaStreamEndCapture(st, &graph));
    TCH_CK(e, cudaGraphInstantiate(&exec, graph, 0));
    for (int s = 0; s < steps; s++) TCH_CK(e, cudaGraphLaunch(exec, st));
    // the loss of the final weights
    mlp_forward_kernel<<<grid_for(n), MLP_THREADS, 0, st>>>(dw, dX, dy, n, nullptr, ds);
    mlp_grad_kernel<<<(NP + 1 + 127) / 128, 128, 0, st>>>(dX, ds, n, dg, dl);
    TCH_CK(e, cudaGetLastError());
    TCH_CK(e, cudaStreamSynchronize(st));
    TCH_CK(e, cudaMemcpy(w, dw, NP * 4, cudaMemcpyDeviceToHost));
    if (loss_out) TCH_CK(e, cudaMemcpy(loss_out, dl, 4, cudaMemcpyDeviceToHost));
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    cudaStreamDestroy(st);
    cudaFree(dw); cudaFree(dX); cudaFree(dy); cudaFree(dl); cudaFree(dg); cudaFree(dm); cudaFree(dv);
    cudaFree(ds); cudaFree(dstep);
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
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (st) cudaStreamDestroy(st);
    cudaFree(dw); cudaFree(dX); cudaFree(dy); cudaFree(dl); cudaFree(dg); cudaFree(dm); cudaFree(dv);
    cudaFree(ds); cudaFree(dstep);
    return 1;
}

bool tau_mlp_weights(float* out) {
    std::lock_guard<std::mutex> lk(g_mlp_mu);
    if (!g_mlp_set) return false;
    memcpy(out, g_mlp_w, sizeof(g_mlp_w));
    return true;
}

}  // namespace tch

using namespace tch;

extern "C" {

int tch_mlp_init(float* w, uint64_t seed) {
    if (!w) return 1;
    // He-normal weights from a splitmix64 stream (Box-Muller), zero biases
    uint64_t s = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&s]() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto normal = [&]() {
        const double u1 = ((next() >> 11) + 1.0) / 9007199254740993.0, u2 = (next() >> 11) / 9007199254740992.0;
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    };
    for (int q = 0; q < NP; q++) w[q] = 0.f;
    for (int q = 0; q < F * H; q++) w[OW1 + q] = (float)(normal() * sqrt(2.0 / F));
    for (int q = 0; q < H * H; q++) w[OW2 + q] = (float)(normal() * sqrt(2.0 / H));
    for (int q = 0; q < H; q++) w[OW3 + q] = (float)(normal() * sqrt(1.0 / H));
    return 0;
}

int tch_mlp_train(int device, float* w, const float* X, const float* y, int n, int steps, float lr, float* loss,
                  char* err, int errlen) {
    Err e{err, errlen};
    return mlp_train(device, w, X, y, n, steps, lr, loss, e);
}

int tch_mlp_predict(int device, const float* w, const float* X, int n, float* y, char* err, int errlen) {
    Err e{err, errlen};
    if (n > 0 && !y) return e.set("null output");
    return mlp_run(device, w, X, nullptr, n, y, nullptr, nullptr, e);
}

int tch_mlp_loss_grad(int device, const float* w, const float* X, const float* y, int n, float* loss, float* grad,
                      char* err, int errlen) {
    Err e{err, errlen};
    if (!y && n > 0) return e.set("null targets");
    return mlp_run(device, w, X, y, n, nullptr, loss, grad, e);
}

int tch_set_tau_mlp(const float* w) {
    std::lock_guard<std::mutex> lk(g_mlp_mu);
    if (!w) {
        g_mlp_set = false;
        return 0;
    }
    for (int q = 0; q < NP; q++)
        if (!isfinite(w[q])) return 1;
    memcpy(g_mlp_w, w, sizeof(g_mlp_w));
    g_mlp_set = true;
    return 0;
}

}  // extern "C"
