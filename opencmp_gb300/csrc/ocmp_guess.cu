// Learned Krylov initial guess (sm_103a): a small per-dof MLP, its training kernels and the
// feature/guess kernels around it. No counterpart in the reference: OpenCMP starts CG/GMRes from
// the previous step's solution (opencmp/models/base_model.py:925-937), which stays the fallback.
//
// Network: y = w3 . tanh(W2 tanh(W1 x + b1) + b2) + b3 + c . x, x in R^F (F <= 8), hidden width
// H = 32, FP32; the linear skip c . x makes polynomial extrapolation in time exactly representable.
// Per dof, x holds the last solution differences and the Jacobi-scaled residual of the previous-step
// guess, all divided by the norm of that dof's differences; y predicts (u^{n+1} - u^n) / that norm.
//
// Training is deterministic: the weight gradients are sums over rows done in two fixed-order stages
// (per-block partial sums in shared memory, then one pass over the blocks), followed by an Adam step.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "ocmp_internal.h"
#include "ocmp_spmv.cuh"

namespace ocmp {
namespace {

constexpr int kH = 32;
constexpr int kMaxF = 8;
constexpr int kRowsPerBlock = 256;

struct Layout {
    int F;
    int W1, b1, W2, b2, w3, b3, c, n;  // offsets into the flat parameter vector; c = linear skip
};
__host__ __device__ inline Layout layout(int F) {
    Layout L;
    L.F = F;
    L.W1 = 0;
    L.b1 = L.W1 + kH * F;
    L.W2 = L.b1 + kH;
    L.b2 = L.W2 + kH * kH;
    L.w3 = L.b2 + kH;
    L.b3 = L.w3 + kH;
    L.c = L.b3 + 1;
    L.n = L.c + F;
    return L;
}

// forward of one row; h1, h2 returned for the backward pass
__device__ __forceinline__ float mlp_row(const float* __restrict__ P, const Layout& L, const float* x, float* h1,
                                         float* h2) {
#pragma unroll
    for (int j = 0; j < kH; j++) {
        float a = P[L.b1 + j];
        for (int f = 0; f < L.F; f++) a = fmaf(P[L.W1 + j * L.F + f], x[f], a);
        h1[j] = tanhf(a);
    }
#pragma unroll
    for (int j = 0; j < kH; j++) {
        float a = P[L.b2 + j];
#pragma unroll
        for (int k = 0; k < kH; k++) a = fmaf(P[L.W2 + j * kH + k], h1[k], a);
        h2[j] = tanhf(a);
    }
    float y = P[L.b3];
#pragma unroll
    for (int j = 0; j < kH; j++) y = fmaf(P[L.w3 + j], h2[j], y);
    for (int f = 0; f < L.F; f++) y = fmaf(P[L.c + f], x[f], y);
    return y;
}

__global__ void __launch_bounds__(kRowsPerBlock) mlp_forward_kernel(int64_t rows, int F, const float* __restrict__ Pg,
                                                                    const float* __restrict__ X, float* __restrict__ Y) {
    extern __shared__ float P[];
    const Layout L = layout(F);
    for (int k = threadIdx.x; k < L.n; k += blockDim.x) P[k] = Pg[k];
    __syncthreads();
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    float x[kMaxF], h1[kH], h2[kH];
    for (int f = 0; f < F; f++) x[f] = X[r * F + f];
    Y[r] = mlp_row(P, L, x, h1, h2);
}

// Per row: forward, loss term (y - t)^2 / rows and the row's gradients; the block sums its rows'
// parameter gradients in shared memory in row order (thread 0 walks the rows), then writes one
// partial gradient vector per block. Loss partials likewise.
__global__ void __launch_bounds__(kRowsPerBlock) mlp_grad_partial_kernel(int64_t rows, int F,
                                                                         const float* __restrict__ Pg,
                                                                         const float* __restrict__ X,
                                                                         const float* __restrict__ T,
                                                                         float* __restrict__ Gpart,
                                                                         double* __restrict__ Lpart) {
    extern __shared__ double smd[];
    const Layout L = layout(F);
    double* sloss = smd;                 // blockDim (first: 8-byte aligned)
    float* P = reinterpret_cast<float*>(smd + kRowsPerBlock);  // n
    float* sh1 = P + L.n;                // blockDim x H   (hidden 1 of each row)
    float* sd2 = sh1 + kRowsPerBlock * kH;  // blockDim x H (delta at layer 2 pre-activation)
    float* sd1 = sd2 + kRowsPerBlock * kH;  // blockDim x H (delta at layer 1 pre-activation)
    float* sx = sd1 + kRowsPerBlock * kH;   // blockDim x F
    float* sdy = sx + kRowsPerBlock * kMaxF;  // blockDim
    float* sh2 = sdy + kRowsPerBlock;       // blockDim x H
    for (int k = threadIdx.x; k < L.n; k += blockDim.x) P[k] = Pg[k];
    __syncthreads();
    const int tid = threadIdx.x;
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + tid;
    const bool valid = r < rows;
    float x[kMaxF], h1[kH], h2[kH];
    float dy = 0.f;
    if (valid) {
        for (int f = 0; f < F; f++) x[f] = X[r * F + f];
        const float y = mlp_row(P, L, x, h1, h2);
        const float e = y - T[r];
        dy = 2.f * e / (float)rows;
        sdy[tid] = dy;
        sloss[tid] = (double)e * (double)e / (double)rows;
        float d2[kH];
#pragma unroll
        for (int j = 0; j < kH; j++) d2[j] = dy * P[L.w3 + j] * (1.f - h2[j] * h2[j]);
#pragma unroll
        for (int k = 0; k < kH; k++) {
            float a = 0.f;
#pragma unroll
            for (int j = 0; j < kH; j++) a = fmaf(P[L.W2 + j * kH + k], d2[j], a);
            sd1[tid * kH + k] = a * (1.f - h1[k] * h1[k]);
        }
#pragma unroll
        for (int j = 0; j < kH; j++) {
            sh1[tid * kH + j] = h1[j];
            sh2[tid * kH + j] = h2[j];
            sd2[tid * kH + j] = d2[j];
        }
        for (int f = 0; f < F; f++) sx[tid * kMaxF + f] = x[f];
    } else {
        sdy[tid] = 0.f;
        sloss[tid] = 0.0;
#pragma unroll
        for (int j = 0; j < kH; j++) {
            sh1[tid * kH + j] = 0.f;
            sh2[tid * kH + j] = 0.f;
            sd2[tid * kH + j] = 0.f;
            sd1[tid * kH + j] = 0.f;
        }
        for (int f = 0; f < F; f++) sx[tid * kMaxF + f] = 0.f;
    }
    __syncthreads();
    if (tid == 0) {
        double ls = 0;
        for (int q = 0; q < kRowsPerBlock; q++) ls += sloss[q];
        Lpart[blockIdx.x] = ls;
    }
    // each thread owns some parameters and sums the block's rows for them in row order
    float* G = Gpart + (int64_t)blockIdx.x * L.n;
    for (int p = tid; p < L.n; p += blockDim.x) {
        float acc = 0.f;
        if (p < L.b1) {  // W1[j][f] = sum d1[j] x[f]
            const int j = p / F, f = p % F;
            for (int q = 0; q < kRowsPerBlock; q++) acc = fmaf(sd1[q * kH + j], sx[q * kMaxF + f], acc);
        } else if (p < L.W2) {
            const int j = p - L.b1;
            for (int q = 0; q < kRowsPerBlock; q++) acc += sd1[q * kH + j];
        } else if (p < L.b2) {  // W2[j][k] = sum d2[j] h1[k]
            const int j = (p - L.W2) / kH, k = (p - L.W2) % kH;
            for (int q = 0; q < kRowsPerBlock; q++) acc = fmaf(sd2[q * kH + j], sh1[q * kH + k], acc);
        } else if (p < L.w3) {
            const int j = p - L.b2;
            for (int q = 0; q < kRowsPerBlock; q++) acc += sd2[q * kH + j];
        } else if (p < L.b3) {  // w3[j] = sum dy h2[j]
            const int j = p - L.w3;
            for (int q = 0; q < kRowsPerBlock; q++) acc = fmaf(sdy[q], sh2[q * kH + j], acc);
        } else if (p == L.b3) {
            for (int q = 0; q < kRowsPerBlock; q++) acc += sdy[q];
        } else {  // linear skip c[f] = sum dy x[f]
            const int f = p - L.c;
            for (int q = 0; q < kRowsPerBlock; q++) acc = fmaf(sdy[q], sx[q * kMaxF + f], acc);
        }
        G[p] = acc;
    }
}

// G[p] = sum over blocks of Gpart[b][p] (block order); loss likewise
__global__ void mlp_grad_reduce_kernel(int nblocks, int n, const float* __restrict__ Gpart, float* __restrict__ G,
                                       const double* __restrict__ Lpart, int64_t nl, double* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        float acc = 0.f;
        for (int b = 0; b < nblocks; b++) acc += Gpart[(int64_t)b * n + p];
        G[p] = acc;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double s = 0;
        for (int64_t q = 0; q < nl; q++) s += Lpart[q];
        *loss = s;
    }
}

__global__ void adam_kernel(int n, float* __restrict__ P, const float* __restrict__ G, float* __restrict__ Mm,
                            float* __restrict__ Vv, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float g = G[p];
    const float m = b1 * Mm[p] + (1.f - b1) * g;
    const float v = b2 * Vv[p] + (1.f - b2) * g * g;
    Mm[p] = m;
    Vv[p] = v;
    P[p] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

// features at dof i: x = [d_0, d_1, ..., q] / s_i with d_j = h_j - h_{j+1} (h_0 = u^n) and the per-dof
// scale s_i = |(d_0, d_1, ...)|_2 at that dof (floored at 1e-300); s_i is written to `scale`
__global__ void features_kernel(int64_t n, int k, const double* __restrict__ h0, const double* __restrict__ h1,
                                const double* __restrict__ h2, const double* __restrict__ h3,
                                const double* __restrict__ q, double* __restrict__ scale, float* __restrict__ X,
                                int F) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* h[4] = {h0, h1, h2, h3};
    double d[4];
    double s2 = 0;
    for (int j = 0; j + 1 < k; j++) {
        d[j] = h[j][i] - h[j + 1][i];
        s2 += d[j] * d[j];
    }
    const double s = fmax(sqrt(s2), 1e-300);
    scale[i] = s;
    const double inv = 1.0 / s;
    int f = 0;
    for (int j = 0; j + 1 < k && f < F; j++, f++) X[i * F + f] = (float)(d[j] * inv);
    if (q && f < F) X[i * F + f++] = (float)fmax(-1e3, fmin(1e3, q[i] * inv));
    for (; f < F; f++) X[i * F + f] = 0.f;
}

// training target t_i = (u^{n+1}_i - u^n_i) / s_i, clamped to [-10, 10]
__global__ void target_kernel(int64_t n, const double* __restrict__ unext, const double* __restrict__ un,
                              const double* __restrict__ scale, float* __restrict__ T) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    T[i] = (float)fmax(-10.0, fmin(10.0, (unext[i] - un[i]) / scale[i]));
}

// x = u^n + scale * y on free dofs (constrained dofs keep u^n)
__global__ void apply_kernel(int64_t n, const double* __restrict__ un, const float* __restrict__ y,
                             const double* __restrict__ scale, const uint8_t* __restrict__ freed, double* __restrict__ x) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = un[i] + ((freed == nullptr || freed[i]) ? scale[i] * (double)y[i] : 0.0);
}

// scale = sqrt(mean((a - b)^2)) (floored at 1e-300), two fixed-order stages in one launch: the last
// block to finish sums the per-block partials in block order.
__global__ void rms_diff_kernel(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                                double* __restrict__ part, unsigned* __restrict__ cnt, double* __restrict__ scale) {
    double acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double d = a[i] - b[i];
        acc += d * d;
    }
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        part[blockIdx.x] = t;
    }
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double t = 0;
    for (unsigned q = 0; q < gridDim.x; q++) t += __ldcg(part + q);
    *cnt = 0;
    const double r = sqrt(t / (double)(n > 0 ? n : 1));
    scale[0] = r > 1e-300 ? r : 1e-300;
}

// q = D^-1 (b - A x) on free rows (0 elsewhere), FP64, TPR lanes per row (the SpMV row kernel)
template <int TPR, int U>
__global__ void __launch_bounds__(256) jacobi_resid_kernel(int64_t n, const int32_t* __restrict__ rp,
                                                           const int32_t* __restrict__ col,
                                                           const double* __restrict__ A,
                                                           const double* __restrict__ dinv,
                                                           const int32_t* __restrict__ diagpos,
                                                           const uint8_t* __restrict__ freed,
                                                           const double* __restrict__ b, const double* __restrict__ x,
                                                           double* __restrict__ q) {
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / TPR;
    const int lane = threadIdx.x % TPR;
    int32_t a = 0, e = 0;
    if (r < n) {
        a = __ldg(rp + r);
        e = __ldg(rp + r + 1);
    }
    const double ax = row_dot<double, double, TPR, U>(a, e, col, A, x, lane);
    if (r < n && lane == 0) {
        if (!freed[r]) {
            q[r] = 0.0;
        } else {
            const double di = dinv ? dinv[r] : 1.0 / A[diagpos[r]];
            q[r] = di * (b[r] - ax);
        }
    }
}

}  // namespace
}  // namespace ocmp

using namespace ocmp;

struct ocmp_guess_s {
    int F = 0;
    Layout L;
    float* P = nullptr;
    float* G = nullptr;
    float* M = nullptr;
    float* V = nullptr;
    float* Gpart = nullptr;
    double* Lpart = nullptr;
    double* loss = nullptr;
    int64_t part_rows = 0;  // capacity (rows) of the partial buffers
    int step = 0;
    double* spart = nullptr;  // scale reduction partials
    unsigned* scnt = nullptr;
};

static void guess_free(ocmp_guess_s* g) {
    void* ps[] = {g->P, g->G, g->M, g->V, g->Gpart, g->Lpart, g->loss, g->spart, g->scnt};
    for (void* p : ps) dfree(p);
}

static int ensure_parts(ocmp_guess_s* g, int64_t rows) {
    if (rows <= g->part_rows) return OCMP_OK;
    dfree(g->Gpart);
    dfree(g->Lpart);
    g->Gpart = nullptr;
    g->Lpart = nullptr;
    const int64_t nb = (rows + kRowsPerBlock - 1) / kRowsPerBlock;
    int st = dalloc(&g->Gpart, (size_t)(nb * g->L.n));
    if (!st) st = dalloc(&g->Lpart, (size_t)nb);
    if (st) return st;
    g->part_rows = nb * kRowsPerBlock;
    return OCMP_OK;
}

extern "C" {

int ocmp_guess_create(int32_t n_features, uint64_t seed, ocmp_guess_t* out) {
    if (!out || n_features < 1 || n_features > kMaxF) return fail(OCMP_ERR_ARG, "ocmp_guess_create: 1..8 features");
    auto* g = new ocmp_guess_s();
    g->F = n_features;
    g->L = layout(n_features);
    const int n = g->L.n;
    int st = dalloc(&g->P, n);
    if (!st) st = dalloc(&g->G, n);
    if (!st) st = dalloc(&g->M, n);
    if (!st) st = dalloc(&g->V, n);
    if (!st) st = dalloc(&g->loss, 1);
    if (st) {
        guess_free(g);
        delete g;
        return st;
    }
    // Xavier-uniform weights from a 64-bit LCG seeded by `seed`; zero biases; small output layer
    std::vector<float> h(n, 0.f);
    uint64_t s = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto rnd = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return (double)(s >> 11) * (1.0 / 9007199254740992.0);
    };
    const Layout& L = g->L;
    const double a1 = std::sqrt(6.0 / (n_features + kH)), a2 = std::sqrt(6.0 / (2 * kH)), a3 = 0.1;
    for (int k = 0; k < kH * n_features; k++) h[L.W1 + k] = (float)((2 * rnd() - 1) * a1);
    for (int k = 0; k < kH * kH; k++) h[L.W2 + k] = (float)((2 * rnd() - 1) * a2);
    for (int k = 0; k < kH; k++) h[L.w3 + k] = (float)((2 * rnd() - 1) * a3);
    if (n_features >= 1) h[L.c] = 1.f;  // start from the previous-difference guess u^n + (u^n - u^{n-1})
    std::vector<float> z(n, 0.f);
    if (cudaMemcpy(g->P, h.data(), sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(g->M, z.data(), sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(g->V, z.data(), sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
        guess_free(g);
        delete g;
        return fail(OCMP_ERR_CUDA, "ocmp_guess_create: upload failed");
    }
    *out = g;
    return OCMP_OK;
}

int ocmp_guess_destroy(ocmp_guess_t g) {
    if (!g) return OCMP_OK;
    guess_free(g);
    delete g;
    return OCMP_OK;
}

int ocmp_guess_nparams(ocmp_guess_t g) { return g ? g->L.n : -1; }

int ocmp_guess_params(ocmp_guess_t g, float* host, int32_t set) {
    if (!g || !host) return fail(OCMP_ERR_ARG, "ocmp_guess_params: null argument");
    if (set) {
        OCMP_CUDA(cudaMemcpy(g->P, host, sizeof(float) * g->L.n, cudaMemcpyHostToDevice));
        g->step = 0;
        OCMP_CUDA(cudaMemset(g->M, 0, sizeof(float) * g->L.n));
        OCMP_CUDA(cudaMemset(g->V, 0, sizeof(float) * g->L.n));
    } else {
        OCMP_CUDA(cudaMemcpy(host, g->P, sizeof(float) * g->L.n, cudaMemcpyDeviceToHost));
    }
    return OCMP_OK;
}

int ocmp_guess_forward(ocmp_guess_t g, const float* X, int64_t rows, float* Y, void* stream) {
    if (!g || !X || !Y || rows < 0) return fail(OCMP_ERR_ARG, "ocmp_guess_forward: bad argument");
    if (rows == 0) return OCMP_OK;
    OCMP_LAUNCH(mlp_forward_kernel<<<(unsigned)((rows + kRowsPerBlock - 1) / kRowsPerBlock), kRowsPerBlock,
                         sizeof(float) * g->L.n, (cudaStream_t)stream>>>(rows, g->F, g->P, X, Y));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int ocmp_guess_loss_grad(ocmp_guess_t g, const float* X, const float* T, int64_t rows, double* loss_host,
                         float* grad_host, void* stream) {
    if (!g || !X || !T || rows <= 0) return fail(OCMP_ERR_ARG, "ocmp_guess_loss_grad: bad argument");
    int st = ensure_parts(g, rows);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = (int)((rows + kRowsPerBlock - 1) / kRowsPerBlock);
    const size_t smem = sizeof(double) * kRowsPerBlock + sizeof(float) * (g->L.n + kRowsPerBlock * (4 * kH + kMaxF + 1));
    OCMP_CUDA(cudaFuncSetAttribute(mlp_grad_partial_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    OCMP_LAUNCH(mlp_grad_partial_kernel<<<nb, kRowsPerBlock, smem, s>>>(rows, g->F, g->P, X, T, g->Gpart, g->Lpart));
    OCMP_LAUNCH(mlp_grad_reduce_kernel<<<(g->L.n + 255) / 256, 256, 0, s>>>(nb, g->L.n, g->Gpart, g->G, g->Lpart, (int64_t)nb,
                                                                g->loss));
    OCMP_CUDA(cudaGetLastError());
    if (loss_host) {
        OCMP_CUDA(cudaMemcpyAsync(loss_host, g->loss, sizeof(double), cudaMemcpyDeviceToHost, s));
        OCMP_CUDA(cudaStreamSynchronize(s));
    }
    if (grad_host) {
        OCMP_CUDA(cudaMemcpyAsync(grad_host, g->G, sizeof(float) * g->L.n, cudaMemcpyDeviceToHost, s));
        OCMP_CUDA(cudaStreamSynchronize(s));
    }
    return OCMP_OK;
}

int ocmp_guess_adam_step(ocmp_guess_t g, float lr, void* stream) {
    if (!g) return fail(OCMP_ERR_ARG, "ocmp_guess_adam_step: null argument");
    g->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)g->step), c2 = 1.f - std::pow(b2, (float)g->step);
    OCMP_LAUNCH(adam_kernel<<<(g->L.n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(g->L.n, g->P, g->G, g->M, g->V, lr, b1, b2,
                                                                        1e-8f, c1, c2));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int ocmp_guess_features(int64_t n, int32_t k, const double* const* hist, const double* q, double* scale,
                        float* X, int32_t F, void* stream) {
    if (!hist || !X || !scale || n < 0 || k < 2 || k > 4 || F < 1 || F > kMaxF)
        return fail(OCMP_ERR_ARG, "ocmp_guess_features: bad argument");
    for (int d = 0; d < k; d++)
        if (!hist[d]) return fail(OCMP_ERR_ARG, "ocmp_guess_features: null history vector");
    if (n == 0) return OCMP_OK;
    OCMP_LAUNCH(features_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        n, k, hist[0], k > 1 ? hist[1] : hist[0], k > 2 ? hist[2] : hist[0], k > 3 ? hist[3] : hist[0], q, scale, X,
        F));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int ocmp_guess_apply(int64_t n, const double* un, const float* y, const double* scale, const uint8_t* freed,
                     double* x, void* stream) {
    if (!un || !y || !x || !scale || n < 0) return fail(OCMP_ERR_ARG, "ocmp_guess_apply: bad argument");
    if (n == 0) return OCMP_OK;
    OCMP_LAUNCH(apply_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, un, y, scale, freed, x));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int ocmp_guess_target(int64_t n, const double* unext, const double* un, const double* scale, float* T,
                      void* stream) {
    if (!unext || !un || !scale || !T || n < 0) return fail(OCMP_ERR_ARG, "ocmp_guess_target: bad argument");
    if (n == 0) return OCMP_OK;
    OCMP_LAUNCH(target_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, unext, un, scale, T));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int ocmp_guess_scale(ocmp_guess_t g, int64_t n, const double* a, const double* b, double* scale, void* stream) {
    if (!g || !a || !b || !scale || n < 0) return fail(OCMP_ERR_ARG, "ocmp_guess_scale: bad argument");
    const int nb = 304;
    if (!g->spart) {
        int st = dalloc(&g->spart, nb);
        if (!st) st = dalloc(&g->scnt, 1);
        if (st) return st;
        OCMP_CUDA(cudaMemset(g->scnt, 0, sizeof(unsigned)));
    }
    OCMP_LAUNCH(rms_diff_kernel<<<nb, 256, 0, (cudaStream_t)stream>>>(n, a, b, g->spart, g->scnt, scale));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int ocmp_jacobi_residual(ocmp_matrix_t mat, const double* b, const double* x, double* q, void* stream) {
    if (!mat || !b || !x || !q) return fail(OCMP_ERR_ARG, "ocmp_jacobi_residual: null argument");
    const ocmp_space_s* s = mat->space;
    const RowCfg rc = row_cfg(s);
    const int64_t n = s->ndof;
    const unsigned g = (unsigned)((n * rc.tpr + 255) / 256);
    cudaStream_t st = (cudaStream_t)stream;
#define JR(TPR, U)                                                                                                    \
    OCMP_LAUNCH(jacobi_resid_kernel<TPR, U><<<g, 256, 0, st>>>(n, s->d_rowptr, s->d_col, mat->vals, mat->dinv, s->d_diag, s->d_free, \
                                                   b, x, q))
    if (rc.tpr == 2) JR(2, 4);
    else if (rc.tpr == 4 && rc.u == 4) JR(4, 4);
    else if (rc.tpr == 4) JR(4, 8);
    else if (rc.tpr == 8 && rc.u == 4) JR(8, 4);
    else if (rc.tpr == 8) JR(8, 8);
    else JR(16, 8);
#undef JR
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

}  // extern "C"
