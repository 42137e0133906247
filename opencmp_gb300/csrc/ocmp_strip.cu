// Strip direct preconditioner of libopencmp_gpu.so (sm_103a): the GPU counterpart of the sparse
// direct solve in opencmp/models/base_model.py:906-922 (a.mat.Inverse(freedofs, 'pardiso' |
// 'umfpack'), then gfu += inv * (L - A gfu)), used as the preconditioner of FP64-refined GMRES.
//
// The dofs are cut into consecutive strips [s_k, s_k+1) chosen so that the matrix is block
// tridiagonal over them: strip k's rows reach no further than strip k+1 (greedy over the row
// bandwidth; a structured mesh whose elements are numbered row by row gives one strip per row of
// elements). Block elimination over the strips (the block Thomas algorithm) needs, per strip,
//     S_k = A_kk - A_k,k-1 S_{k-1}^-1 A_k-1,k,      G_k = S_k^-1,
// and a solve is a forward sweep y_k = G_k (b_k - A_k,k-1 y_k-1) and a backward sweep
// x_k = y_k - G_k A_k,k+1 x_k+1. Every G_k is kept explicitly (FP32, dense, padded to a multiple of
// 128), so each sweep step is one dense matrix-vector product instead of two triangular solves.
//
// Factorisation of strip k, all in FP32 on the device:
//  1. S_k is scattered from the CSR rows of the strip (constrained rows and columns dropped, unit
//     diagonal there and on the padding).
//  2. Schur update through the interface only: I = rows of strip k coupled to strip k-1, J = rows of
//     strip k-1 coupled to strip k; S_k[I,I] -= A[I,J] G_k-1[J,J] A[J,I] as two dense products.
//  3. Block Gauss-Jordan inversion in place with 128 x 128 diagonal-tile pivots (each tile inverted
//     with partial pivoting inside it): per tile one small inversion, two panel kernels and one
//     rank-128 update S -= C R^T of the whole strip, the dominant flops.
// The dense products are C = beta C + alpha A B^T with both operands K-contiguous (gemm_nt).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "ocmp_internal.h"

namespace ocmp {

constexpr int kNb = 128;   // Gauss-Jordan tile and padding granule

struct Strip {
    int K = 0;
    std::vector<int64_t> s;          // K + 1 strip boundaries
    std::vector<int> m, mp;          // strip sizes and padded sizes
    std::vector<int64_t> goff;       // offsets of G_k in d_G (floats)
    std::vector<int> nI, nJ;         // interface sizes: I_k (k >= 1) and J_k (k <= K-2)
    std::vector<int64_t> ioff, joff; // offsets into d_I / d_J
    int mp_max = 0, nIp_max = 0, nJp_max = 0;
    int32_t* d_I = nullptr;          // local indices of I_k, strip after strip
    int32_t* d_J = nullptr;          // local indices of J_k
    int32_t* d_Iinv = nullptr;       // per dof: its position in I of its strip, or -1
    int32_t* d_Jinv = nullptr;       // per dof: its position in J of its strip, or -1
    int32_t* d_lo_ptr = nullptr;     // per dof: CSR positions whose column lies in the previous strip
    int32_t* d_lo_pos = nullptr;
    int32_t* d_hi_ptr = nullptr;     // per dof: CSR positions whose column lies in the next strip
    int32_t* d_hi_pos = nullptr;
    float* d_G = nullptr;            // the explicit strip inverses
    float* d_Bt = nullptr;           // interface scratch
    float* d_Cc = nullptr;
    float* d_Gjj = nullptr;
    float* d_Tt = nullptr;
    float* d_U = nullptr;
    float* d_P = nullptr;            // Gauss-Jordan panels
    float* d_Ck = nullptr;
    float* d_Rt = nullptr;
    float* d_r = nullptr;            // solve scratch (one strip)
    int* d_flag = nullptr;           // [0] pivot tiles that were singular or non-finite, [1] a tensor-core
                                     // product whose bounded wait gave up
    int64_t bytes = 0;
    // statistics of the last factorisation
    bool timing = false;
    std::vector<cudaEvent_t> ev;
    size_t ev_used = 0;
    cudaEvent_t fev[2] = {nullptr, nullptr};
    double factor_ms = 0, gemm_ms = 0, gemm_flops = 0, gemm_flops_pending = 0;
    int singular = 0;
    int gemm_kind = 0;               // 0: FP32 SIMT, 1: tensor cores (3xTF32)
};

namespace {

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }
inline int pad(int64_t v) { return (int)((v + kNb - 1) / kNb * kNb); }

// ------------------------------------------------------------------ dense products (FP32 SIMT)
// C[M x N] = beta C + alpha A[M x K] B[N x K]^T, row-major with leading dimensions lda/ldb/ldc;
// M, N multiples of 128, K a multiple of 16, rows 16-byte aligned. 256 threads, 128 x 128 tile,
// 8 x 8 outputs per thread, double-buffered K slices of 16.
constexpr int GB = 128, GK = 16;
__global__ void __launch_bounds__(256) sgemm_nt(int M, int N, int K, const float* __restrict__ A, int64_t lda,
                                                const float* __restrict__ B, int64_t ldb, float* __restrict__ C,
                                                int64_t ldc, float alpha, float beta) {
    __shared__ __align__(16) float As[2][GK][GB + 4];
    __shared__ __align__(16) float Bs[2][GK][GB + 4];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t m0 = (int64_t)blockIdx.y * GB, n0 = (int64_t)blockIdx.x * GB;
    if (m0 >= M || n0 >= N) return;
    const int lr = tid >> 2, lk = (tid & 3) * 4;   // load: rows lr, lr + 64; k lk..lk+3
    float4 ra[2], rb[2];
    auto gload = [&](int k0) {
#pragma unroll
        for (int q = 0; q < 2; q++) {
            ra[q] = *reinterpret_cast<const float4*>(A + (m0 + lr + 64 * q) * lda + k0 + lk);
            rb[q] = *reinterpret_cast<const float4*>(B + (n0 + lr + 64 * q) * ldb + k0 + lk);
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int r = lr + 64 * q;
            As[buf][lk + 0][r] = ra[q].x;
            As[buf][lk + 1][r] = ra[q].y;
            As[buf][lk + 2][r] = ra[q].z;
            As[buf][lk + 3][r] = ra[q].w;
            Bs[buf][lk + 0][r] = rb[q].x;
            Bs[buf][lk + 1][r] = rb[q].y;
            Bs[buf][lk + 2][r] = rb[q].z;
            Bs[buf][lk + 3][r] = rb[q].w;
        }
    };
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
    gload(0);
    sstore(0);
    __syncthreads();
    int buf = 0;
    for (int k0 = 0; k0 < K; k0 += GK) {
        const bool more = k0 + GK < K;
        if (more) gload(k0 + GK);
#pragma unroll
        for (int kk = 0; kk < GK; kk++) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4 + 64]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4 + 64]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (more) sstore(buf ^ 1);
        __syncthreads();
        buf ^= 1;
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int64_t r = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float4* p = reinterpret_cast<float4*>(C + r * ldc + n0 + h * 64 + tx * 4);
            float4 o = beta != 0.f ? *p : make_float4(0.f, 0.f, 0.f, 0.f);
            o.x = alpha * acc[i][h * 4 + 0] + beta * o.x;
            o.y = alpha * acc[i][h * 4 + 1] + beta * o.y;
            o.z = alpha * acc[i][h * 4 + 2] + beta * o.z;
            o.w = alpha * acc[i][h * 4 + 3] + beta * o.w;
            *p = o;
        }
    }
}

// ------------------------------------------------------------------ strip assembly
// S (mp x mp, zeroed) <- the strip's diagonal block; unit diagonal on constrained rows and padding
__global__ void k_fill_strip(int m, int mp, int64_t s0, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                             const double* __restrict__ vals, const uint8_t* __restrict__ freed, float* __restrict__ S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mp) return;
    float* row = S + (int64_t)i * mp;
    if (i >= m || !freed[s0 + i]) {
        row[i] = 1.f;
        return;
    }
    const int64_t r = s0 + i;
    for (int32_t k = rp[r]; k < rp[r + 1]; k++) {
        const int64_t c = col[k];
        if (c >= s0 && c < s0 + m && freed[c]) row[c - s0] = (float)vals[k];
    }
}

// Interface blocks of the boundary between strip k-1 (start sp) and strip k (start s0):
// Cc[a, b] = A[I_a, J_b] (rows of strip k, columns of strip k-1) and Bt[a, b] = A[J_b, I_a].
__global__ void k_fill_iface(int nI, int nJ, int nJp, int64_t s0, int64_t sp, const int32_t* __restrict__ I,
                             const int32_t* __restrict__ J, const int32_t* __restrict__ Iinv,
                             const int32_t* __restrict__ Jinv, const int32_t* __restrict__ lo_ptr,
                             const int32_t* __restrict__ lo_pos, const int32_t* __restrict__ hi_ptr,
                             const int32_t* __restrict__ hi_pos, const int32_t* __restrict__ col,
                             const double* __restrict__ vals, const uint8_t* __restrict__ freed, float* __restrict__ Cc,
                             float* __restrict__ Bt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nI) {
        const int64_t r = s0 + I[t];
        if (!freed[r]) return;
        for (int32_t q = lo_ptr[r]; q < lo_ptr[r + 1]; q++) {
            const int32_t k = lo_pos[q];
            const int64_t c = col[k];
            const int b = Jinv[c];
            if (freed[c] && b >= 0) Cc[(int64_t)t * nJp + b] = (float)vals[k];
        }
    } else if (t < nI + nJ) {
        const int bj = t - nI;
        const int64_t r = sp + J[bj];
        if (!freed[r]) return;
        for (int32_t q = hi_ptr[r]; q < hi_ptr[r + 1]; q++) {
            const int32_t k = hi_pos[q];
            const int64_t c = col[k];
            const int a = Iinv[c];
            if (freed[c] && a >= 0) Bt[(int64_t)a * nJp + bj] = (float)vals[k];
        }
    }
}

// Gjj[a, b] = G[J_a, J_b] (zero padding)
__global__ void k_gather_gjj(int nJ, int nJp, const int32_t* __restrict__ J, const float* __restrict__ G, int mpG,
                             float* __restrict__ Gjj) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nJp * nJp) return;
    const int a = (int)(t / nJp), b = (int)(t % nJp);
    Gjj[t] = (a < nJ && b < nJ) ? G[(int64_t)J[a] * mpG + J[b]] : 0.f;
}

// S[I_a, I_c] -= U[a, c]
__global__ void k_scatter_sub(int nI, int nIp, const int32_t* __restrict__ I, const float* __restrict__ U, int mp,
                              float* __restrict__ S) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nI * nI) return;
    const int a = (int)(t / nI), c = (int)(t % nI);
    S[(int64_t)I[a] * mp + I[c]] -= U[(int64_t)a * nIp + c];
}

// ------------------------------------------------------------------ block Gauss-Jordan
// P <- inverse of the tile S[t0:t0+128, t0:t0+128] by Gauss-Jordan with partial pivoting inside
// the tile. A zero or non-finite pivot is counted in *flag and replaced by a tiny value.
constexpr int kTileThreads = 1024;
__global__ void __launch_bounds__(kTileThreads) k_tile_inv(const float* __restrict__ S, int mp, int t0,
                                                           float* __restrict__ P, int* __restrict__ flag) {
    extern __shared__ float sm[];
    constexpr int LD = kNb + 1;
    float* a = sm;                      // kNb x LD
    float* f = sm + kNb * LD;           // column k before the update
    __shared__ int piv[kNb];
    __shared__ int sp;
    __shared__ float sd;
    const int tid = threadIdx.x;
    for (int e = tid; e < kNb * kNb; e += kTileThreads) {
        const int r = e / kNb, c = e % kNb;
        a[r * LD + c] = S[(int64_t)(t0 + r) * mp + t0 + c];
    }
    __syncthreads();
    for (int k = 0; k < kNb; k++) {
        if (tid < 32) {
            float best = -1.f;
            int bi = k;
            for (int i = k + tid; i < kNb; i += 32) {
                const float v = fabsf(a[i * LD + k]);
                if (v > best) {
                    best = v;
                    bi = i;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ob = __shfl_down_sync(0xffffffffu, best, o);
                const int oi = __shfl_down_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (tid == 0) {
                sp = bi;
                piv[k] = bi;
            }
        }
        __syncthreads();
        const int p = sp;
        if (p != k && tid < kNb) {
            const float t = a[k * LD + tid];
            a[k * LD + tid] = a[p * LD + tid];
            a[p * LD + tid] = t;
        }
        __syncthreads();
        if (tid == 0) {
            float d = a[k * LD + k];
            if (!(fabsf(d) > 0.f) || !isfinite(d)) {
                atomicAdd(flag, 1);
                d = 1e-30f;
            }
            sd = 1.f / d;
        }
        __syncthreads();
        if (tid < kNb) {
            f[tid] = a[tid * LD + k];
            const float v = tid == k ? 1.f : a[k * LD + tid];
            a[k * LD + tid] = v * sd;
        }
        __syncthreads();
        for (int e = tid; e < kNb * kNb; e += kTileThreads) {
            const int r = e / kNb, c = e % kNb;
            if (r == k) continue;
            const float prev = c == k ? 0.f : a[r * LD + c];
            a[r * LD + c] = prev - f[r] * a[k * LD + c];
        }
        __syncthreads();
    }
    // undo the row interchanges: swap columns in reverse order
    for (int k = kNb - 1; k >= 0; k--) {
        const int p = piv[k];
        if (p != k && tid < kNb) {
            const float t = a[tid * LD + k];
            a[tid * LD + k] = a[tid * LD + p];
            a[tid * LD + p] = t;
        }
        __syncthreads();
    }
    for (int e = tid; e < kNb * kNb; e += kTileThreads) P[e] = a[(e / kNb) * LD + e % kNb];
}

// For the 32 columns c0..c0+31: Rt[c, r] = sum_l P[r, l] S[t0 + l, c] (the pivot rows times P, stored
// transposed), and for the 32 rows c0..c0+31: Ck[i, l] = S[i, t0 + l], zero on the pivot rows.
__global__ void __launch_bounds__(256) k_panel_prep(const float* __restrict__ S, int mp, int t0,
                                                    const float* __restrict__ P, float* __restrict__ Rt,
                                                    float* __restrict__ Ck) {
    extern __shared__ float sm[];
    float* Ps = sm;                  // kNb x kNb
    float* Sc = sm + kNb * kNb;      // kNb x 33: S[t0 + l, c0 + j]
    const int tid = threadIdx.x, c0 = blockIdx.x * 32;
    for (int e = tid; e < kNb * kNb; e += 256) Ps[e] = P[e];
    for (int e = tid; e < kNb * 32; e += 256) {
        const int l = e / 32, j = e % 32;
        Sc[l * 33 + j] = S[(int64_t)(t0 + l) * mp + c0 + j];
    }
    // Ck rows
    for (int e = tid; e < 32 * kNb; e += 256) {
        const int i = c0 + e / kNb, l = e % kNb;
        Ck[(int64_t)i * kNb + l] = (i >= t0 && i < t0 + kNb) ? 0.f : S[(int64_t)i * mp + t0 + l];
    }
    __syncthreads();
    const int j = tid & 31, rw = tid >> 5;   // column c0 + j, rows rw, rw + 8, ...
    float acc[16];
#pragma unroll
    for (int q = 0; q < 16; q++) acc[q] = 0.f;
    for (int l = 0; l < kNb; l++) {
        const float s = Sc[l * 33 + j];
#pragma unroll
        for (int q = 0; q < 16; q++) acc[q] = fmaf(Ps[(rw + 8 * q) * kNb + l], s, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 16; q++) Rt[(int64_t)(c0 + j) * kNb + rw + 8 * q] = acc[q];
}

// After the rank-128 update: S[i, t0 + l] = -(Ck P)[i, l] for the non-pivot rows i of this block's 32
// rows; S[t0 + r, c] = Rt[c, r] for this block's 32 columns c outside the tile, P inside it.
__global__ void __launch_bounds__(256) k_panel_finish(float* __restrict__ S, int mp, int t0,
                                                      const float* __restrict__ P, const float* __restrict__ Rt,
                                                      const float* __restrict__ Ck) {
    extern __shared__ float sm[];
    float* Ps = sm;                  // kNb x kNb
    float* Cs = sm + kNb * kNb;      // 32 x (kNb + 1)
    const int tid = threadIdx.x, c0 = blockIdx.x * 32;
    for (int e = tid; e < kNb * kNb; e += 256) Ps[e] = P[e];
    for (int e = tid; e < 32 * kNb; e += 256) Cs[(e / kNb) * (kNb + 1) + e % kNb] = Ck[(int64_t)(c0 + e / kNb) * kNb + e % kNb];
    __syncthreads();
    // column block: row i = c0 + ii, column l; thread: l = tid & 127, rows ii = (tid >> 7) + 2 q
    {
        const int l = tid & (kNb - 1), r0 = tid >> 7;
        for (int ii = r0; ii < 32; ii += 2) {
            const int i = c0 + ii;
            if (i >= t0 && i < t0 + kNb) continue;
            float acc = 0.f;
            for (int q = 0; q < kNb; q++) acc = fmaf(Cs[ii * (kNb + 1) + q], Ps[q * kNb + l], acc);
            S[(int64_t)i * mp + t0 + l] = -acc;
        }
    }
    // row block
    for (int e = tid; e < 32 * kNb; e += 256) {
        const int jj = e / kNb, r = e % kNb;
        const int c = c0 + jj;
        const float v = (c >= t0 && c < t0 + kNb) ? Ps[r * kNb + (c - t0)] : Rt[(int64_t)c * kNb + r];
        S[(int64_t)(t0 + r) * mp + c] = v;
    }
}

// ------------------------------------------------------------------ sweeps
// forward right-hand side of strip [s0, s0 + m): r_i = sc v_i - sum A[i, c] z_c over the entries
// whose column lies in the previous strip (z holds that strip's y); zero on constrained rows and
// on the padding up to mp
template <class T>
__global__ void k_fwd_rhs(int m, int mp, int64_t s0, const int32_t* __restrict__ lo_ptr,
                          const int32_t* __restrict__ lo_pos, const int32_t* __restrict__ col,
                          const double* __restrict__ vals, const uint8_t* __restrict__ freed, const T* __restrict__ v,
                          const double* __restrict__ scale, int j, const T* __restrict__ z, float* __restrict__ r,
                          const int* __restrict__ flags) {
    if (flags && flags[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mp) return;
    if (i >= m) {
        r[i] = 0.f;
        return;
    }
    const int64_t row = s0 + i;
    if (!freed[row]) {
        r[i] = 0.f;
        return;
    }
    const double sc = scale ? scale[j] : 1.0;
    float acc = (float)(sc * (double)v[row]);
    for (int32_t q = lo_ptr[row]; q < lo_ptr[row + 1]; q++) {
        const int32_t k = lo_pos[q];
        const int32_t c = col[k];
        if (freed[c]) acc -= (float)vals[k] * (float)z[c];
    }
    r[i] = acc;
}

// backward right-hand side: r_i = sum A[i, c] z_c over the entries in the next strip
template <class T>
__global__ void k_bwd_rhs(int m, int mp, int64_t s0, const int32_t* __restrict__ hi_ptr,
                          const int32_t* __restrict__ hi_pos, const int32_t* __restrict__ col,
                          const double* __restrict__ vals, const uint8_t* __restrict__ freed, const T* __restrict__ z,
                          float* __restrict__ r, const int* __restrict__ flags) {
    if (flags && flags[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mp) return;
    if (i >= m || !freed[s0 + i]) {
        r[i] = 0.f;
        return;
    }
    const int64_t row = s0 + i;
    float acc = 0.f;
    for (int32_t q = hi_ptr[row]; q < hi_ptr[row + 1]; q++) {
        const int32_t k = hi_pos[q];
        const int32_t c = col[k];
        if (freed[c]) acc += (float)vals[k] * (float)z[c];
    }
    r[i] = acc;
}

// z_i = (G r)_i (mode 0) or z_i -= (G r)_i (mode 1) for the strip's m rows; a warp per row, 16-byte
// loads (mp is a multiple of 128)
template <class T>
__global__ void __launch_bounds__(256) k_strip_gemv(int m, int mp, const float* __restrict__ G,
                                                    const float* __restrict__ r, T* __restrict__ z, int mode,
                                                    const int* __restrict__ flags) {
    if (flags && flags[0]) return;
    const int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= m) return;
    const float4* g = reinterpret_cast<const float4*>(G + (int64_t)row * mp);
    const float4* rv = reinterpret_cast<const float4*>(r);
    float acc = 0.f;
    for (int q = lane; q < mp / 4; q += 32) {
        const float4 a = __ldg(g + q);
        const float4 b = __ldg(rv + q);
        acc = fmaf(a.x, b.x, acc);
        acc = fmaf(a.y, b.y, acc);
        acc = fmaf(a.z, b.z, acc);
        acc = fmaf(a.w, b.w, acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
        if (mode == 0) z[row] = (T)acc;
        else z[row] = (T)((float)z[row] - acc);
    }
}

template <class T>
__global__ void k_add_to(int64_t n, const T* __restrict__ z, double* __restrict__ x, const int* __restrict__ flags) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) x[i] += (double)z[i];
}

// ------------------------------------------------------------------ host helpers
void strip_free(Strip* p) {
    void* ps[] = {p->d_I, p->d_J, p->d_Iinv, p->d_Jinv, p->d_lo_ptr, p->d_lo_pos, p->d_hi_ptr, p->d_hi_pos, p->d_G,
                  p->d_Bt, p->d_Cc, p->d_Gjj, p->d_Tt, p->d_U, p->d_P, p->d_Ck, p->d_Rt, p->d_r, p->d_flag};
    for (void* q : ps) dfree(q);
    for (cudaEvent_t e : p->ev) cudaEventDestroy(e);
    for (cudaEvent_t e : p->fev)
        if (e) cudaEventDestroy(e);
}

int gemm(Strip* p, int M, int N, int K, const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
         float alpha, float beta, cudaStream_t st) {
    if (M % GB || N % GB || K % GK || M <= 0 || N <= 0 || K <= 0)
        return fail(OCMP_ERR_ARG, "strip gemm: sizes must be multiples of the tile");
    const bool t = p->timing;
    if (t) {
        while (p->ev.size() < p->ev_used + 2) {
            cudaEvent_t e;
            OCMP_CUDA(cudaEventCreate(&e));
            p->ev.push_back(e);
        }
        OCMP_CUDA(cudaEventRecord(p->ev[p->ev_used], st));
    }
    if (p->gemm_kind == 1) {
        const int r = tc_gemm_nt(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, p->d_flag + 1, st);
        if (r) return r;
    } else {
        const dim3 g(N / GB, M / GB);
        OCMP_LAUNCH(sgemm_nt<<<g, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta));
    }
    if (t) {
        OCMP_CUDA(cudaEventRecord(p->ev[p->ev_used + 1], st));
        p->ev_used += 2;
    }
    p->gemm_flops_pending += 2.0 * M * N * (double)K;
    return OCMP_OK;
}

}  // namespace

int strip_create(const ocmp_space_s* s, Strip** out) {
    *out = nullptr;
    const int64_t n = s->ndof;
    if (n <= 0) return fail(OCMP_ERR_ARG, "strip preconditioner: empty space");
    const std::vector<int64_t>& rp = s->rowptr;
    const std::vector<int32_t>& col = s->col;
    std::vector<int64_t> mx(n), mn(n);
    for (int64_t r = 0; r < n; r++) {
        int64_t a = r, b = r;
        for (int64_t k = rp[r]; k < rp[r + 1]; k++) {
            a = std::min<int64_t>(a, col[k]);
            b = std::max<int64_t>(b, col[k]);
        }
        mn[r] = a;
        mx[r] = b;
    }
    auto* p = new Strip();
    p->s.push_back(0);
    while (p->s.back() < n) {
        int64_t nxt;
        if (p->s.size() == 1) nxt = mx[0] + 1;
        else {
            nxt = 0;
            for (int64_t r = p->s[p->s.size() - 2]; r < p->s.back(); r++) nxt = std::max(nxt, mx[r] + 1);
        }
        nxt = std::min<int64_t>(n, std::max<int64_t>(nxt, p->s.back() + 1));
        p->s.push_back(nxt);
    }
    p->K = (int)p->s.size() - 1;
    const int K = p->K;
    // every row must reach only its own and the neighbouring strips
    {
        int64_t k = 0;
        for (int64_t r = 0; r < n; r++) {
            while (r >= p->s[k + 1]) k++;
            const int64_t lo = k > 0 ? p->s[k - 1] : 0, hi = k + 2 <= K ? p->s[k + 2] : n;
            if (mn[r] < lo || mx[r] >= hi) {
                delete p;
                return fail(OCMP_ERR_UNSUPPORTED, "strip preconditioner: the pattern is not block tridiagonal over "
                                                  "its bandwidth strips (structurally unsymmetric)");
            }
        }
    }
    p->m.resize(K);
    p->mp.resize(K);
    p->goff.resize(K + 1);
    int64_t total = 0;
    for (int k = 0; k < K; k++) {
        p->m[k] = (int)(p->s[k + 1] - p->s[k]);
        p->mp[k] = pad(p->m[k]);
        p->goff[k] = total;
        total += (int64_t)p->mp[k] * p->mp[k];
        p->mp_max = std::max(p->mp_max, p->mp[k]);
    }
    p->goff[K] = total;
    if (p->mp_max > 16384) {
        const int mm = p->mp_max;
        delete p;
        return fail(OCMP_ERR_UNSUPPORTED, "strip preconditioner: a strip of " + std::to_string(mm) +
                                              " dofs exceeds the 16384-dof limit (number the dofs so the matrix is banded)");
    }
    // interface sets and coupling lists
    std::vector<int32_t> I, J, Iinv(n, -1), Jinv(n, -1);
    std::vector<int32_t> lo_ptr(n + 1, 0), hi_ptr(n + 1, 0), lo_pos, hi_pos;
    p->nI.assign(K, 0);
    p->nJ.assign(K, 0);
    p->ioff.assign(K + 1, 0);
    p->joff.assign(K + 1, 0);
    for (int k = 0; k < K; k++) {
        const int64_t s0 = p->s[k], s1 = p->s[k + 1];
        std::vector<char> inI(p->m[k], 0), inJ(p->m[k], 0);
        for (int64_t r = s0; r < s1; r++) {
            for (int64_t q = rp[r]; q < rp[r + 1]; q++) {
                const int64_t c = col[q];
                if (c < s0) inI[r - s0] = 1;
                if (c >= s1) inJ[r - s0] = 1;
            }
        }
        // column sides (structurally unsymmetric patterns): columns of this strip reached from the
        // neighbours' rows belong to the interface too
        if (k > 0)
            for (int64_t r = p->s[k - 1]; r < s0; r++)
                for (int64_t q = rp[r]; q < rp[r + 1]; q++)
                    if (col[q] >= s0) inI[col[q] - s0] = 1;
        if (k + 1 < K)
            for (int64_t r = s1; r < p->s[k + 2]; r++)
                for (int64_t q = rp[r]; q < rp[r + 1]; q++)
                    if (col[q] < s1) inJ[col[q] - s0] = 1;
        p->ioff[k] = (int64_t)I.size();
        p->joff[k] = (int64_t)J.size();
        for (int i = 0; i < p->m[k]; i++) {
            if (inI[i]) {
                Iinv[s0 + i] = p->nI[k]++;
                I.push_back(i);
            }
            if (inJ[i]) {
                Jinv[s0 + i] = p->nJ[k]++;
                J.push_back(i);
            }
        }
        p->nIp_max = std::max(p->nIp_max, pad(p->nI[k]));
        p->nJp_max = std::max(p->nJp_max, pad(p->nJ[k]));
        for (int64_t r = s0; r < s1; r++) {
            for (int64_t q = rp[r]; q < rp[r + 1]; q++) {
                if (col[q] < s0) lo_pos.push_back((int32_t)q);
                else if (col[q] >= s1) hi_pos.push_back((int32_t)q);
            }
            lo_ptr[r + 1] = (int32_t)lo_pos.size();
            hi_ptr[r + 1] = (int32_t)hi_pos.size();
        }
    }
    p->ioff[K] = (int64_t)I.size();
    p->joff[K] = (int64_t)J.size();
    const int ifp = std::max(p->nIp_max, p->nJp_max);
    const int64_t need = total * 4 + (int64_t)3 * ifp * ifp * 4 + (int64_t)2 * ifp * ifp * 4 +
                         (int64_t)p->mp_max * kNb * 8 + kNb * kNb * 4;
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    if ((size_t)need > fr) {
        delete p;
        return fail(OCMP_ERR_NOMEM, "strip preconditioner: the strip inverses need " + std::to_string(need >> 20) +
                                        " MiB of device memory");
    }
    int st = OCMP_OK;
    auto U = [&](auto** d, const auto& h) {
        if (!st) st = upload(d, h.data(), h.size());
    };
    U(&p->d_I, I);
    U(&p->d_J, J);
    U(&p->d_Iinv, Iinv);
    U(&p->d_Jinv, Jinv);
    U(&p->d_lo_ptr, lo_ptr);
    U(&p->d_lo_pos, lo_pos);
    U(&p->d_hi_ptr, hi_ptr);
    U(&p->d_hi_pos, hi_pos);
    auto A = [&](auto** d, size_t cnt) {
        if (!st) st = dalloc(d, cnt);
    };
    A(&p->d_G, (size_t)total);
    A(&p->d_Bt, (size_t)ifp * ifp);
    A(&p->d_Cc, (size_t)ifp * ifp);
    A(&p->d_Gjj, (size_t)ifp * ifp);
    A(&p->d_Tt, (size_t)ifp * ifp);
    A(&p->d_U, (size_t)ifp * ifp);
    A(&p->d_P, (size_t)kNb * kNb);
    A(&p->d_Ck, (size_t)p->mp_max * kNb);
    A(&p->d_Rt, (size_t)p->mp_max * kNb);
    A(&p->d_r, (size_t)p->mp_max);
    A(&p->d_flag, 2);
    if (!st && cudaEventCreate(&p->fev[0]) != cudaSuccess) st = fail(OCMP_ERR_CUDA, "cudaEventCreate");
    if (!st && cudaEventCreate(&p->fev[1]) != cudaSuccess) st = fail(OCMP_ERR_CUDA, "cudaEventCreate");
    if (!st) {
        const int tsm = (kNb * (kNb + 1) + kNb) * (int)sizeof(float);
        const int psm = (kNb * kNb + kNb * 33) * (int)sizeof(float);
        const int fsm = (kNb * kNb + 32 * (kNb + 1)) * (int)sizeof(float);
        if (cudaFuncSetAttribute(k_tile_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm) != cudaSuccess ||
            cudaFuncSetAttribute(k_panel_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, psm) != cudaSuccess ||
            cudaFuncSetAttribute(k_panel_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm) != cudaSuccess)
            st = fail(OCMP_ERR_CUDA, "strip preconditioner: shared-memory attribute");
    }
    p->bytes = total * 4 + (int64_t)(I.size() + J.size() + 2 * n + 2 * (n + 1) + lo_pos.size() + hi_pos.size()) * 4;
    if (st) {
        strip_free(p);
        delete p;
        return st;
    }
    *out = p;
    return OCMP_OK;
}

void strip_destroy(Strip* p) {
    if (!p) return;
    strip_free(p);
    delete p;
}

int strip_factor(Strip* p, const ocmp_space_s* s, const double* vals, cudaStream_t st) {
    const int K = p->K;
    p->ev_used = 0;
    p->gemm_flops_pending = 0;
    OCMP_CUDA(cudaEventRecord(p->fev[0], st));
    OCMP_CUDA(cudaMemsetAsync(p->d_flag, 0, 2 * sizeof(int), st));
    const int tsm = (kNb * (kNb + 1) + kNb) * (int)sizeof(float);
    const int psm = (kNb * kNb + kNb * 33) * (int)sizeof(float);
    const int fsm = (kNb * kNb + 32 * (kNb + 1)) * (int)sizeof(float);
    for (int k = 0; k < K; k++) {
        const int m = p->m[k], mp = p->mp[k];
        const int64_t s0 = p->s[k];
        float* S = p->d_G + p->goff[k];
        OCMP_CUDA(cudaMemsetAsync(S, 0, sizeof(float) * (size_t)mp * mp, st));
        OCMP_LAUNCH(k_fill_strip<<<nblk(mp, 128), 128, 0, st>>>(m, mp, s0, s->d_rowptr, s->d_col, vals, s->d_free, S));
        if (k > 0 && p->nI[k] > 0 && p->nJ[k - 1] > 0) {
            const int nI = p->nI[k], nJ = p->nJ[k - 1], nIp = pad(nI), nJp = pad(nJ);
            const int mpp = p->mp[k - 1];
            OCMP_CUDA(cudaMemsetAsync(p->d_Cc, 0, sizeof(float) * (size_t)nIp * nJp, st));
            OCMP_CUDA(cudaMemsetAsync(p->d_Bt, 0, sizeof(float) * (size_t)nIp * nJp, st));
            OCMP_LAUNCH(k_fill_iface<<<nblk(nI + nJ, 128), 128, 0, st>>>(
                nI, nJ, nJp, s0, p->s[k - 1], p->d_I + p->ioff[k], p->d_J + p->joff[k - 1], p->d_Iinv, p->d_Jinv,
                p->d_lo_ptr, p->d_lo_pos, p->d_hi_ptr, p->d_hi_pos, s->d_col, vals, s->d_free, p->d_Cc, p->d_Bt));
            OCMP_LAUNCH(k_gather_gjj<<<nblk((int64_t)nJp * nJp, 256), 256, 0, st>>>(
                nJ, nJp, p->d_J + p->joff[k - 1], p->d_G + p->goff[k - 1], mpp, p->d_Gjj));
            // Tt = Bt Gjj^T (= (G_JJ A_JI)^T), U = Cc Tt^T
            int r = gemm(p, nIp, nJp, nJp, p->d_Bt, nJp, p->d_Gjj, nJp, p->d_Tt, nJp, 1.f, 0.f, st);
            if (!r) r = gemm(p, nIp, nIp, nJp, p->d_Cc, nJp, p->d_Tt, nJp, p->d_U, nIp, 1.f, 0.f, st);
            if (r) return r;
            OCMP_LAUNCH(k_scatter_sub<<<nblk((int64_t)nI * nI, 256), 256, 0, st>>>(nI, nIp, p->d_I + p->ioff[k], p->d_U,
                                                                                  mp, S));
        }
        for (int t0 = 0; t0 < mp; t0 += kNb) {
            OCMP_LAUNCH(k_tile_inv<<<1, kTileThreads, tsm, st>>>(S, mp, t0, p->d_P, p->d_flag));
            OCMP_LAUNCH(k_panel_prep<<<mp / 32, 256, psm, st>>>(S, mp, t0, p->d_P, p->d_Rt, p->d_Ck));
            int r = gemm(p, mp, mp, kNb, p->d_Ck, kNb, p->d_Rt, kNb, S, mp, -1.f, 1.f, st);
            if (r) return r;
            OCMP_LAUNCH(k_panel_finish<<<mp / 32, 256, fsm, st>>>(S, mp, t0, p->d_P, p->d_Rt, p->d_Ck));
        }
    }
    OCMP_CUDA(cudaGetLastError());
    OCMP_CUDA(cudaEventRecord(p->fev[1], st));
    int flags[2] = {0, 0};
    OCMP_CUDA(cudaMemcpyAsync(flags, p->d_flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    OCMP_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    OCMP_CUDA(cudaEventElapsedTime(&ms, p->fev[0], p->fev[1]));
    p->factor_ms = ms;
    const int flag = flags[0];
    p->singular = flag;
    if (flags[1]) return fail(OCMP_TIMEOUT, "strip preconditioner: a tensor-core product gave up a bounded wait");
    p->gemm_flops = p->gemm_flops_pending;
    p->gemm_ms = 0;
    for (size_t q = 0; q + 1 < p->ev_used; q += 2) {
        float e = 0;
        OCMP_CUDA(cudaEventElapsedTime(&e, p->ev[q], p->ev[q + 1]));
        p->gemm_ms += e;
    }
    if (flag) return fail(OCMP_BREAKDOWN, "strip preconditioner: " + std::to_string(flag) +
                                              " zero or non-finite pivots in the strip factorisation");
    return OCMP_OK;
}

template <class T>
int strip_apply(Strip* p, const ocmp_space_s* s, const double* vals, const T* v, const double* scale, int j, T* z,
                const int* flags, cudaStream_t st) {
    const int K = p->K;
    for (int k = 0; k < K; k++) {
        const int m = p->m[k], mp = p->mp[k];
        const int64_t s0 = p->s[k];
        OCMP_LAUNCH(k_fwd_rhs<T><<<nblk(mp, 256), 256, 0, st>>>(m, mp, s0, p->d_lo_ptr, p->d_lo_pos, s->d_col, vals,
                                                               s->d_free, v, scale, j, z, p->d_r, flags));
        OCMP_LAUNCH(k_strip_gemv<T><<<nblk(m, 8), 256, 0, st>>>(m, mp, p->d_G + p->goff[k], p->d_r, z + s0, 0, flags));
    }
    for (int k = K - 2; k >= 0; k--) {
        const int m = p->m[k], mp = p->mp[k];
        const int64_t s0 = p->s[k];
        OCMP_LAUNCH(k_bwd_rhs<T><<<nblk(mp, 256), 256, 0, st>>>(m, mp, s0, p->d_hi_ptr, p->d_hi_pos, s->d_col, vals,
                                                               s->d_free, z, p->d_r, flags));
        OCMP_LAUNCH(k_strip_gemv<T><<<nblk(m, 8), 256, 0, st>>>(m, mp, p->d_G + p->goff[k], p->d_r, z + s0, 1, flags));
    }
    return OCMP_OK;
}
template int strip_apply<double>(Strip*, const ocmp_space_s*, const double*, const double*, const double*, int,
                                 double*, const int*, cudaStream_t);
template int strip_apply<float>(Strip*, const ocmp_space_s*, const double*, const float*, const double*, int, float*,
                                const int*, cudaStream_t);

template <class T>
int strip_add(int64_t n, const T* z, double* x, cudaStream_t st) {
    OCMP_LAUNCH(k_add_to<T><<<nblk(n, 256), 256, 0, st>>>(n, z, x, nullptr));
    return OCMP_OK;
}
template int strip_add<double>(int64_t, const double*, double*, cudaStream_t);
template int strip_add<float>(int64_t, const float*, double*, cudaStream_t);

void strip_stats(const Strip* p, ocmp_strip_stats_t* o) {
    o->nstrips = p->K;
    o->max_strip = p->mp_max;
    o->bytes = p->bytes;
    o->factor_ms = p->factor_ms;
    o->gemm_ms = p->gemm_ms;
    o->gemm_flops = p->gemm_flops;
    o->singular_tiles = p->singular;
    o->gemm_kind = p->gemm_kind;
}

void strip_set_timing(Strip* p, bool on) { p->timing = on; }
void strip_set_gemm(Strip* p, int kind) { p->gemm_kind = kind; }

}  // namespace ocmp

using namespace ocmp;

extern "C" int ocmp_dense_gemm_nt(int32_t kind, int32_t M, int32_t N, int32_t K, const float* A, int64_t lda,
                                  const float* B, int64_t ldb, float* C, int64_t ldc, float alpha, float beta,
                                  void* stream) {
    if (!A || !B || !C) return fail(OCMP_ERR_ARG, "ocmp_dense_gemm_nt: null argument");
    if (kind != 0 && kind != 1) return fail(OCMP_ERR_ARG, "ocmp_dense_gemm_nt: kind is 0 (SIMT) or 1 (tensor cores)");
    if (lda < K || ldb < K || ldc < N) return fail(OCMP_ERR_ARG, "ocmp_dense_gemm_nt: leading dimension too small");
    cudaStream_t st = (cudaStream_t)stream;
    if (kind == 0) {
        if (M <= 0 || N <= 0 || K <= 0 || M % GB || N % GB || K % GK || (lda | ldb | ldc) & 3)
            return fail(OCMP_ERR_ARG, "ocmp_dense_gemm_nt: M, N must be multiples of 128, K of 16");
        const dim3 g(N / GB, M / GB);
        OCMP_LAUNCH(sgemm_nt<<<g, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta));
        OCMP_CUDA(cudaGetLastError());
        return OCMP_OK;
    }
    int* err = nullptr;
    OCMP_CUDA(cudaMallocAsync((void**)&err, sizeof(int), st));
    OCMP_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    int r = tc_gemm_nt(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, err, st);
    int h = 0;
    if (!r && cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        r = fail(OCMP_ERR_CUDA, "ocmp_dense_gemm_nt: flag copy");
    cudaFreeAsync(err, st);
    if (!r) OCMP_CUDA(cudaStreamSynchronize(st));
    if (!r && h) r = fail(OCMP_TIMEOUT, "ocmp_dense_gemm_nt: a bounded wait of the tensor-core product gave up");
    return r;
}

namespace ocmp {

}  // namespace ocmp
