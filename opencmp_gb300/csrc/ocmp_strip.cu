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
// x_k = y_k - G_k A_k,k+1 x_k+1. Every G_k is kept explicitly (FP32, dense), so each sweep step is
// one dense matrix-vector product instead of two triangular solves; the sweeps of a
// preconditioner application are replayed from a CUDA graph.
//
// Within a strip the dofs are ordered [N | I]: I = the dofs coupled to the previous strip (the
// only rows and columns the Schur update A_k,k-1 S_{k-1}^-1 A_k-1,k touches), N = the rest, each
// part padded to a multiple of 128 with decoupled unit rows. G_k is the block Gauss-Jordan inverse
// of S_k with 128 x 128 diagonal-tile pivots (each tile inverted with partial pivoting inside it):
// per tile one small inversion, two panel kernels and one rank-128 update of the whole strip, the
// dominant flops. Since the Schur update only adds to the II block, the N pivots can be eliminated
// before it:
//   phase 1 (side streams, all strips independent): fill S_k, eliminate its N tiles;
//   phase 2 (the caller's stream, strip after strip): S_k[I,I] -= A[I,J] G_k-1[J,J] A[J,I] (two
//     dense products over the interface, J = the dofs of strip k-1 coupled to strip k), then
//     eliminate the I tiles.
// On a structured triangle mesh half of each strip's elements touch the previous row of elements,
// so phase 2, the sequential chain, does half of the pivot tiles.
// The dense products are C = beta C + alpha A B^T with both operands K-contiguous: FP32 SIMT
// (sgemm_nt) or the tensor cores (tc_gemm_nt, ocmp_tcgemm.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "ocmp_internal.h"

namespace ocmp {

constexpr int kNb = 128;   // Gauss-Jordan tile and padding granule
constexpr int kSide = 3;   // side streams of phase 1

struct StripWork {
    float* P = nullptr;    // pivot-tile inverse, kNb x kNb
    float* Ck = nullptr;   // column panel, mp_max x kNb
    float* Rt = nullptr;   // row panel (transposed), mp_max x kNb
};

struct Strip {
    int K = 0;
    std::vector<int64_t> s;          // K + 1 strip boundaries
    std::vector<int> m, mp;          // strip sizes and padded sizes (nNp + nIp)
    std::vector<int> nN, nNp, nI, nJ;
    std::vector<int64_t> goff;       // offsets of G_k in d_G (floats)
    std::vector<int64_t> poff;       // offsets of strip k's permutation in d_perm
    std::vector<int64_t> ioff, joff; // offsets into d_I / d_J
    int mp_max = 0, nIp_max = 0, nJp_max = 0;
    int32_t* d_perm = nullptr;       // per strip position: local dof, -1 on padding
    int32_t* d_I = nullptr;          // I_k as positions in strip k's order (nNp + a)
    int32_t* d_J = nullptr;          // J_k as positions in strip k's order
    int32_t* jrow = nullptr;         // J_k as local dofs
    int32_t* d_pinv = nullptr;       // per dof: its position in its strip's order
    int32_t* d_Iinv = nullptr;       // per dof: its index in I of its strip, or -1
    int32_t* d_Jinv = nullptr;       // per dof: its index in J of its strip, or -1
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
    StripWork work[kSide + 1];       // [0]: the caller's stream, [1..]: side streams
    float* d_r = nullptr;            // solve scratch (one strip)
    int* d_flag = nullptr;           // [0] pivot tiles that were singular or non-finite, [1] a tensor-core
                                     // product whose bounded wait gave up
    int64_t bytes = 0;
    cudaStream_t side[kSide] = {};
    cudaStream_t chain = nullptr;    // phase 2, at the highest stream priority so that the side streams'
                                     // products never hold the chain's kernels back
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_done = nullptr;
    std::vector<cudaEvent_t> ev_phase1;
    // sweeps replayed from graphs: [0] gated on the solver's convergence flag, [1] not gated
    cudaStream_t cap = nullptr;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    unsigned long long gkernels[2] = {0, 0};
    const void* g_z[2] = {nullptr, nullptr};
    const int* g_flags[2] = {nullptr, nullptr};
    const double* g_vals[2] = {nullptr, nullptr};
    int g_type[2] = {0, 0};
    // statistics of the last factorisation
    bool timing = false;
    std::vector<cudaEvent_t> ev;
    size_t ev_used = 0;
    std::vector<int> ev_tag;            // per event pair: 0 product, 1 tile inversion, 2 panels
    double part_ms[3] = {0, 0, 0};
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
// S (mp x mp, zeroed) <- the strip's diagonal block in the strip's [N | I] order; unit diagonal on
// constrained rows and on the padding. pinv: per dof its position in its strip's order.
__global__ void k_fill_strip(int mp, int64_t s0, const int32_t* __restrict__ perm, const int32_t* __restrict__ pinv,
                             const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                             const double* __restrict__ vals, const uint8_t* __restrict__ freed, int64_t s1,
                             float* __restrict__ S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mp) return;
    float* row = S + (int64_t)i * mp;
    const int ld = perm[i];
    if (ld < 0 || !freed[s0 + ld]) {
        row[i] = 1.f;
        return;
    }
    const int64_t r = s0 + ld;
    for (int32_t k = rp[r]; k < rp[r + 1]; k++) {
        const int64_t c = col[k];
        if (c >= s0 && c < s1 && freed[c]) row[pinv[c]] = (float)vals[k];
    }
}

// Interface blocks of the boundary between strip k-1 (start sp) and strip k (start s0):
// Cc[a, b] = A[I_a, J_b] (rows of strip k, columns of strip k-1) and Bt[a, b] = A[J_b, I_a].
// Irow / Jrow: the local dofs of I_k and J_k-1.
__global__ void k_fill_iface(int nI, int nJ, int nJp, int64_t s0, int64_t sp, const int32_t* __restrict__ Irow,
                             const int32_t* __restrict__ Jrow, const int32_t* __restrict__ Iinv,
                             const int32_t* __restrict__ Jinv, const int32_t* __restrict__ lo_ptr,
                             const int32_t* __restrict__ lo_pos, const int32_t* __restrict__ hi_ptr,
                             const int32_t* __restrict__ hi_pos, const int32_t* __restrict__ col,
                             const double* __restrict__ vals, const uint8_t* __restrict__ freed, float* __restrict__ Cc,
                             float* __restrict__ Bt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nI) {
        const int64_t r = s0 + Irow[t];
        if (!freed[r]) return;
        for (int32_t q = lo_ptr[r]; q < lo_ptr[r + 1]; q++) {
            const int32_t k = lo_pos[q];
            const int64_t c = col[k];
            const int b = Jinv[c];
            if (freed[c] && b >= 0) Cc[(int64_t)t * nJp + b] = (float)vals[k];
        }
    } else if (t < nI + nJ) {
        const int bj = t - nI;
        const int64_t r = sp + Jrow[bj];
        if (!freed[r]) return;
        for (int32_t q = hi_ptr[r]; q < hi_ptr[r + 1]; q++) {
            const int32_t k = hi_pos[q];
            const int64_t c = col[k];
            const int a = Iinv[c];
            if (freed[c] && a >= 0) Bt[(int64_t)a * nJp + bj] = (float)vals[k];
        }
    }
}

// Gjj[a, b] = G[J_a, J_b] (positions in the previous strip's order; zero padding)
__global__ void k_gather_gjj(int nJ, int nJp, const int32_t* __restrict__ J, const float* __restrict__ G, int mpG,
                             float* __restrict__ Gjj) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nJp * nJp) return;
    const int a = (int)(t / nJp), b = (int)(t % nJp);
    Gjj[t] = (a < nJ && b < nJ) ? G[(int64_t)J[a] * mpG + J[b]] : 0.f;
}

// S[nNp + a, nNp + c] -= U[a, c]: the I block is contiguous in the strip's order
__global__ void k_sub_block(int nI, int nIp, int nNp, const float* __restrict__ U, int mp, float* __restrict__ S) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nI * nI) return;
    const int a = (int)(t / nI), c = (int)(t % nI);
    S[(int64_t)(nNp + a) * mp + nNp + c] -= U[(int64_t)a * nIp + c];
}

// ------------------------------------------------------------------ block Gauss-Jordan
// P <- inverse of the tile S[t0:t0+128, t0:t0+128] by Gauss-Jordan with partial pivoting inside
// the tile. The tile stays in registers (thread t holds column t % 128 of rows t / 128 + 8 j) and
// rows are never moved: step k takes as pivot the largest |a_rk| over the rows not yet used, and
// the row and column permutation is applied when the result is written (P[step(r)][piv(c)] =
// M[r][c]). Per step the eight owners of column k publish it with their best unused row, every
// thread reduces the eight candidates, the owners of the pivot row publish that row
// (double-buffered in shared memory): two barriers per step. A zero or non-finite pivot is
// counted in *flag and replaced by a tiny value.
constexpr int kTileThreads = 1024;
constexpr int kTileSmem = 0;
__global__ void __launch_bounds__(kTileThreads) k_tile_inv(const float* __restrict__ S, int mp, int t0,
                                                           float* __restrict__ P, int* __restrict__ flag) {
    __shared__ float colk[2][kNb];
    __shared__ float prow[2][kNb];
    __shared__ float cval[2][8];
    __shared__ int crow[2][8];
    __shared__ int piv[kNb];
    __shared__ int step[kNb];
    const int tid = threadIdx.x, c = tid & (kNb - 1), r0 = tid >> 7;
    constexpr int R = kNb / 8;   // rows per thread
    float v[R];
#pragma unroll
    for (int j = 0; j < R; j++) v[j] = S[(int64_t)(t0 + r0 + 8 * j) * mp + t0 + c];
    unsigned usedmask = 0;       // which of this thread's rows have been pivots
    for (int k = 0; k < kNb; k++) {
        const int b = k & 1;
        if (c == k) {
            float best = -1.f;
            int bi = kNb;
#pragma unroll
            for (int j = 0; j < R; j++) {
                colk[b][r0 + 8 * j] = v[j];
                const float a = (usedmask >> j) & 1u ? -1.f : fabsf(v[j]);
                if (a > best) {
                    best = a;
                    bi = r0 + 8 * j;
                }
            }
            cval[b][r0] = best;
            crow[b][r0] = bi;
        }
        __syncthreads();
        float best = cval[b][0];
        int p = crow[b][0];
#pragma unroll
        for (int g = 1; g < 8; g++) {
            const float a = cval[b][g];
            const int r = crow[b][g];
            if (a > best || (a == best && r < p)) {
                best = a;
                p = r;
            }
        }
        if (p >= kNb) {   // every remaining |a_rk| is NaN: take the smallest unused row
            p = kNb;
#pragma unroll
            for (int g = 0; g < 8; g++) p = min(p, crow[b][g] < kNb ? crow[b][g] : kNb);
            if (p >= kNb) p = k;
        }
        float pv = colk[b][p];
        if (!(fabsf(pv) > 0.f) || !isfinite(pv)) {
            if (tid == 0) atomicAdd(flag, 1);
            pv = 1e-30f;
        }
        const float d = 1.f / pv;
        if (r0 == (p & 7)) {
            // v[p >> 3] without dynamic register indexing
            float x = 0.f;
#pragma unroll
            for (int j = 0; j < R; j++)
                if (j == (p >> 3)) x = v[j];
            prow[b][c] = (c == k ? 1.f : x) * d;
            usedmask |= 1u << (p >> 3);
        }
        __syncthreads();
        if (tid == 0) {
            piv[k] = p;
            step[p] = k;
        }
        const float pr = prow[b][c];
#pragma unroll
        for (int j = 0; j < R; j++) {
            const int r = r0 + 8 * j;
            if (r == p) v[j] = pr;
            else v[j] = (c == k ? 0.f : v[j]) - colk[b][r] * pr;
        }
    }
    __syncthreads();
    const int pc = piv[c];
#pragma unroll
    for (int j = 0; j < R; j++) {
        const int r = r0 + 8 * j;
        P[step[r] * kNb + pc] = v[j];
    }
}

// For the 32 columns c0..c0+31: Rt[c, r] = sum_l P[r, l] S[t0 + l, c] (the pivot rows times P, stored
// transposed), and for the 32 rows c0..c0+31: Ck[i, l] = S[i, t0 + l], zero on the pivot rows.
constexpr int kPrepSmem = (kNb * kNb + kNb * 33) * (int)sizeof(float);
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
        const float sv = Sc[l * 33 + j];
#pragma unroll
        for (int q = 0; q < 16; q++) acc[q] = fmaf(Ps[(rw + 8 * q) * kNb + l], sv, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 16; q++) Rt[(int64_t)(c0 + j) * kNb + rw + 8 * q] = acc[q];
}

// After the rank-128 update: S[i, t0 + l] = -(Ck P)[i, l] for the non-pivot rows i of this block's 32
// rows; S[t0 + r, c] = Rt[c, r] for this block's 32 columns c outside the tile, P inside it.
constexpr int kFinishSmem = (kNb * kNb + 32 * (kNb + 1)) * (int)sizeof(float);
__global__ void __launch_bounds__(256) k_panel_finish(float* __restrict__ S, int mp, int t0,
                                                      const float* __restrict__ P, const float* __restrict__ Rt,
                                                      const float* __restrict__ Ck) {
    extern __shared__ float sm[];
    float* Ps = sm;                  // kNb x kNb
    float* Cs = sm + kNb * kNb;      // 32 x (kNb + 1)
    const int tid = threadIdx.x, c0 = blockIdx.x * 32;
    for (int e = tid; e < kNb * kNb; e += 256) Ps[e] = P[e];
    for (int e = tid; e < 32 * kNb; e += 256)
        Cs[(e / kNb) * (kNb + 1) + e % kNb] = Ck[(int64_t)(c0 + e / kNb) * kNb + e % kNb];
    __syncthreads();
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
    for (int e = tid; e < 32 * kNb; e += 256) {
        const int jj = e / kNb, r = e % kNb;
        const int c = c0 + jj;
        const float v = (c >= t0 && c < t0 + kNb) ? Ps[r * kNb + (c - t0)] : Rt[(int64_t)c * kNb + r];
        S[(int64_t)(t0 + r) * mp + c] = v;
    }
}

// ------------------------------------------------------------------ sweeps
// z = sc v with sc = scale[j] (the GMRES basis vector into the preconditioner's input)
template <class T>
__global__ void k_scale_copy(int64_t n, const T* __restrict__ v, const double* __restrict__ scale, int j,
                             T* __restrict__ z, const int* __restrict__ flags) {
    if (flags && flags[0]) return;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) z[i] = (T)((double)v[i] * scale[j]);
}

// forward right-hand side of strip [s0, s1) in the strip's order: r_p = z_i - sum A[i, c] z_c over
// the entries whose column lies in the previous strip (z holds that strip's y, and this strip's
// input); zero on constrained rows and on the padding
template <class T>
__global__ void k_fwd_rhs(int mp, int64_t s0, const int32_t* __restrict__ perm, const int32_t* __restrict__ lo_ptr,
                          const int32_t* __restrict__ lo_pos, const int32_t* __restrict__ col,
                          const double* __restrict__ vals, const uint8_t* __restrict__ freed, const T* __restrict__ z,
                          float* __restrict__ r, const int* __restrict__ flags) {
    if (flags && flags[0]) return;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= mp) return;
    const int ld = perm[p];
    if (ld < 0 || !freed[s0 + ld]) {
        r[p] = 0.f;
        return;
    }
    const int64_t row = s0 + ld;
    float acc = (float)z[row];
    for (int32_t q = lo_ptr[row]; q < lo_ptr[row + 1]; q++) {
        const int32_t k = lo_pos[q];
        const int32_t c = col[k];
        if (freed[c]) acc -= (float)vals[k] * (float)z[c];
    }
    r[p] = acc;
}

// backward right-hand side: r_p = sum A[i, c] z_c over the entries in the next strip
template <class T>
__global__ void k_bwd_rhs(int mp, int64_t s0, const int32_t* __restrict__ perm, const int32_t* __restrict__ hi_ptr,
                          const int32_t* __restrict__ hi_pos, const int32_t* __restrict__ col,
                          const double* __restrict__ vals, const uint8_t* __restrict__ freed, const T* __restrict__ z,
                          float* __restrict__ r, const int* __restrict__ flags) {
    if (flags && flags[0]) return;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= mp) return;
    const int ld = perm[p];
    if (ld < 0 || !freed[s0 + ld]) {
        r[p] = 0.f;
        return;
    }
    const int64_t row = s0 + ld;
    float acc = 0.f;
    for (int32_t q = hi_ptr[row]; q < hi_ptr[row + 1]; q++) {
        const int32_t k = hi_pos[q];
        const int32_t c = col[k];
        if (freed[c]) acc += (float)vals[k] * (float)z[c];
    }
    r[p] = acc;
}

// z_i = (G r)_p (mode 0) or z_i -= (G r)_p (mode 1), i = the local dof at position p; a warp per
// row, 16-byte loads (mp is a multiple of 128)
template <class T>
__global__ void __launch_bounds__(256) k_strip_gemv(int mp, int64_t s0, const int32_t* __restrict__ perm,
                                                    const float* __restrict__ G, const float* __restrict__ r,
                                                    T* __restrict__ z, int mode, const int* __restrict__ flags) {
    if (flags && flags[0]) return;
    const int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= mp) return;
    const int ld = perm[row];
    if (ld < 0) return;
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
        T* zi = z + s0 + ld;
        if (mode == 0) *zi = (T)acc;
        else *zi = (T)((float)*zi - acc);
    }
}

template <class T>
__global__ void k_add_to(int64_t n, const T* __restrict__ z, double* __restrict__ x) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) x[i] += (double)z[i];
}

// ------------------------------------------------------------------ host helpers
void strip_free(Strip* p) {
    void* ps[] = {p->d_perm, p->d_I, p->d_J, p->jrow, p->d_pinv, p->d_Iinv, p->d_Jinv, p->d_lo_ptr, p->d_lo_pos, p->d_hi_ptr,
                  p->d_hi_pos, p->d_G, p->d_Bt, p->d_Cc, p->d_Gjj, p->d_Tt, p->d_U, p->d_r, p->d_flag};
    for (void* q : ps) dfree(q);
    for (auto& w : p->work) {
        dfree(w.P);
        dfree(w.Ck);
        dfree(w.Rt);
    }
    for (cudaEvent_t e : p->ev) cudaEventDestroy(e);
    for (cudaEvent_t e : p->ev_phase1) cudaEventDestroy(e);
    for (cudaEvent_t e : p->fev)
        if (e) cudaEventDestroy(e);
    if (p->ev_start) cudaEventDestroy(p->ev_start);
    if (p->ev_done) cudaEventDestroy(p->ev_done);
    if (p->chain) cudaStreamDestroy(p->chain);
    for (cudaStream_t q : p->side)
        if (q) cudaStreamDestroy(q);
    for (cudaGraphExec_t g : p->gexec)
        if (g) cudaGraphExecDestroy(g);
    if (p->cap) cudaStreamDestroy(p->cap);
}

// timing of the factorisation's kernels by class (ocmp_solver_strip_timing): an event pair around
// each launch on its stream
int tbegin(Strip* p, cudaStream_t st) {
    if (!p->timing) return OCMP_OK;
    while (p->ev.size() < p->ev_used + 2) {
        cudaEvent_t e;
        OCMP_CUDA(cudaEventCreate(&e));
        p->ev.push_back(e);
    }
    OCMP_CUDA(cudaEventRecord(p->ev[p->ev_used], st));
    return OCMP_OK;
}
int tend(Strip* p, cudaStream_t st, int tag) {
    if (!p->timing) return OCMP_OK;
    OCMP_CUDA(cudaEventRecord(p->ev[p->ev_used + 1], st));
    p->ev_used += 2;
    p->ev_tag.push_back(tag);
    return OCMP_OK;
}

int gemm(Strip* p, int M, int N, int K, const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
         float alpha, float beta, cudaStream_t st) {
    if (M % GB || N % GB || K % 32 || M <= 0 || N <= 0 || K <= 0)
        return fail(OCMP_ERR_ARG, "strip gemm: sizes must be multiples of the tile");
    const bool t = p->timing;
    if (t && tbegin(p, st)) return OCMP_ERR_CUDA;
    if (p->gemm_kind == 1) {
        const int r = tc_gemm_nt(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, p->d_flag + 1, st);
        if (r) return r;
    } else {
        const dim3 g(N / GB, M / GB);
        OCMP_LAUNCH(sgemm_nt<<<g, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta));
    }
    if (t && tend(p, st, 0)) return OCMP_ERR_CUDA;
    p->gemm_flops_pending += 2.0 * M * N * (double)K;
    return OCMP_OK;
}

// Gauss-Jordan over the pivot tiles [t_begin, t_end) of S (mp x mp) on stream st with workspace w
int gj_tiles(Strip* p, float* S, int mp, int t_begin, int t_end, const StripWork& w, cudaStream_t st) {
    for (int t0 = t_begin; t0 < t_end; t0 += kNb) {
        int r = tbegin(p, st);
        OCMP_LAUNCH(k_tile_inv<<<1, kTileThreads, kTileSmem, st>>>(S, mp, t0, w.P, p->d_flag));
        if (!r) r = tend(p, st, 1);
        if (!r) r = tbegin(p, st);
        OCMP_LAUNCH(k_panel_prep<<<mp / 32, 256, kPrepSmem, st>>>(S, mp, t0, w.P, w.Rt, w.Ck));
        if (!r) r = tend(p, st, 2);
        if (!r) r = gemm(p, mp, mp, kNb, w.Ck, kNb, w.Rt, kNb, S, mp, -1.f, 1.f, st);
        if (!r) r = tbegin(p, st);
        OCMP_LAUNCH(k_panel_finish<<<mp / 32, 256, kFinishSmem, st>>>(S, mp, t0, w.P, w.Rt, w.Ck));
        if (!r) r = tend(p, st, 2);
        if (r) return r;
    }
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
    // consecutive strips merge (the block-tridiagonal structure survives) until a strip holds at
    // least kMergeMin dofs: narrow bands (a P1 Laplacian's band is one row of vertices) would
    // otherwise give many small strips, whose sweeps are launch-bound
    {
        constexpr int64_t kMergeMin = 1024, kMergeMax = 4096;
        std::vector<int64_t> merged{0};
        size_t q = 1;
        while (q < p->s.size()) {
            int64_t end = p->s[q++];
            while (q < p->s.size() && end - merged.back() < kMergeMin && p->s[q] - merged.back() <= kMergeMax)
                end = p->s[q++];
            merged.push_back(end);
        }
        p->s.swap(merged);
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
    // interface sets: I_k = dofs of strip k coupled to strip k-1 (by their row or their column),
    // J_k = dofs of strip k coupled to strip k+1
    p->m.resize(K);
    p->nN.resize(K);
    p->nNp.resize(K);
    p->nI.assign(K, 0);
    p->nJ.assign(K, 0);
    std::vector<std::vector<char>> inI(K), inJ(K);
    for (int k = 0; k < K; k++) {
        p->m[k] = (int)(p->s[k + 1] - p->s[k]);
        inI[k].assign(p->m[k], 0);
        inJ[k].assign(p->m[k], 0);
    }
    for (int k = 0; k < K; k++) {
        const int64_t s0 = p->s[k], s1 = p->s[k + 1];
        for (int64_t r = s0; r < s1; r++)
            for (int64_t q = rp[r]; q < rp[r + 1]; q++) {
                const int64_t c = col[q];
                if (c < s0) {
                    inI[k][r - s0] = 1;
                    inJ[k - 1][c - p->s[k - 1]] = 1;
                } else if (c >= s1) {
                    inJ[k][r - s0] = 1;
                    inI[k + 1][c - s1] = 1;
                }
            }
    }
    p->mp.resize(K);
    p->goff.resize(K + 1);
    p->poff.resize(K + 1);
    p->ioff.assign(K + 1, 0);
    p->joff.assign(K + 1, 0);
    std::vector<int32_t> perm, pinv(n, -1), Ipos, Jpos, Iinv(n, -1), Jinv(n, -1);
    int64_t total = 0;
    for (int k = 0; k < K; k++) {
        const int m = p->m[k];
        const int64_t s0 = p->s[k];
        std::vector<int32_t> Nl, Il;
        for (int i = 0; i < m; i++) (inI[k][i] ? Il : Nl).push_back(i);
        p->nN[k] = (int)Nl.size();
        p->nNp[k] = pad(p->nN[k]);
        p->nI[k] = (int)Il.size();
        p->mp[k] = p->nNp[k] + pad(p->nI[k]);
        p->goff[k] = total;
        total += (int64_t)p->mp[k] * p->mp[k];
        p->poff[k] = (int64_t)perm.size();
        p->mp_max = std::max(p->mp_max, p->mp[k]);
        std::vector<int32_t> pm(p->mp[k], -1);
        for (int q = 0; q < p->nN[k]; q++) pm[q] = Nl[q];
        for (int q = 0; q < p->nI[k]; q++) pm[p->nNp[k] + q] = Il[q];
        for (int q = 0; q < p->mp[k]; q++)
            if (pm[q] >= 0) pinv[s0 + pm[q]] = q;
        perm.insert(perm.end(), pm.begin(), pm.end());
        p->ioff[k] = (int64_t)Ipos.size();
        for (int q = 0; q < p->nI[k]; q++) {
            Iinv[s0 + Il[q]] = q;
            Ipos.push_back(Il[q]);         // local dofs (fill_iface); their positions are nNp + q
        }
        p->joff[k] = (int64_t)Jpos.size();
        for (int i = 0; i < m; i++)
            if (inJ[k][i]) {
                Jinv[s0 + i] = p->nJ[k]++;
                Jpos.push_back(i);
            }
        p->nIp_max = std::max(p->nIp_max, pad(p->nI[k]));
        p->nJp_max = std::max(p->nJp_max, pad(p->nJ[k]));
    }
    p->goff[K] = total;
    p->poff[K] = (int64_t)perm.size();
    p->ioff[K] = (int64_t)Ipos.size();
    p->joff[K] = (int64_t)Jpos.size();
    if (p->mp_max > 16384) {
        const int mm = p->mp_max;
        delete p;
        return fail(OCMP_ERR_UNSUPPORTED, "strip preconditioner: a strip of " + std::to_string(mm) +
                                              " dofs exceeds the 16384-dof limit (number the dofs so the matrix is banded)");
    }
    // J_k as positions in strip k's order (the Schur update gathers G_k[J, J]); the local dofs stay in
    // Jrow for the interface fill
    std::vector<int32_t> Jp(Jpos.size());
    for (int k = 0; k < K; k++)
        for (int64_t q = p->joff[k]; q < p->joff[k + 1]; q++) Jp[q] = pinv[p->s[k] + Jpos[q]];
    std::vector<int32_t> lo_ptr(n + 1, 0), hi_ptr(n + 1, 0), lo_pos, hi_pos;
    for (int k = 0; k < K; k++) {
        const int64_t s0 = p->s[k], s1 = p->s[k + 1];
        for (int64_t r = s0; r < s1; r++) {
            for (int64_t q = rp[r]; q < rp[r + 1]; q++) {
                if (col[q] < s0) lo_pos.push_back((int32_t)q);
                else if (col[q] >= s1) hi_pos.push_back((int32_t)q);
            }
            lo_ptr[r + 1] = (int32_t)lo_pos.size();
            hi_ptr[r + 1] = (int32_t)hi_pos.size();
        }
    }
    const int ifp = std::max(p->nIp_max, p->nJp_max);
    const int64_t need = total * 4 + (int64_t)5 * ifp * ifp * 4 + (int64_t)(kSide + 1) * (2 * p->mp_max * kNb + kNb * kNb) * 4;
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
    U(&p->d_perm, perm);
    U(&p->d_pinv, pinv);
    U(&p->d_I, Ipos);
    U(&p->d_J, Jp);
    U(&p->d_Iinv, Iinv);
    U(&p->d_Jinv, Jinv);
    U(&p->d_lo_ptr, lo_ptr);
    U(&p->d_lo_pos, lo_pos);
    U(&p->d_hi_ptr, hi_ptr);
    U(&p->d_hi_pos, hi_pos);
    p->bytes = total * 4 + (int64_t)(perm.size() + Ipos.size() + Jp.size() + 3 * n + 2 * (n + 1) + lo_pos.size() +
                                     hi_pos.size()) * 4;
    auto A = [&](auto** d, size_t cnt) {
        if (!st) st = dalloc(d, cnt);
    };
    A(&p->d_G, (size_t)total);
    A(&p->d_Bt, (size_t)ifp * ifp);
    A(&p->d_Cc, (size_t)ifp * ifp);
    A(&p->d_Gjj, (size_t)ifp * ifp);
    A(&p->d_Tt, (size_t)ifp * ifp);
    A(&p->d_U, (size_t)ifp * ifp);
    for (auto& w : p->work) {
        A(&w.P, (size_t)kNb * kNb);
        A(&w.Ck, (size_t)p->mp_max * kNb);
        A(&w.Rt, (size_t)p->mp_max * kNb);
    }
    A(&p->d_r, (size_t)p->mp_max);
    A(&p->d_flag, 2);
    U(&p->jrow, Jpos);
    p->bytes += (int64_t)Jpos.size() * 4;
    if (!st && (cudaEventCreateWithFlags(&p->fev[0], cudaEventDefault) != cudaSuccess ||
                cudaEventCreateWithFlags(&p->fev[1], cudaEventDefault) != cudaSuccess ||
                cudaEventCreateWithFlags(&p->ev_start, cudaEventDisableTiming) != cudaSuccess))
        st = fail(OCMP_ERR_CUDA, "cudaEventCreate");
    for (int q = 0; q < kSide && !st; q++)
        if (cudaStreamCreateWithFlags(&p->side[q], cudaStreamNonBlocking) != cudaSuccess)
            st = fail(OCMP_ERR_CUDA, "cudaStreamCreateWithFlags");
    if (!st && cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking) != cudaSuccess)
        st = fail(OCMP_ERR_CUDA, "cudaStreamCreateWithFlags");
    if (!st) {
        int lo = 0, hi = 0;
        if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess ||
            cudaStreamCreateWithPriority(&p->chain, cudaStreamNonBlocking, hi) != cudaSuccess ||
            cudaEventCreateWithFlags(&p->ev_done, cudaEventDisableTiming) != cudaSuccess)
            st = fail(OCMP_ERR_CUDA, "strip preconditioner: chain stream");
    }
    p->ev_phase1.assign(K, nullptr);
    for (int k = 0; k < K && !st; k++)
        if (cudaEventCreateWithFlags(&p->ev_phase1[k], cudaEventDisableTiming) != cudaSuccess)
            st = fail(OCMP_ERR_CUDA, "cudaEventCreate");
    if (!st) {
        if (cudaFuncSetAttribute(k_tile_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmem) != cudaSuccess ||
            cudaFuncSetAttribute(k_panel_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, kPrepSmem) != cudaSuccess ||
            cudaFuncSetAttribute(k_panel_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, kFinishSmem) != cudaSuccess)
            st = fail(OCMP_ERR_CUDA, "strip preconditioner: shared-memory attribute");
    }
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
    p->ev_tag.clear();
    p->gemm_flops_pending = 0;
    OCMP_CUDA(cudaEventRecord(p->fev[0], st));
    OCMP_CUDA(cudaMemsetAsync(p->d_flag, 0, 2 * sizeof(int), st));
    OCMP_CUDA(cudaEventRecord(p->ev_start, st));
    for (int q = 0; q < kSide; q++) OCMP_CUDA(cudaStreamWaitEvent(p->side[q], p->ev_start, 0));
    cudaStream_t cs = p->chain;
    OCMP_CUDA(cudaStreamWaitEvent(cs, p->ev_start, 0));
    // phase 1: fill every strip and eliminate its N pivots, strips spread over the side streams
    for (int k = 0; k < K; k++) {
        const int q = k % kSide;
        cudaStream_t ss = p->side[q];
        const int mp = p->mp[k];
        float* S = p->d_G + p->goff[k];
        OCMP_CUDA(cudaMemsetAsync(S, 0, sizeof(float) * (size_t)mp * mp, ss));
        OCMP_LAUNCH(k_fill_strip<<<nblk(mp, 128), 128, 0, ss>>>(mp, p->s[k], p->d_perm + p->poff[k], p->d_pinv, s->d_rowptr,
                                                               s->d_col, vals, s->d_free, p->s[k + 1], S));
        int r = gj_tiles(p, S, mp, 0, p->nNp[k], p->work[1 + q], ss);
        if (r) return r;
        OCMP_CUDA(cudaEventRecord(p->ev_phase1[k], ss));
    }
    // phase 2 on the chain stream, strip after strip: the Schur update from the previous strip's
    // inverse, then the I pivots
    for (int k = 0; k < K; k++) {
        OCMP_CUDA(cudaStreamWaitEvent(cs, p->ev_phase1[k], 0));
        const int mp = p->mp[k];
        const int64_t s0 = p->s[k];
        float* S = p->d_G + p->goff[k];
        if (k > 0 && p->nI[k] > 0 && p->nJ[k - 1] > 0) {
            const int nI = p->nI[k], nJ = p->nJ[k - 1], nIp = pad(nI), nJp = pad(nJ);
            OCMP_CUDA(cudaMemsetAsync(p->d_Cc, 0, sizeof(float) * (size_t)nIp * nJp, cs));
            OCMP_CUDA(cudaMemsetAsync(p->d_Bt, 0, sizeof(float) * (size_t)nIp * nJp, cs));
            OCMP_LAUNCH(k_fill_iface<<<nblk(nI + nJ, 128), 128, 0, cs>>>(
                nI, nJ, nJp, s0, p->s[k - 1], p->d_I + p->ioff[k], p->jrow + p->joff[k - 1], p->d_Iinv, p->d_Jinv,
                p->d_lo_ptr, p->d_lo_pos, p->d_hi_ptr, p->d_hi_pos, s->d_col, vals, s->d_free, p->d_Cc, p->d_Bt));
            OCMP_LAUNCH(k_gather_gjj<<<nblk((int64_t)nJp * nJp, 256), 256, 0, cs>>>(
                nJ, nJp, p->d_J + p->joff[k - 1], p->d_G + p->goff[k - 1], p->mp[k - 1], p->d_Gjj));
            // Tt = Bt Gjj^T (= (G_JJ A_JI)^T), U = Cc Tt^T
            int r = gemm(p, nIp, nJp, nJp, p->d_Bt, nJp, p->d_Gjj, nJp, p->d_Tt, nJp, 1.f, 0.f, cs);
            if (!r) r = gemm(p, nIp, nIp, nJp, p->d_Cc, nJp, p->d_Tt, nJp, p->d_U, nIp, 1.f, 0.f, cs);
            if (r) return r;
            OCMP_LAUNCH(k_sub_block<<<nblk((int64_t)nI * nI, 256), 256, 0, cs>>>(nI, nIp, p->nNp[k], p->d_U, mp, S));
        }
        int r = gj_tiles(p, S, mp, p->nNp[k], mp, p->work[0], cs);
        if (r) return r;
    }
    OCMP_CUDA(cudaGetLastError());
    OCMP_CUDA(cudaEventRecord(p->ev_done, cs));
    OCMP_CUDA(cudaStreamWaitEvent(st, p->ev_done, 0));
    OCMP_CUDA(cudaEventRecord(p->fev[1], st));
    int flags[2] = {0, 0};
    OCMP_CUDA(cudaMemcpyAsync(flags, p->d_flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    OCMP_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    OCMP_CUDA(cudaEventElapsedTime(&ms, p->fev[0], p->fev[1]));
    p->factor_ms = ms;
    p->singular = flags[0];
    if (flags[1]) return fail(OCMP_TIMEOUT, "strip preconditioner: a tensor-core product gave up a bounded wait");
    p->gemm_flops = p->gemm_flops_pending;
    p->gemm_ms = 0;
    for (double& x : p->part_ms) x = 0;
    for (size_t q = 0; q + 1 < p->ev_used; q += 2) {
        float e = 0;
        OCMP_CUDA(cudaEventElapsedTime(&e, p->ev[q], p->ev[q + 1]));
        p->part_ms[p->ev_tag[q / 2]] += e;
    }
    p->gemm_ms = p->part_ms[0];
    if (flags[0]) return fail(OCMP_BREAKDOWN, "strip preconditioner: " + std::to_string(flags[0]) +
                                                  " zero or non-finite pivots in the strip factorisation");
    return OCMP_OK;
}

namespace {
// the two sweeps, in place on z (input: the vector to precondition)
template <class T>
void sweeps(Strip* p, const ocmp_space_s* s, const double* vals, T* z, const int* flags, cudaStream_t st) {
    const int K = p->K;
    for (int k = 0; k < K; k++) {
        const int mp = p->mp[k];
        const int32_t* pm = p->d_perm + p->poff[k];
        OCMP_LAUNCH(k_fwd_rhs<T><<<nblk(mp, 256), 256, 0, st>>>(mp, p->s[k], pm, p->d_lo_ptr, p->d_lo_pos, s->d_col,
                                                               vals, s->d_free, z, p->d_r, flags));
        OCMP_LAUNCH(k_strip_gemv<T><<<nblk(mp, 8), 256, 0, st>>>(mp, p->s[k], pm, p->d_G + p->goff[k], p->d_r, z, 0,
                                                                flags));
    }
    for (int k = K - 2; k >= 0; k--) {
        const int mp = p->mp[k];
        const int32_t* pm = p->d_perm + p->poff[k];
        OCMP_LAUNCH(k_bwd_rhs<T><<<nblk(mp, 256), 256, 0, st>>>(mp, p->s[k], pm, p->d_hi_ptr, p->d_hi_pos, s->d_col,
                                                               vals, s->d_free, z, p->d_r, flags));
        OCMP_LAUNCH(k_strip_gemv<T><<<nblk(mp, 8), 256, 0, st>>>(mp, p->s[k], pm, p->d_G + p->goff[k], p->d_r, z, 1,
                                                                flags));
    }
}
}  // namespace

template <class T>
int strip_apply(Strip* p, const ocmp_space_s* s, const double* vals, const T* v, const double* scale, int j, T* z,
                const int* flags, cudaStream_t st) {
    const int64_t n = s->ndof;
    if (v != z) {
        if (scale) OCMP_LAUNCH(k_scale_copy<T><<<nblk(n, 256), 256, 0, st>>>(n, v, scale, j, z, flags));
        else OCMP_CUDA(cudaMemcpyAsync(z, v, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
    }
    // the sweeps (4 launches per strip) replay from a graph captured on first use for this
    // (vector, flag, matrix) on the library's own stream
    const int gi = flags ? 0 : 1;
    const int type = sizeof(T) == 8 ? 1 : 2;
    if (!p->gexec[gi] || p->g_z[gi] != z || p->g_flags[gi] != flags || p->g_vals[gi] != vals || p->g_type[gi] != type) {
        if (p->gexec[gi]) {
            cudaGraphExecDestroy(p->gexec[gi]);
            p->gexec[gi] = nullptr;
        }
        cudaGraph_t g;
        const unsigned long long l0 = g_launches.load();
        OCMP_CUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
        sweeps<T>(p, s, vals, z, flags, p->cap);
        OCMP_CUDA(cudaStreamEndCapture(p->cap, &g));
        p->gkernels[gi] = g_launches.load() - l0;
        g_launches.fetch_sub(p->gkernels[gi]);
        cudaError_t e = cudaGraphInstantiate(&p->gexec[gi], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (strip sweeps)");
        p->g_z[gi] = z;
        p->g_flags[gi] = flags;
        p->g_vals[gi] = vals;
        p->g_type[gi] = type;
    }
    OCMP_CUDA(cudaGraphLaunch(p->gexec[gi], st));
    g_launches.fetch_add(p->gkernels[gi]);
    return OCMP_OK;
}
template int strip_apply<double>(Strip*, const ocmp_space_s*, const double*, const double*, const double*, int,
                                 double*, const int*, cudaStream_t);
template int strip_apply<float>(Strip*, const ocmp_space_s*, const double*, const float*, const double*, int, float*,
                                const int*, cudaStream_t);

template <class T>
int strip_add(int64_t n, const T* z, double* x, cudaStream_t st) {
    OCMP_LAUNCH(k_add_to<T><<<nblk(n, 256), 256, 0, st>>>(n, z, x));
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
    o->tile_ms = p->part_ms[1];
    o->panel_ms = p->part_ms[2];
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
