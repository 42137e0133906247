// Strip direct preconditioner of libopencmp_gpu.so (sm_103a): the GPU counterpart of the sparse
// direct solve in opencmp/models/base_model.py:906-922 (a.mat.Inverse(freedofs, 'pardiso' |
// 'umfpack'), then gfu += inv * (L - A gfu)), used as the preconditioner of FP64-refined GMRES.
//
// The dofs are cut into consecutive strips [s_k, s_k+1) chosen so that the matrix is block
// tridiagonal over them: strip k's rows reach no further than strip k+1 (greedy over the row
// bandwidth, or, when the pattern repeats with a period, uniform strips of that period: one row of
// elements of a structured mesh numbered row by row). Block elimination over the strips (the block Thomas algorithm) needs, per strip,
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
//   phase 2 (the chain stream, strip after strip): S_k[I,I] -= A[I,J] G_k-1[J,J] A[J,I] (J = the
//     dofs of strip k-1 coupled to strip k; A[I,J] and A[J,I] hold a few entries per row, so the
//     update is two sparse-times-dense kernels over per-dof coupling lists), then eliminate the I
//     tiles.
// On a structured triangle mesh half of each strip's elements touch the previous row of elements,
// so phase 2, the sequential chain, does half of the pivot tiles.
// Newton-Schulz path, for a strip whose N dofs fall into independent groups of at most 32 (the
// elements of a row of DG elements that do not touch the previous row): phase 1 inverts the groups
// (a warp each) and forms the interface complement W0 = S_II - S_IN S_NN^-1 S_NI with one dense
// product; phase 2 subtracts the Schur update from W0 and inverts it by Newton-Schulz iteration
// started from the previous strip's interface inverse (two steps on a uniform DG mesh), then
// assembles G_k from the 2 x 2 block inverse with three dense products.
// The dense products are C = beta C + alpha A B^T with both operands K-contiguous: FP32 SIMT
// (sgemm_nt) or the tensor cores (tc_gemm_nt, ocmp_tcgemm.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>
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
    float* d_G = nullptr;            // the explicit strip inverses
    // per I dof (over all strips, indexed like d_I): its couplings to the previous strip's J, as
    // entries [cptr[i], cptr[i+1]) of (index b in J, CSR position of A[I_i, J_b], of A[J_b, I_i])
    int32_t* d_cptr = nullptr;
    int32_t* d_cb = nullptr;
    int32_t* d_crow = nullptr;
    int32_t* d_ccol = nullptr;
    int cmax = 0;                    // longest list
    float* d_T = nullptr;            // Schur update scratch: T = G_k-1[J, J] A[J, I] (nJ x nIp)
    StripWork work[kSide + 1];       // [0]: the caller's stream, [1..]: side streams
    float* d_r = nullptr;            // solve scratch (one strip)
    // ELL coupling lists of the sweeps' right-hand sides: per strip, the forward list (columns in
    // the previous strip) then the backward one (columns in the next), entry-major; the values and
    // the free rows' dofs are refreshed by every factorisation
    std::vector<int64_t> eoff;       // per strip: first entry
    std::vector<int> elo, ehi;       // per strip: widths
    int32_t* d_prow = nullptr;       // per position (over all strips): its dof, -1 on padding
    int32_t* d_rdof = nullptr;       // per position: its dof if free, else -1
    int32_t* d_erow = nullptr;
    int32_t* d_ecol = nullptr;       // per entry: the column's dof, -1 on padding
    int32_t* d_epos = nullptr;       // per entry: its CSR position, -1 on padding
    float* d_ev = nullptr;           // per entry: the value, 0 where the row or the column is constrained
    int64_t nell = 0, npos = 0;
    int* d_flag = nullptr;           // [0] pivot tiles that were singular or non-finite, [1] a tensor-core
                                     // product whose bounded wait gave up
    int64_t bytes = 0;
    int64_t schur_flops_pending = 0;
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
    double factor_ms = 0, gemm_ms = 0, gemm_flops = 0, gemm_flops_pending = 0, gemm_bytes = 0, gemm_bytes_pending = 0;
    int singular = 0;
    int gemm_kind = 0;               // 0: FP32 SIMT, 1: tensor cores (3xTF32)
    // Newton-Schulz path (strips whose N dofs form small independent groups, e.g. the elements of a
    // row of DG elements that do not touch the previous row)
    std::vector<char> fast;          // per strip
    std::vector<int64_t> gofs;       // per strip: first group in d_gptr
    std::vector<int> ngrp;           // per strip: groups
    int32_t* d_gptr = nullptr;       // group offsets into d_gidx (concatenated per strip, each ends with its total)
    int32_t* d_gidx = nullptr;       // group members: positions in the strip's order (all in N)
    int32_t* d_gcomp = nullptr;      // per member: its component within the group (start << 8 | size)
    float* d_Yt[kSide] = {};         // phase 1 scratch per side stream: Y^T
    float* d_Xa = nullptr;           // chain scratch: Newton-Schulz iterates, residual, transposes
    float* d_Xb = nullptr;
    float* d_R = nullptr;
    float* d_Rt = nullptr;
    float* d_Xt = nullptr;
    float* d_H[3] = {};              // the last three interface inverses, newest first (Newton-Schulz starts)
    int h_n[3] = {0, 0, 0};          // their padded sizes (0: none)
    bool schulz = true;              // Newton-Schulz path on (off: block Gauss-Jordan throughout)
    float* d_T1 = nullptr;
    float* d_Zt = nullptr;
    unsigned* d_rmax = nullptr;
    unsigned* h_rmax = nullptr;      // pinned
    int nfast = 0;
    int ns_iters = 0, ns_strips = 0, ns_fallbacks = 0;
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

// Schur update of strip k (rows and columns of its I block, I dofs at global s0 + Irow[i]) from the
// previous strip's inverse G (its J dofs at positions Jp, local dofs Jrow, strip start sp):
//   T[b, c] = sum_{(d, A[J_d, I_c]) in list(c)} G[J_b, J_d] A[J_d, I_c]           (k_schur_t)
//   S[I_a, I_c] -= sum_{(b, A[I_a, J_b]) in list(a)} A[I_a, J_b] T[b, c]           (k_schur_u)
// An entry counts only when both its row and its column dof are free (the constrained rows and
// columns of the strips are unit rows and columns).
constexpr int kSchurRows = 8;   // rows b of T per thread in k_schur_t
__global__ void __launch_bounds__(128) k_schur_t(int nI, int nJ, int nIp, int64_t s0, int64_t sp,
                                                 const int32_t* __restrict__ Irow, const int32_t* __restrict__ Jrow,
                                                 const int32_t* __restrict__ Jp, const int32_t* __restrict__ cptr,
                                                 const int32_t* __restrict__ cb, const int32_t* __restrict__ ccol,
                                                 const double* __restrict__ vals, const uint8_t* __restrict__ freed,
                                                 const float* __restrict__ G, int mpG, float* __restrict__ T) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x, b0 = blockIdx.y * kSchurRows;
    if (c >= nIp) return;
    const float* grow[kSchurRows];
#pragma unroll
    for (int u = 0; u < kSchurRows; u++) grow[u] = G + (int64_t)Jp[min(b0 + u, nJ - 1)] * mpG;
    float acc[kSchurRows];
#pragma unroll
    for (int u = 0; u < kSchurRows; u++) acc[u] = 0.f;
    if (c < nI && freed[s0 + Irow[c]]) {
        for (int32_t e = cptr[c]; e < cptr[c + 1]; e++) {
            const int d = cb[e];
            const int32_t q = ccol[e];
            if (q < 0 || !freed[sp + Jrow[d]]) continue;
            const float v = (float)vals[q];
            const int jc = Jp[d];
#pragma unroll
            for (int u = 0; u < kSchurRows; u++) acc[u] = fmaf(grow[u][jc], v, acc[u]);
        }
    }
#pragma unroll
    for (int u = 0; u < kSchurRows; u++)
        if (b0 + u < nJ) T[(int64_t)(b0 + u) * nIp + c] = acc[u];
}

// four columns c per thread (T's rows are 16-byte aligned: nIp is a multiple of 128)
__global__ void __launch_bounds__(128) k_schur_u(int nI, int nIp, int nNp, int64_t s0, int64_t sp,
                                                 const int32_t* __restrict__ Irow, const int32_t* __restrict__ Jrow,
                                                 const int32_t* __restrict__ cptr, const int32_t* __restrict__ cb,
                                                 const int32_t* __restrict__ crow, const double* __restrict__ vals,
                                                 const uint8_t* __restrict__ freed, const float* __restrict__ T,
                                                 float* __restrict__ S, int mp) {
    const int c = 4 * (blockIdx.x * blockDim.x + threadIdx.x), a = blockIdx.y;
    if (c >= nI || !freed[s0 + Irow[a]]) return;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int32_t e = cptr[a]; e < cptr[a + 1]; e++) {
        const int b = cb[e];
        const int32_t q = crow[e];
        if (q < 0 || !freed[sp + Jrow[b]]) continue;
        const float v = (float)vals[q];
        const float4 t = *reinterpret_cast<const float4*>(T + (int64_t)b * nIp + c);
        acc.x = fmaf(v, t.x, acc.x);
        acc.y = fmaf(v, t.y, acc.y);
        acc.z = fmaf(v, t.z, acc.z);
        acc.w = fmaf(v, t.w, acc.w);
    }
    float* srow = S + (int64_t)(nNp + a) * mp + nNp + c;
    const float av[4] = {acc.x, acc.y, acc.z, acc.w};
#pragma unroll
    for (int u = 0; u < 4; u++)
        if (c + u < nI) srow[u] -= av[u];
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

// ------------------------------------------------------------------ Newton-Schulz path
// Inverse of each small group of N dofs (b <= 32 positions, packed from independent components),
// a warp per group, in place in the strip. Lane c owns column c of the group's block in shared
// memory; gcomp gives each position its component (start << 8 | size) within the group, and every
// component is eliminated on its own lanes at the same time: Gauss-Jordan with partial pivoting
// over the component's rows (each lane of a component scans them for the pivot, so all agree),
// rows never moved (as in k_tile_inv).
constexpr int kGroupWarps = 8;
__global__ void __launch_bounds__(32 * kGroupWarps) k_group_inv(float* __restrict__ S, int mp, const int32_t* __restrict__ gptr,
                                                                const int32_t* __restrict__ gidx,
                                                                const int32_t* __restrict__ gcomp, int ngroups,
                                                                int* __restrict__ flag) {
    __shared__ float tile[kGroupWarps][32][33];
    __shared__ float colk[kGroupWarps][32];
    __shared__ int pivs[kGroupWarps][32], steps[kGroupWarps][32];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = blockIdx.x * kGroupWarps + wl;
    if (grp >= ngroups) return;
    const int g0 = gptr[grp], b = gptr[grp + 1] - g0;
    const int32_t* g = gidx + g0;
    float(*t)[33] = tile[wl];
    const bool in = lane < b;
    const int cw = in ? gcomp[g0 + lane] : 0;
    const int cs = cw >> 8, cn = in ? (cw & 255) : 0;
    if (in) {
        const int myg = g[lane];
        for (int r = cs; r < cs + cn; r++) t[r][lane] = S[(int64_t)g[r] * mp + myg];
    }
    int maxn = cn;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) maxn = max(maxn, __shfl_xor_sync(0xffffffffu, maxn, off));
    __syncwarp();
    unsigned used = 0;
    for (int k = 0; k < maxn; k++) {
        const bool act = k < cn;
        const int pc = cs + k;
        int p = cs;
        float nk = 0.f;
        if (act) {
            float best = -1.f;
            for (int r = cs; r < cs + cn; r++) {
                if ((used >> r) & 1u) continue;
                float a = fabsf(t[r][pc]);
                if (!(a >= 0.f)) a = 0.f;
                if (a > best) {
                    best = a;
                    p = r;
                }
            }
            float pv = t[p][pc];
            if (!(fabsf(pv) > 0.f) || !isfinite(pv)) {
                if (lane == pc) atomicAdd(flag, 1);
                pv = 1e-30f;
            }
            nk = (lane == pc ? 1.f : t[p][lane]) / pv;
            colk[wl][lane] = t[lane][pc];   // row `lane` is in this component
        }
        __syncwarp();
        if (act) {
            for (int r = cs; r < cs + cn; r++)
                t[r][lane] = r == p ? nk : (lane == pc ? 0.f : t[r][lane]) - colk[wl][r] * nk;
            if (lane == pc) {
                pivs[wl][pc] = p;
                steps[wl][p] = pc;
            }
            used |= 1u << p;
        }
        __syncwarp();
    }
    if (in) {
        const int pcol = g[pivs[wl][lane]];
        for (int r = cs; r < cs + cn; r++) S[(int64_t)g[steps[wl][r]] * mp + pcol] = t[r][lane];
    }
}

// Y = X S_NI in place (rows of each group, columns of I): a block per group and 128 columns, a
// thread per column (X is zero between the group's components)
__global__ void __launch_bounds__(128) k_group_y(float* __restrict__ S, int mp, int nNp,
                                                 const int32_t* __restrict__ gptr, const int32_t* __restrict__ gidx) {
    __shared__ float X[32][33];
    __shared__ int gs[32];
    const int grp = blockIdx.x, tid = threadIdx.x;
    const int g0 = gptr[grp], b = gptr[grp + 1] - g0;
    if (tid < b) gs[tid] = gidx[g0 + tid];
    __syncthreads();
    for (int e = tid; e < b * b; e += 128) X[e / b][e % b] = S[(int64_t)gs[e / b] * mp + gs[e % b]];
    __syncthreads();
    const int c = nNp + blockIdx.y * 128 + tid;
    float sv[32];
#pragma unroll
    for (int q = 0; q < 32; q++) sv[q] = q < b ? S[(int64_t)gs[q < b ? q : 0] * mp + c] : 0.f;
    for (int r = 0; r < b; r++) {
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < 32; q++)
            if (q < b) acc = fmaf(X[r][q], sv[q], acc);
        S[(int64_t)gs[r] * mp + c] = acc;
    }
}

// S_IN <- Z = -S_IN X in place (rows i of I, the N columns of each group): a block per group and
// 128 rows, a thread per row, which reads its row's group entries before writing them
__global__ void __launch_bounds__(128) k_group_z(float* __restrict__ S, int mp, int nNp, int nIp,
                                                 const int32_t* __restrict__ gptr, const int32_t* __restrict__ gidx) {
    __shared__ float X[32][33];
    __shared__ int gs[32];
    const int grp = blockIdx.x, tid = threadIdx.x;
    const int g0 = gptr[grp], b = gptr[grp + 1] - g0;
    if (tid < b) gs[tid] = gidx[g0 + tid];
    __syncthreads();
    for (int e = tid; e < b * b; e += 128) X[e / b][e % b] = S[(int64_t)gs[e / b] * mp + gs[e % b]];
    __syncthreads();
    const int i = blockIdx.y * 128 + tid;
    if (i >= nIp) return;
    float* row = S + (int64_t)(nNp + i) * mp;
    float sv[32];
#pragma unroll
    for (int q = 0; q < 32; q++) sv[q] = q < b ? row[gs[q < b ? q : 0]] : 0.f;
    for (int r = 0; r < b; r++) {
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < 32; q++)
            if (q < b) acc = fmaf(sv[q], X[q][r], acc);
        row[gs[r]] = -acc;
    }
}

// dst (cols x rows, leading dimension ldd) = src^T (rows x cols, leading dimension lds); 32 x 32 tiles
__global__ void k_transpose(const float* __restrict__ src, int64_t lds, int rows, int cols, float* __restrict__ dst,
                            int64_t ldd) {
    __shared__ float tl[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32, tx = threadIdx.x, ty = threadIdx.y;
    for (int j = ty; j < 32; j += 8) {
        const int r = by + j, c = bx + tx;
        tl[j][tx] = (r < rows && c < cols) ? src[(int64_t)r * lds + c] : 0.f;
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        const int r = bx + j, c = by + tx;   // dst row = src column
        if (r < cols && c < rows) dst[(int64_t)r * ldd + c] = tl[tx][j];
    }
}

// dst = scale * src (rows x cols, leading dimensions) or, with src == null, the identity
__global__ void k_copy2d(const float* __restrict__ src, int64_t lds, int rows, int cols, float* __restrict__ dst,
                         int64_t ldd, float scale) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)rows * cols) return;
    const int r = (int)(t / cols), c = (int)(t % cols);
    dst[(int64_t)r * ldd + c] = src ? scale * src[(int64_t)r * lds + c] : (r == c ? 1.f : 0.f);
}

// X0 = c1 H1 + c2 H2 + c3 H3 over n4 float4s (c3 = 0: H3 unused)
__global__ void k_extrap(int64_t n4, const float4* __restrict__ h1, const float4* __restrict__ h2,
                         const float4* __restrict__ h3, float c1, float c2, float c3, float4* __restrict__ x) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n4) return;
    const float4 a = h1[t];
    const float4 b = h2 ? h2[t] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 c = h3 ? h3[t] : make_float4(0.f, 0.f, 0.f, 0.f);
    x[t] = make_float4(c1 * a.x + c2 * b.x + c3 * c.x, c1 * a.y + c2 * b.y + c3 * c.y, c1 * a.z + c2 * b.z + c3 * c.z,
                       c1 * a.w + c2 * b.w + c3 * c.w);
}

// *out = max over rows of sum |A[r, :]| (the infinity norm; non-negative floats order like their
// bits, NaN above all): a warp per row
__global__ void k_infnorm(const float* __restrict__ A, int64_t lda, int rows, int cols, unsigned* __restrict__ out) {
    const int r = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (r >= rows) return;
    const float* a = A + (int64_t)r * lda;
    float sm = 0.f;
    for (int c = lane; c < cols; c += 32) sm += fabsf(a[c]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, off);
    if (lane == 0) atomicMax(out, sm == sm ? __float_as_uint(sm) : 0x7FFFFFFFu);
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

// right-hand side of a strip step in the strip's order, from its ELL list (L entries per position,
// entry-major: entry e of position q at e * mp + q): forward r_q = z_i - sum A[i, c] z_c over the
// previous strip's columns, backward r_q = sum A[i, c] z_c over the next strip's; zero on
// constrained rows and on the padding (rdof = -1)
template <class T>
__global__ void k_strip_rhs(int mp, int L, int fwd, const int32_t* __restrict__ rdof, const int32_t* __restrict__ ecol,
                            const float* __restrict__ ev, const T* __restrict__ z, float* __restrict__ r,
                            const int* __restrict__ flags) {
    if (flags && flags[0]) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= mp) return;
    const int row = rdof[q];
    float acc = 0.f;
    for (int e = 0; e < L; e++) {
        const int cc = ecol[(int64_t)e * mp + q];
        if (cc >= 0) acc = fmaf(ev[(int64_t)e * mp + q], (float)z[cc], acc);
    }
    r[q] = row < 0 ? 0.f : (fwd ? (float)z[row] - acc : acc);
}

// z_i = (G r)_p (mode 0) or z_i -= (G r)_p (mode 1), i = the local dof at position p. A block of
// 8 warps takes 8 rows, a warp per row; r is staged in shared memory, and each lane keeps eight
// 16-byte loads of G in flight (streamed past L1). mp is a multiple of 128.
constexpr int kGemvDepth = 8;
template <class T>
__global__ void __launch_bounds__(256) k_strip_gemv(int mp, int64_t s0, const int32_t* __restrict__ perm,
                                                    const float* __restrict__ G, const float* __restrict__ r,
                                                    T* __restrict__ z, int mode, const int* __restrict__ flags) {
    extern __shared__ float4 rs[];
    if (flags && flags[0]) return;
    const int nq = mp / 4;
    const float4* r4 = reinterpret_cast<const float4*>(r);
    for (int i = threadIdx.x; i < nq; i += blockDim.x) rs[i] = r4[i];
    __syncthreads();
    const int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= mp) return;
    const int ld = perm[row];
    if (ld < 0) return;
    const float4* g = reinterpret_cast<const float4*>(G + (int64_t)row * mp);
    float acc = 0.f;
    for (int q0 = lane; q0 < nq; q0 += 32 * kGemvDepth) {
        float4 a[kGemvDepth];
#pragma unroll
        for (int u = 0; u < kGemvDepth; u++)
            if (q0 + 32 * u < nq) a[u] = __ldcs(g + q0 + 32 * u);
#pragma unroll
        for (int u = 0; u < kGemvDepth; u++)
            if (q0 + 32 * u < nq) {
                const float4 b = rs[q0 + 32 * u];
                acc = fmaf(a[u].x, b.x, acc);
                acc = fmaf(a[u].y, b.y, acc);
                acc = fmaf(a[u].z, b.z, acc);
                acc = fmaf(a[u].w, b.w, acc);
            }
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

// the ELL right-hand-side values and the free rows' dofs of every strip, after an assembly
__global__ void k_ell_refresh(int64_t nent, const int32_t* __restrict__ erow, const int32_t* __restrict__ ecol,
                              const int32_t* __restrict__ epos, const double* __restrict__ vals,
                              const uint8_t* __restrict__ freed, float* __restrict__ ev, int64_t npos,
                              const int32_t* __restrict__ prow, int32_t* __restrict__ rdof) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < nent) {
        const int32_t q = epos[t];
        ev[t] = (q >= 0 && freed[erow[t]] && freed[ecol[t]]) ? (float)vals[q] : 0.f;
    }
    if (t < npos) {
        const int32_t d = prow[t];
        rdof[t] = (d >= 0 && freed[d]) ? d : -1;
    }
}

// ------------------------------------------------------------------ host helpers
void strip_free(Strip* p) {
    void* ps[] = {p->d_perm, p->d_I, p->d_J, p->jrow, p->d_pinv, p->d_G, p->d_cptr, p->d_cb, p->d_crow, p->d_ccol, p->d_T, p->d_r, p->d_flag};
    for (void* q : ps) dfree(q);
    for (auto& w : p->work) {
        dfree(w.P);
        dfree(w.Ck);
        dfree(w.Rt);
    }
    void* qs2[] = {p->d_prow, p->d_rdof, p->d_erow, p->d_ecol, p->d_epos, p->d_ev};
    for (void* q : qs2) dfree(q);
    void* qs[] = {p->d_gptr, p->d_gidx, p->d_gcomp, p->d_Xa, p->d_Xb, p->d_R, p->d_Rt, p->d_Xt, p->d_T1, p->d_Zt, p->d_rmax,
                  p->d_H[0], p->d_H[1], p->d_H[2]};
    for (void* q : qs) dfree(q);
    for (float* q : p->d_Yt) dfree(q);
    if (p->h_rmax) cudaFreeHost(p->h_rmax);
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
    // operands read once, C written (and read when beta != 0): the product's algorithmic bytes
    p->gemm_bytes_pending += 4.0 * ((double)M * K + (double)N * K + (beta != 0.f ? 2.0 : 1.0) * M * (double)N);
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

int transpose(const float* src, int64_t lds, int rows, int cols, float* dst, int64_t ldd, cudaStream_t st) {
    const dim3 g(nblk(cols, 32), nblk(rows, 32)), b(32, 8);
    OCMP_LAUNCH(k_transpose<<<g, b, 0, st>>>(src, lds, rows, cols, dst, ldd));
    return OCMP_OK;
}
int copy2d(const float* src, int64_t lds, int rows, int cols, float* dst, int64_t ldd, float scale, cudaStream_t st) {
    OCMP_LAUNCH(k_copy2d<<<nblk((int64_t)rows * cols, 256), 256, 0, st>>>(src, lds, rows, cols, dst, ldd, scale));
    return OCMP_OK;
}

// Phase 1 of a strip whose N block is block diagonal (groups of at most 32 positions): X = S_NN^-1
// group by group, S_NI <- Y = X S_NI, S_II <- W0 = S_II - S_IN Y (one dense product), S_IN <- Z =
// -S_IN X. The strip then holds [[X, Y], [Z, W0]].
int phase1_groups(Strip* p, int k, float* S, int q, cudaStream_t ss) {
    const int mp = p->mp[k], nNp = p->nNp[k], nIp = mp - nNp, ng = p->ngrp[k];
    const int32_t* gp = p->d_gptr + p->gofs[k];
    int r = tbegin(p, ss);
    OCMP_LAUNCH(k_group_inv<<<nblk(ng, kGroupWarps), 32 * kGroupWarps, 0, ss>>>(S, mp, gp, p->d_gidx, p->d_gcomp, ng,
                                                                              p->d_flag));
    if (!r) r = tend(p, ss, 1);
    OCMP_LAUNCH(k_group_y<<<dim3(ng, nIp / 128), 128, 0, ss>>>(S, mp, nNp, gp, p->d_gidx));
    if (!r) r = transpose(S + nNp, mp, nNp, nIp, p->d_Yt[q], nNp, ss);
    if (!r) r = gemm(p, nIp, nIp, nNp, S + (int64_t)nNp * mp, mp, p->d_Yt[q], nNp, S + (int64_t)nNp * mp + nNp, mp, -1.f,
                     1.f, ss);
    if (r) return r;
    OCMP_LAUNCH(k_group_z<<<dim3(ng, nblk(nIp, 128)), 128, 0, ss>>>(S, mp, nNp, nIp, gp, p->d_gidx));
    return OCMP_OK;
}

// Inverse of the interface Schur complement W = S_II (n x n, leading dimension mp) into a buffer
// of the chain (returned in *X, its transpose in d_Xt). Newton-Schulz X <- X + X R, R = I - W X,
// started from the previous strips' interface inverses extrapolated along the strips (quadratic
// from three, linear from two, the last one alone; the interface complements of the strips of a
// row-by-row structured mesh vary smoothly from row to row). The step squares R, so with
// rho = ||R||_inf read back after each product: rho <= kSchulzTol: X is taken; rho^2 <= kSchulzTol:
// one more step is taken unchecked; a step that does not reduce rho (or a non-finite rho, or
// kSchulzMax steps) falls back to block Gauss-Jordan on a copy of W, as does a strip without a
// previous inverse of its size.
constexpr float kSchulzTol = 1e-5f;
constexpr int kSchulzMax = 8;
int invert_interface(Strip* p, const float* W, int mp, int n, float** X, cudaStream_t cs) {
    float* cur = p->d_Xa;
    float* nxt = p->d_Xb;
    int hist = 0;
    while (hist < 3 && p->h_n[hist] == n) hist++;
    bool ok = false;
    if (p->schulz && hist > 0) {
        const int64_t n4 = (int64_t)n * n / 4;
        const float c[3][3] = {{1.f, 0.f, 0.f}, {2.f, -1.f, 0.f}, {3.f, -3.f, 1.f}};
        const float* cc = c[hist - 1];
        OCMP_LAUNCH(k_extrap<<<nblk(n4, 256), 256, 0, cs>>>(
            n4, reinterpret_cast<const float4*>(p->d_H[0]), hist > 1 ? reinterpret_cast<const float4*>(p->d_H[1]) : nullptr,
            hist > 2 ? reinterpret_cast<const float4*>(p->d_H[2]) : nullptr, cc[0], cc[1], cc[2],
            reinterpret_cast<float4*>(cur)));
        float rprev = INFINITY;
        for (int it = 0; it < kSchulzMax; it++) {
            int r = transpose(cur, n, n, n, p->d_Xt, n, cs);
            if (!r) r = copy2d(nullptr, 0, n, n, p->d_R, n, 1.f, cs);
            if (!r) r = gemm(p, n, n, n, W, mp, p->d_Xt, n, p->d_R, n, -1.f, 1.f, cs);
            if (r) return r;
            OCMP_CUDA(cudaMemsetAsync(p->d_rmax, 0, sizeof(unsigned), cs));
            OCMP_LAUNCH(k_infnorm<<<nblk(n, 8), 256, 0, cs>>>(p->d_R, n, n, n, p->d_rmax));
            OCMP_CUDA(cudaMemcpyAsync(p->h_rmax, p->d_rmax, sizeof(unsigned), cudaMemcpyDeviceToHost, cs));
            OCMP_CUDA(cudaStreamSynchronize(cs));
            float rho;
            std::memcpy(&rho, p->h_rmax, sizeof(float));
            if (!std::isfinite(rho) || rho >= rprev) break;
            if (rho <= kSchulzTol) {
                ok = true;
                break;
            }
            rprev = rho;
            r = transpose(p->d_R, n, n, n, p->d_Rt, n, cs);
            if (!r) r = copy2d(cur, n, n, n, nxt, n, 1.f, cs);
            if (!r) r = gemm(p, n, n, n, cur, n, p->d_Rt, n, nxt, n, 1.f, 1.f, cs);
            if (r) return r;
            std::swap(cur, nxt);
            p->ns_iters++;
            if (rho * rho <= kSchulzTol) {
                ok = true;
                if ((r = transpose(cur, n, n, n, p->d_Xt, n, cs))) return r;
                break;
            }
        }
        if (ok) p->ns_strips++;
        else p->ns_fallbacks++;
    }
    if (!ok) {
        int r = copy2d(W, mp, n, n, cur, n, 1.f, cs);
        if (!r) r = gj_tiles(p, cur, n, 0, n, p->work[0], cs);
        if (!r) r = transpose(cur, n, n, n, p->d_Xt, n, cs);
        if (r) return r;
    }
    // the new inverse joins the history, the oldest buffer taking it
    float* h = p->d_H[2];
    p->d_H[2] = p->d_H[1];
    p->d_H[1] = p->d_H[0];
    p->d_H[0] = h;
    p->h_n[2] = p->h_n[1];
    p->h_n[1] = p->h_n[0];
    p->h_n[0] = n;
    OCMP_CUDA(cudaMemcpyAsync(h, cur, sizeof(float) * (size_t)n * n, cudaMemcpyDeviceToDevice, cs));
    *X = cur;
    return OCMP_OK;
}

// Phase 2 of a block-diagonal-N strip after the Schur update: with X_I = W^-1 (W = S_II),
//   G_II = X_I, G_IN = X_I Z, G_NI = -T, G_NN = X - T Z, T = Y X_I.
int phase2_groups(Strip* p, int k, float* S, cudaStream_t cs) {
    const int mp = p->mp[k], nNp = p->nNp[k], n = mp - nNp;
    float* Wi = nullptr;
    int r = invert_interface(p, S + (int64_t)nNp * mp + nNp, mp, n, &Wi, cs);
    if (!r) r = gemm(p, nNp, n, n, S + nNp, mp, p->d_Xt, n, p->d_T1, n, 1.f, 0.f, cs);
    if (!r) r = transpose(S + (int64_t)nNp * mp, mp, n, nNp, p->d_Zt, n, cs);
    if (!r) r = gemm(p, nNp, nNp, n, p->d_T1, n, p->d_Zt, n, S, mp, -1.f, 1.f, cs);
    if (!r) r = gemm(p, n, nNp, n, Wi, n, p->d_Zt, n, S + (int64_t)nNp * mp, mp, 1.f, 0.f, cs);
    if (!r) r = copy2d(p->d_T1, n, nNp, n, S + nNp, mp, -1.f, cs);
    if (!r) r = copy2d(Wi, n, n, n, S + (int64_t)nNp * mp + nNp, mp, 1.f, cs);
    return r;
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
    // uniform strips when the pattern repeats with a period w (a structured mesh numbered row by
    // row of elements): strips of exactly w dofs, each one row, make neighbouring strips' Schur
    // complements alike (the Newton-Schulz start relies on it) where the greedy strips drift
    // against the rows. w: the smallest width from half to twice the greedy one for which the
    // rows of a sample match the rows w further on (same column offsets) and the uniform strips
    // are block tridiagonal.
    if (p->s.size() > 4) {
        std::vector<int64_t> wd;
        for (size_t q = 2; q + 1 < p->s.size(); q++) wd.push_back(p->s[q] - p->s[q - 1]);
        std::nth_element(wd.begin(), wd.begin() + wd.size() / 2, wd.end());
        const int64_t wg = wd[wd.size() / 2];
        auto same = [&](int64_t r, int64_t w) {
            const int64_t r2 = r + w;
            if (rp[r + 1] - rp[r] != rp[r2 + 1] - rp[r2]) return false;
            for (int64_t e = 0; e < rp[r + 1] - rp[r]; e++)
                if ((int64_t)col[rp[r2] + e] - r2 != (int64_t)col[rp[r] + e] - r) return false;
            return true;
        };
        auto valid = [&](int64_t w) {
            for (int64_t r = 0; r < n; r++) {
                const int64_t k = r / w;
                if (mn[r] < (k - 1) * w || mx[r] >= (k + 2) * w) return false;
            }
            return true;
        };
        constexpr int kSample = 64;
        for (int64_t w = std::max<int64_t>(1, wg / 2); w <= 2 * wg && 3 * w <= n; w++) {
            int hits = 0;
            for (int q = 0; q < kSample; q++) {
                const int64_t r = (n - w - 1) * (2 * q + 1) / (2 * kSample);
                hits += same(r, w);
            }
            if (hits * 8 < kSample * 7 || !valid(w)) continue;
            std::vector<int64_t> u;
            for (int64_t b = 0; b < n; b += w) u.push_back(b);
            u.push_back(n);
            p->s.swap(u);
            break;
        }
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
    // strips whose N positions split into independent groups of at most 32 (union-find over the
    // pattern inside the strip, constrained dofs included, so the groups hold for any constraints),
    // packed greedily into warps' worth; the padding of N joins as single positions
    p->fast.assign(K, 0);
    p->gofs.assign(K + 1, 0);
    p->ngrp.assign(K, 0);
    std::vector<int32_t> gptr{0}, gidx, gcomp;
    for (int k = 0; k < K; k++) {
        p->gofs[k] = (int64_t)gptr.size() - 1;
        const int nN = p->nN[k];
        if (nN == 0 || p->nI[k] == 0) continue;
        const int64_t s0 = p->s[k], s1 = p->s[k + 1];
        std::vector<int> par(nN);
        std::iota(par.begin(), par.end(), 0);
        auto find = [&](int a) {
            while (par[a] != a) a = par[a] = par[par[a]];
            return a;
        };
        for (int q = 0; q < nN; q++) {
            const int64_t r = s0 + perm[p->poff[k] + q];
            for (int64_t e = rp[r]; e < rp[r + 1]; e++) {
                const int64_t c = col[e];
                if (c < s0 || c >= s1) continue;
                const int pc = pinv[c];
                if (pc < nN) {
                    const int a = find(q), b = find(pc);
                    if (a != b) par[std::max(a, b)] = std::min(a, b);
                }
            }
        }
        std::vector<std::vector<int32_t>> comp(nN);
        bool small = true;
        for (int q = 0; q < nN && small; q++) {
            auto& c = comp[find(q)];
            c.push_back(q);
            small = c.size() <= 32;
        }
        if (!small) continue;
        for (int q = nN; q < p->nNp[k]; q++) comp.push_back({q});
        const size_t g0 = gptr.size();
        int fill = 0;
        for (const auto& c : comp) {
            if (c.empty()) continue;
            if (fill + (int)c.size() > 32) {
                gptr.push_back((int32_t)gidx.size());
                fill = 0;
            }
            gidx.insert(gidx.end(), c.begin(), c.end());
            for (size_t e = 0; e < c.size(); e++) gcomp.push_back((fill << 8) | (int32_t)c.size());
            fill += (int)c.size();
        }
        gptr.push_back((int32_t)gidx.size());
        p->ngrp[k] = (int)(gptr.size() - g0);
        p->fast[k] = 1;
        p->nfast++;
    }
    p->gofs[K] = (int64_t)gptr.size() - 1;
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
    // coupling lists of the I dofs to the previous strip's J dofs (the Schur update's sparse factors)
    std::vector<int32_t> cptr{0}, cb, crow, ccol;
    for (int k = 0; k < K; k++) {
        const int64_t s0 = p->s[k];
        std::vector<std::vector<std::array<int32_t, 3>>> lists(p->nI[k]);
        if (k > 0) {
            auto entry = [&](int a, int32_t b) -> std::array<int32_t, 3>& {
                for (auto& e : lists[a])
                    if (e[0] == b) return e;
                lists[a].push_back({b, -1, -1});
                return lists[a].back();
            };
            for (int a = 0; a < p->nI[k]; a++) {
                const int64_t r = s0 + Ipos[p->ioff[k] + a];
                for (int64_t q = rp[r]; q < rp[r + 1]; q++)
                    if (col[q] < s0) entry(a, Jinv[col[q]])[1] = (int32_t)q;
            }
            const int64_t sp = p->s[k - 1];
            for (int64_t d = sp; d < s0; d++)
                for (int64_t q = rp[d]; q < rp[d + 1]; q++)
                    if (col[q] >= s0 && col[q] < p->s[k + 1]) entry(Iinv[col[q]], Jinv[d])[2] = (int32_t)q;
        }
        for (auto& l : lists) {
            std::sort(l.begin(), l.end());
            for (auto& e : l) {
                cb.push_back(e[0]);
                crow.push_back(e[1]);
                ccol.push_back(e[2]);
            }
            cptr.push_back((int32_t)cb.size());
            p->cmax = std::max(p->cmax, (int)l.size());
        }
    }
    const int64_t fast_floats = p->nfast ? (int64_t)8 * p->nIp_max * p->nIp_max +
                                                (int64_t)(2 + kSide) * p->mp_max * p->nIp_max
                                          : 0;
    const int64_t need = total * 4 + (int64_t)p->nJp_max * p->nIp_max * 4 +
                         (int64_t)(kSide + 1) * (2 * p->mp_max * kNb + kNb * kNb) * 4 + fast_floats * 4;
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
    p->bytes = total * 4 + (int64_t)(perm.size() + Ipos.size() + Jp.size() + n) * 4;
    auto A = [&](auto** d, size_t cnt) {
        if (!st) st = dalloc(d, cnt);
    };
    A(&p->d_G, (size_t)total);
    U(&p->d_cptr, cptr);
    U(&p->d_cb, cb);
    U(&p->d_crow, crow);
    U(&p->d_ccol, ccol);
    p->bytes += (int64_t)(cptr.size() + 3 * cb.size()) * 4;
    A(&p->d_T, (size_t)std::max(1, p->nJp_max * p->nIp_max));
    for (auto& w : p->work) {
        A(&w.P, (size_t)kNb * kNb);
        A(&w.Ck, (size_t)p->mp_max * kNb);
        A(&w.Rt, (size_t)p->mp_max * kNb);
    }
    A(&p->d_r, (size_t)p->mp_max);
    A(&p->d_flag, 2);
    {
        // ELL coupling lists of the sweeps' right-hand sides
        std::vector<int64_t> eoff(K + 1, 0);
        std::vector<int> elo(K, 0), ehi(K, 0);
        std::vector<int32_t> prow, erow, ecol, epos;
        for (int k = 0; k < K; k++) {
            const int mpk = p->mp[k];
            const int64_t s0 = p->s[k];
            for (int q = 0; q < mpk; q++) {
                const int ld = perm[p->poff[k] + q];
                prow.push_back(ld < 0 ? -1 : (int32_t)(s0 + ld));
                if (ld < 0) continue;
                const int64_t r = s0 + ld;
                elo[k] = std::max(elo[k], lo_ptr[r + 1] - lo_ptr[r]);
                ehi[k] = std::max(ehi[k], hi_ptr[r + 1] - hi_ptr[r]);
            }
            eoff[k] = (int64_t)erow.size();
            for (int part = 0; part < 2; part++) {
                const int L = part == 0 ? elo[k] : ehi[k];
                const std::vector<int32_t>& ptr = part == 0 ? lo_ptr : hi_ptr;
                const std::vector<int32_t>& pos = part == 0 ? lo_pos : hi_pos;
                for (int e = 0; e < L; e++)
                    for (int q = 0; q < mpk; q++) {
                        const int ld = perm[p->poff[k] + q];
                        const int64_t r = ld < 0 ? -1 : s0 + ld;
                        const bool has = ld >= 0 && ptr[r] + e < ptr[r + 1];
                        const int32_t cp = has ? pos[ptr[r] + e] : -1;
                        erow.push_back(ld < 0 ? 0 : (int32_t)r);
                        ecol.push_back(has ? col[cp] : -1);
                        epos.push_back(cp);
                    }
            }
        }
        eoff[K] = (int64_t)erow.size();
        p->eoff = eoff;
        p->elo = elo;
        p->ehi = ehi;
        p->nell = (int64_t)erow.size();
        p->npos = (int64_t)prow.size();
        U(&p->d_prow, prow);
        U(&p->d_erow, erow);
        U(&p->d_ecol, ecol);
        U(&p->d_epos, epos);
        A(&p->d_rdof, prow.size());
        A(&p->d_ev, std::max<size_t>(1, erow.size()));
        p->bytes += (int64_t)(prow.size() * 2 + erow.size() * 4) * 4;
    }
    if (p->nfast) {
        const size_t i2 = (size_t)p->nIp_max * p->nIp_max, mi = (size_t)p->mp_max * p->nIp_max;
        U(&p->d_gptr, gptr);
        U(&p->d_gidx, gidx);
        U(&p->d_gcomp, gcomp);
        A(&p->d_Xa, i2);
        A(&p->d_Xb, i2);
        A(&p->d_R, i2);
        A(&p->d_Rt, i2);
        A(&p->d_Xt, i2);
        for (float*& h : p->d_H) A(&h, i2);
        A(&p->d_T1, mi);
        A(&p->d_Zt, mi);
        for (float*& y : p->d_Yt) A(&y, mi);
        A(&p->d_rmax, 1);
        if (!st && cudaMallocHost((void**)&p->h_rmax, sizeof(unsigned)) != cudaSuccess)
            st = fail(OCMP_ERR_NOMEM, "strip preconditioner: pinned flag");
        p->bytes += (int64_t)(gptr.size() + 2 * gidx.size()) * 4;
    }
    U(&p->jrow, Jpos);
    p->bytes += (int64_t)Jpos.size() * 4;
    // every buffer a kernel of the factorisation or the sweeps dereferences must exist
    if (!st) {
        const void* need_ptr[] = {p->d_perm, p->d_pinv, p->d_G, p->d_cptr, p->d_T, p->d_r, p->d_flag, p->d_prow, p->d_rdof,
                                  p->d_ev, p->work[0].P, p->work[0].Ck, p->work[0].Rt};
        bool ok = std::all_of(std::begin(need_ptr), std::end(need_ptr), [](const void* q) { return q != nullptr; });
        if (p->nfast) {
            const void* fast_ptr[] = {p->d_gptr, p->d_gidx, p->d_gcomp, p->d_Xa, p->d_Xb, p->d_R, p->d_Rt, p->d_Xt,
                                      p->d_H[0], p->d_H[1], p->d_H[2], p->d_T1, p->d_Zt, p->d_Yt[0], p->d_Yt[1],
                                      p->d_Yt[2], p->d_rmax, p->h_rmax};
            ok = ok && std::all_of(std::begin(fast_ptr), std::end(fast_ptr), [](const void* q) { return q != nullptr; });
        }
        if (p->nell) ok = ok && p->d_erow && p->d_ecol && p->d_epos;
        if (!ok) st = fail(OCMP_ERR_NOMEM, "strip preconditioner: a work buffer was not allocated");
    }
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
            cudaFuncSetAttribute(k_panel_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, kFinishSmem) != cudaSuccess ||
            cudaFuncSetAttribute(k_strip_gemv<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * p->mp_max) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_strip_gemv<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * p->mp_max) !=
                cudaSuccess)
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
    p->gemm_bytes_pending = 0;
    p->ns_iters = p->ns_strips = p->ns_fallbacks = 0;
    for (int& h : p->h_n) h = 0;
    OCMP_CUDA(cudaEventRecord(p->fev[0], st));
    OCMP_CUDA(cudaMemsetAsync(p->d_flag, 0, 2 * sizeof(int), st));
    {
        const int64_t nt = std::max(p->nell, p->npos);
        OCMP_LAUNCH(k_ell_refresh<<<nblk(nt, 256), 256, 0, st>>>(p->nell, p->d_erow, p->d_ecol, p->d_epos, vals, s->d_free,
                                                                  p->d_ev, p->npos, p->d_prow, p->d_rdof));
    }
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
        const int r = p->schulz && p->fast[k] ? phase1_groups(p, k, S, q, ss)
                                              : gj_tiles(p, S, mp, 0, p->nNp[k], p->work[1 + q], ss);
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
            const int nI = p->nI[k], nJ = p->nJ[k - 1], nIp = pad(nI);
            const int64_t sp = p->s[k - 1];
            const int32_t* Irow = p->d_I + p->ioff[k];
            const int32_t* Jrow = p->jrow + p->joff[k - 1];
            const int32_t* cp = p->d_cptr + p->ioff[k];
            OCMP_LAUNCH(k_schur_t<<<dim3(nblk(nIp, 128), nblk(nJ, kSchurRows)), 128, 0, cs>>>(
                nI, nJ, nIp, s0, sp, Irow, Jrow, p->d_J + p->joff[k - 1], cp, p->d_cb, p->d_ccol, vals, s->d_free,
                p->d_G + p->goff[k - 1], p->mp[k - 1], p->d_T));
            OCMP_LAUNCH(k_schur_u<<<dim3(nblk(nI, 4 * 128), nI), 128, 0, cs>>>(nI, nIp, p->nNp[k], s0, sp, Irow, Jrow,
                                                                              cp, p->d_cb, p->d_crow, vals, s->d_free,
                                                                              p->d_T, S, mp));
        }
        if (!p->fast[k])
            for (int& h : p->h_n) h = 0;
        const int r = p->schulz && p->fast[k] ? phase2_groups(p, k, S, cs) : gj_tiles(p, S, mp, p->nNp[k], mp, p->work[0], cs);
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
    p->gemm_bytes = p->gemm_bytes_pending;
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
void sweeps(Strip* p, T* z, const int* flags, cudaStream_t st) {
    const int K = p->K;
    for (int pass = 0; pass < 2; pass++) {
        for (int step = 0; step < (pass == 0 ? K : K - 1); step++) {
            const int k = pass == 0 ? step : K - 2 - step;
            const int mp = p->mp[k];
            const int L = pass == 0 ? p->elo[k] : p->ehi[k];
            const int64_t e0 = p->eoff[k] + (pass == 0 ? 0 : (int64_t)p->elo[k] * mp);
            OCMP_LAUNCH(k_strip_rhs<T><<<nblk(mp, 128), 128, 0, st>>>(mp, L, pass == 0, p->d_rdof + p->poff[k],
                                                                     p->d_ecol + e0, p->d_ev + e0, z, p->d_r, flags));
            OCMP_LAUNCH(k_strip_gemv<T><<<nblk(mp, 8), 256, sizeof(float) * mp, st>>>(
                mp, p->s[k], p->d_perm + p->poff[k], p->d_G + p->goff[k], p->d_r, z, pass, flags));
        }
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
        sweeps<T>(p, z, flags, p->cap);
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
    o->gemm_bytes = p->gemm_bytes;
    o->singular_tiles = p->singular;
    o->gemm_kind = p->gemm_kind;
    o->tile_ms = p->part_ms[1];
    o->panel_ms = p->part_ms[2];
    o->fast_strips = p->schulz ? p->nfast : 0;
    o->schulz_strips = p->ns_strips;
    o->schulz_iterations = p->ns_iters;
    o->schulz_fallbacks = p->ns_fallbacks;
}

void strip_set_timing(Strip* p, bool on) { p->timing = on; }
void strip_set_gemm(Strip* p, int kind) { p->gemm_kind = kind; }
void strip_set_schulz(Strip* p, bool on) { p->schulz = on; }

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
