// Krylov solvers of libopencmp_gpu.so (sm_103a): the GPU counterpart of the linear solve in
// opencmp/models/base_model.py:886-947 (solvers.CG with the 'local' = point-Jacobi preconditioner
// restricted to free dofs, solvers.GMRes with freedofs).
//
// The whole iteration stays on the device: Hessenberg matrix, Givens rotations, residual
// estimate and convergence/breakdown flags live in device memory and are updated by one-thread
// kernels; the host only reads the flags every `check_every` iterations. Every reduction is a
// fixed two-stage tree (per-block partials, then one block per value), so results are
// bit-reproducible run to run.
//
// Precision: OCMP_FP64 runs everything in FP64. OCMP_MIXED runs an outer FP64 iterative
// refinement (r = b - A x with the FP64 matrix, x += correction) around an inner GMRES/CG whose
// matrix values, vectors and preconditioner are FP32 and whose dot products are accumulated per
// thread in FP32 and across threads in FP64; the Hessenberg matrix and rotations stay FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <type_traits>

#include "ocmp_internal.h"
#include "ocmp_spmv.cuh"

namespace ocmp {
// Per-instance strides of a batch of independent systems that share one sparsity pattern: the
// instance is blockIdx.y; a single system uses zero strides and gridDim.y = 1.
struct Bat {
    int64_t n, nnz, V, part, st, flags, scale, H, red, cnt;
};
// One instance of a solver group (ocmp_group_*): its system and its slice of its member solver's
// GMRES buffers. The group's kernels stride a fixed grid over a list of (instance, block) pairs
// of the instances still iterating: block k of gbn (reduction kernels) or of sbn (SpMV).
struct GInst {
    int64_t n;
    const int32_t* rp;
    const int32_t* col;
    const uint8_t* freed;
    const int32_t* lift_ptr;
    const int32_t* lift_pos;
    const double* A64;   // FP64 matrix values (residuals)
    const void* K;       // Krylov matrix values (T)
    const void* dinv;    // T: D^-1 of the final update, or null
    void* V;             // T: (m + 1) x n basis
    double* part;
    unsigned* cnt;
    double* st;
    int* flags;
    double* scale;
    double* H;           // Hessenberg, then cos/sin/g
    double* red;
    const double* b;
    double* x;
    int gbn, sbn;
    int cfg;             // SpMV rows: 0 (2, 4), 1 (4, 4), 2 (4, 8), 3 (8, 4), 4 (8, 8), 5 (16, 8) threads per row, loads in flight
};
}  // namespace ocmp

// Cahouet-Chabard block preconditioner of a Taylor-Hood saddle-point system [u | p]
// (OCMP_PRE_CAHOUET_CHABARD): velocity point Jacobi, and on the pressure block
// z_p = -(alpha S^-1 r_p + beta M_p,diag^-1 r_p) / tc^2 with S = L_p + delta M_p solved exactly by the
// strip direct factorisation of the pressure operator.
struct CCPre {
    ocmp::Strip* strip = nullptr;
    ocmp_matrix_s* pop = nullptr;   // the pressure operator S (pressure space)
    int64_t nu = 0, np = 0;         // velocity dofs (all components) and pressure dofs
    double alpha = 1, beta = 0, tc = 1;
    double* vdinv = nullptr;        // nu
    double* mpinv = nullptr;        // np
    double* zp64 = nullptr;         // np: pressure-solve vector
    float* zp32 = nullptr;
};

struct ocmp_solver_s {
    ocmp_matrix_s* mat = nullptr;
    ocmp_space_s* s = nullptr;
    ocmp_solve_params_t prm{};
    int64_t n = 0;
    int nb = 0;                 // reduction blocks
    int m = 0;                  // GMRES restart
    // FP64 path
    double* dinv = nullptr;     // Jacobi (0 on constrained rows)
    double* udiag = nullptr;    // caller's inverse diagonal (OCMP_PRE_USER)
    bool udiag_set = false;
    double* Binv = nullptr;     // block Jacobi (L2 element blocks)
    ocmp::Strip* strip = nullptr;  // strip direct preconditioner (OCMP_PRE_STRIP)
    bool strip_ready = false;       // factorised by ocmp_solver_update since the last failure
    CCPre* cc = nullptr;           // Cahouet-Chabard data (OCMP_PRE_CAHOUET_CHABARD), once set
    double* V = nullptr;        // (m+1) x n
    double* w = nullptr;
    double* z = nullptr;
    double* r = nullptr;
    double* p = nullptr;
    // FP32 inner path (OCMP_MIXED)
    float* dinv32 = nullptr;
    float* Binv32 = nullptr;
    float* V32 = nullptr;
    float* w32 = nullptr;
    float* z32 = nullptr;
    float* r32 = nullptr;
    float* p32 = nullptr;
    float* d32 = nullptr;       // inner correction
    // reductions and small state
    double* part = nullptr;     // (m+4) x nb
    double* pspmv = nullptr;    // one partial per SpMV block (CG p . Ap)
    double* red = nullptr;      // m+2 reduced values
    double* st = nullptr;       // small state, see enum below
    double* H = nullptr;        // (m+1) x m
    int* flags = nullptr;       // device flags
    int* hflags = nullptr;      // pinned host mirror
    // fused GMRES
    double* As64 = nullptr;     // A D^-1 (Jacobi folded) or A, FP64 Krylov matrix (owned)
    float* As32 = nullptr;      // same in FP32 (OCMP_MIXED)
    const double* K64 = nullptr;  // Krylov matrix in use: As64, or the matrix's own scaled values
    const float* K32 = nullptr;
    bool borrow = false;        // Jacobi-scaled values and D^-1 come from the assembly
    double* scale = nullptr;    // basis scales: v_k = scale[k] * V[k]
    unsigned* cnt = nullptr;    // last-block counters (zero between launches)
    int grid = 0;               // persistent grid of the fused kernels
    int B = 1;                  // systems in the batch (matrix instances)
    ocmp::Bat bat{};            // per-instance strides
    bool use_graph = false;     // replay each restart cycle from a captured CUDA graph
    cudaGraphExec_t gexec = nullptr;
    unsigned long long graph_kernels = 0;  // kernel launches captured in gexec
    // optional live timing of the Krylov SpMV launches (ocmp_solver_spmv_timing)
    bool time_spmv = false;
    std::vector<cudaEvent_t> tev;
    size_t tev_used = 0;
    int* worklog = nullptr;     // per timed launch: 1 if it ran (not past convergence), written by the kernel
    int worklog_cap = 0;
    // the FP32 Krylov matrix is the assembly's SELL-32 copy (OCMP_MAT_SELL32, borrowed)
    bool sell = false;
    int last_iters = 0;         // iterations of the last GMRES solve (adaptive host checks)
    int64_t spmv_launches = 0;
    double spmv_ms = 0;
    cudaStream_t gstream = nullptr;   // capture/launch stream when the caller passes the default stream
    cudaEvent_t gev[2] = {nullptr, nullptr};
    const double* g_b = nullptr;
    const double* g_x = nullptr;
    cudaStream_t g_stream = nullptr;
};

// A group of GMRES solvers whose instances (every system of every member, members of different
// sizes and patterns) are solved by one kernel sequence.
struct ocmp_group_s {
    std::vector<ocmp_solver_s*> members;
    std::vector<int> first;          // per member: its first instance
    int ninst = 0, m = 0, maxit = 0;
    bool mixed = false;
    std::vector<ocmp::GInst> h_inst;
    ocmp::GInst* d_inst = nullptr;
    int2* d_glist = nullptr;         // (instance, block) pairs of the active instances: reduction kernels
    int2* d_slist = nullptr;         // the same for the SpMV
    int* d_nact = nullptr;           // [0] pairs in d_glist, [1] in d_slist
    int2* h_glist = nullptr;         // pinned staging of the lists
    int2* h_slist = nullptr;
    int* h_nact = nullptr;
    int gtot = 0, stot = 0;          // pairs of all instances
    int grid[2][6] = {};             // resident grid per kernel and precision: [FP32, FP64][spmv, dots, orth,
                                     // combine, resid, -]
    cudaStream_t gstream = nullptr;  // capture stream
    cudaGraphExec_t gexec = nullptr; // one restart cycle over all instances
    unsigned long long graph_kernels = 0;
};

namespace ocmp {
namespace {

// small-state slots (doubles)
enum { S_BETA = 0, S_NB, S_INV, S_RES, S_HN2, S_NW2, S_ALPHA, S_RZ, S_TOL, S_SCALE, S_G0, S_NSLOT = 16 };
// flags
enum { F_CONV = 0, F_REORTH, F_BREAK, F_NONFIN, F_JDONE, F_ITERS, F_NFLAG = 8 };

constexpr int kThreads = 256;
inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

template <class T>
__device__ __forceinline__ double block_sum(T v) {
    __shared__ double sh[kThreads / 32];
    double d = (double)v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = d;
    __syncthreads();
    double t = 0;
    if (wid == 0) {
        t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    }
    return t;  // valid in thread 0
}

// out[k] = sum_b part[k * nb + b]; one block per k
__global__ void reduce_kernel(int nb, int nk, const double* __restrict__ part, double* __restrict__ out,
                              const int* __restrict__ flags, int gate) {
    if (gate >= 0 && flags[gate] == 0) return;
    const int k = blockIdx.x;
    if (k >= nk) return;
    double acc = 0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += part[(int64_t)k * nb + b];
    double t = block_sum(acc);
    if (threadIdx.x == 0) out[k] = t;
}

// y = free ? A x : 0, optional partial of dot(x, y) (CG: p . A p).
template <class TM, class TV, int TPR>
__global__ void __launch_bounds__(kThreads) spmv_masked(int64_t n, const int32_t* __restrict__ rp,
                                                        const int32_t* __restrict__ col, const TM* __restrict__ val,
                                                        const uint8_t* __restrict__ freed, const TV* __restrict__ x,
                                                        TV* __restrict__ y, double* __restrict__ part,
                                                        const int* __restrict__ flags) {
    if (flags && flags[F_CONV]) return;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t r = t / TPR;
    const int lane = threadIdx.x % TPR;
    TV acc = 0;
    if (r < n) {
        const int32_t a = rp[r], b = rp[r + 1];
        for (int32_t k = a + lane; k < b; k += TPR) acc += (TV)__ldg(val + k) * __ldg(x + __ldg(col + k));
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, TPR);
    TV dv = 0;
    if (r < n && lane == 0) {
        const TV yv = freed[r] ? acc : (TV)0;
        y[r] = yv;
        dv = yv * x[r];
    }
    if (part) {
        double s = block_sum(dv);
        if (threadIdx.x == 0) part[blockIdx.x] = s;
    }
}

// r = free ? b - Ax : 0 ; partial of |r|^2.  Also used with Ax = A x_D to get the rhs norm.
template <class T>
__global__ void resid_kernel(int64_t n, const double* __restrict__ b, const double* __restrict__ Ax,
                             const uint8_t* __restrict__ freed, T* __restrict__ r, double* __restrict__ part,
                             int nparts) {
    double acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = freed[i] ? b[i] - Ax[i] : 0.0;
        if (r) r[i] = (T)v;
        acc += v * v;
    }
    double s = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
    (void)nparts;
}

__global__ void zero_free(int64_t n, const uint8_t* __restrict__ freed, const double* __restrict__ x,
                          double* __restrict__ xd) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        xd[i] = freed[i] ? 0.0 : x[i];
}

template <class T>
__global__ void jacobi_setup(int64_t n, const int32_t* __restrict__ diag, const double* __restrict__ vals,
                             const uint8_t* __restrict__ freed, T* __restrict__ dinv) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = vals[diag[i]];
    dinv[i] = (T)((freed[i] && d != 0.0) ? 1.0 / d : 0.0);
}

// block-Jacobi inverse of each element block (L2 spaces), Gauss-Jordan with partial pivoting, FP64
template <int L>
__global__ void block_jacobi_setup(int64_t ne, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                   const double* __restrict__ vals, double* __restrict__ Binv,
                                   float* __restrict__ Binv32) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double A[L][2 * L];
    for (int i = 0; i < L; i++) {
        const int64_t r = e * L + i;
        const int32_t a = rp[r], b = rp[r + 1];
        for (int j = 0; j < L; j++) {
            A[i][j] = 0;
            A[i][L + j] = (i == j) ? 1.0 : 0.0;
        }
        for (int32_t k = a; k < b; k++) {
            const int32_t c = col[k];
            if (c >= e * L && c < (e + 1) * L) A[i][c - e * L] = vals[k];
        }
    }
    for (int c = 0; c < L; c++) {
        int pr = c;
        for (int i = c + 1; i < L; i++)
            if (fabs(A[i][c]) > fabs(A[pr][c])) pr = i;
        if (pr != c)
            for (int j = 0; j < 2 * L; j++) {
                double t = A[c][j];
                A[c][j] = A[pr][j];
                A[pr][j] = t;
            }
        const double d = A[c][c];
        const double id = d != 0.0 ? 1.0 / d : 0.0;
        for (int j = 0; j < 2 * L; j++) A[c][j] *= id;
        for (int i = 0; i < L; i++)
            if (i != c) {
                const double mm = A[i][c];
                for (int j = 0; j < 2 * L; j++) A[i][j] -= mm * A[c][j];
            }
    }
    for (int i = 0; i < L; i++)
        for (int j = 0; j < L; j++) {
            Binv[(e * L + i) * L + j] = A[i][L + j];
            if (Binv32) Binv32[(e * L + i) * L + j] = (float)A[i][L + j];
        }
}

template <class T, int L>
__global__ void block_prec(int64_t ne, const T* __restrict__ Binv, const T* __restrict__ v, T* __restrict__ z,
                           const int* __restrict__ flags) {
    if (flags && flags[F_CONV]) return;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= ne * L) return;
    const int64_t e = t / L;
    const int i = (int)(t % L);
    T acc = 0;
#pragma unroll
    for (int j = 0; j < L; j++) acc += Binv[(e * L + i) * L + j] * v[e * L + j];
    z[t] = acc;
}

// ---- CG pieces
template <class T>
__global__ void cg_update(int64_t n, const double* __restrict__ st, T* __restrict__ x, T* __restrict__ r,
                          const T* __restrict__ p, const T* __restrict__ q, const T* __restrict__ dinv,
                          T* __restrict__ z, double* __restrict__ part, int nb, const int* __restrict__ flags) {
    if (flags[F_CONV]) return;
    const T alpha = (T)st[S_ALPHA];
    T rz = 0, rr = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const T ri = r[i] - alpha * q[i];
        r[i] = ri;
        const T zi = dinv[i] * ri;
        z[i] = zi;
        rz += ri * zi;
        rr += ri * ri;
    }
    double s1 = block_sum(rz);
    if (threadIdx.x == 0) part[blockIdx.x] = s1;
    double s2 = block_sum(rr);
    if (threadIdx.x == 0) part[nb + blockIdx.x] = s2;
}

template <class T>
__global__ void cg_pupdate(int64_t n, const double* __restrict__ st, const T* __restrict__ z, T* __restrict__ p,
                           const int* __restrict__ flags) {
    if (flags[F_CONV]) return;
    const T beta = (T)st[S_SCALE];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

template <class T>
__global__ void cg_init(int64_t n, const T* __restrict__ r, const T* __restrict__ dinv, T* __restrict__ z,
                        T* __restrict__ p, double* __restrict__ part, int nb) {
    T rz = 0, rr = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const T zi = dinv[i] * r[i];
        z[i] = zi;
        p[i] = zi;
        rz += r[i] * zi;
        rr += r[i] * r[i];
    }
    double s1 = block_sum(rz);
    if (threadIdx.x == 0) part[blockIdx.x] = s1;
    double s2 = block_sum(rr);
    if (threadIdx.x == 0) part[nb + blockIdx.x] = s2;
}

__global__ void cg_scalars_init(const double* __restrict__ red, double* st, int* flags) {
    st[S_RZ] = red[0];
    const double res = sqrt(fmax(red[1], 0.0)) / st[S_NB];
    st[S_RES] = res;
    flags[F_CONV] = res <= st[S_TOL] ? 1 : 0;
    if (!isfinite(res)) {
        flags[F_NONFIN] = 1;
        flags[F_CONV] = 1;
    }
}
__global__ void cg_alpha(const double* __restrict__ red, double* st, int* flags) {
    if (flags[F_CONV]) return;
    const double pq = red[0];
    if (pq == 0.0 || !isfinite(pq)) {
        flags[pq == 0.0 ? F_BREAK : F_NONFIN] = 1;
        flags[F_CONV] = 1;
        st[S_ALPHA] = 0;
        return;
    }
    st[S_ALPHA] = st[S_RZ] / pq;
}
__global__ void cg_beta(const double* __restrict__ red, double* st, int* flags) {
    if (flags[F_CONV]) return;
    const double rz1 = red[0];
    st[S_SCALE] = st[S_RZ] != 0.0 ? rz1 / st[S_RZ] : 0.0;
    st[S_RZ] = rz1;
    const double res = sqrt(fmax(red[1], 0.0)) / st[S_NB];
    st[S_RES] = res;
    flags[F_ITERS] += 1;
    if (!isfinite(res)) {
        flags[F_NONFIN] = 1;
        flags[F_CONV] = 1;
    } else if (res <= st[S_TOL])
        flags[F_CONV] = 1;
}

__global__ void set_state(double* st, int slot, double v) { st[slot] = v; }
__global__ void set_nb_from(const double* __restrict__ red, double* st) {
    const double nb = sqrt(fmax(red[0], 0.0));
    st[S_NB] = nb > 0 ? nb : 1.0;
}
__global__ void scale_to_float(int64_t n, const double* __restrict__ r, const double* __restrict__ st,
                               float* __restrict__ r32) {
    const double inv = st[S_BETA] > 0 ? 1.0 / st[S_BETA] : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r32[i] = (float)(r[i] * inv);
}
__global__ void add_scaled_float(int64_t n, const float* __restrict__ d, const double* __restrict__ st,
                                 double* __restrict__ x) {
    const double s = st[S_BETA];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += s * (double)d[i];
}

// ------------------------------------------------------------------ host-side drivers
struct Ctx {
    ocmp_solver_s* sv;
    cudaStream_t st;
    int tpr;
    int grid;  // grid-stride vector kernels
};

int pick_tpr(const ocmp_space_s* s) {
    const double avg = (double)s->nnz / (double)s->ndof;
    if (avg <= 6) return 2;
    if (avg <= 14) return 4;
    if (avg <= 40) return 8;
    return 16;
}

template <class TM, class TV>
void launch_spmv_masked(const Ctx& c, const TM* vals, const TV* x, TV* y, double* part, const int* flags) {
    const ocmp_space_s* s = c.sv->s;
    const int64_t n = s->ndof;
    switch (c.tpr) {
    case 2: OCMP_LAUNCH(spmv_masked<TM, TV, 2><<<nblk(n * 2, kThreads), kThreads, 0, c.st>>>(n, s->d_rowptr, s->d_col, vals, s->d_free, x, y, part, flags)); break;
    case 4: OCMP_LAUNCH(spmv_masked<TM, TV, 4><<<nblk(n * 4, kThreads), kThreads, 0, c.st>>>(n, s->d_rowptr, s->d_col, vals, s->d_free, x, y, part, flags)); break;
    case 8: OCMP_LAUNCH(spmv_masked<TM, TV, 8><<<nblk(n * 8, kThreads), kThreads, 0, c.st>>>(n, s->d_rowptr, s->d_col, vals, s->d_free, x, y, part, flags)); break;
    default: OCMP_LAUNCH(spmv_masked<TM, TV, 16><<<nblk(n * 16, kThreads), kThreads, 0, c.st>>>(n, s->d_rowptr, s->d_col, vals, s->d_free, x, y, part, flags)); break;
    }
}
inline int spmv_blocks(const Ctx& c) { return (int)nblk(c.sv->s->ndof * c.tpr, kThreads); }

template <class T>
void launch_block_prec(const Ctx& c, const T* Binv, const T* v, T* z, const int* flags) {
    const ocmp_space_s* s = c.sv->s;
    const int64_t ne = s->mesh->ne;
    switch (s->nloc) {
    case 3: OCMP_LAUNCH(block_prec<T, 3><<<nblk(ne * 3, kThreads), kThreads, 0, c.st>>>(ne, Binv, v, z, flags)); break;
    case 6: OCMP_LAUNCH(block_prec<T, 6><<<nblk(ne * 6, kThreads), kThreads, 0, c.st>>>(ne, Binv, v, z, flags)); break;
    case 10: OCMP_LAUNCH(block_prec<T, 10><<<nblk(ne * 10, kThreads), kThreads, 0, c.st>>>(ne, Binv, v, z, flags)); break;
    default: break;
    }
}

// ||(b - A x_D)_free||: the norm the relative residual is measured against
int rhs_norm(const Ctx& c, const double* b, const double* x) {
    ocmp_solver_s* sv = c.sv;
    const int64_t n = sv->n;
    OCMP_LAUNCH(zero_free<<<c.grid, kThreads, 0, c.st>>>(n, sv->s->d_free, x, sv->z));
    launch_spmv64(sv->s, sv->mat->vals, sv->z, sv->w, c.st);
    OCMP_LAUNCH(resid_kernel<double><<<sv->nb, kThreads, 0, c.st>>>(n, b, sv->w, sv->s->d_free, (double*)nullptr, sv->part, sv->nb));
    OCMP_LAUNCH(reduce_kernel<<<1, kThreads, 0, c.st>>>(sv->nb, 1, sv->part, sv->red, nullptr, -1));
    OCMP_LAUNCH(set_nb_from<<<1, 1, 0, c.st>>>(sv->red, sv->st));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

// FP64 residual r = (b - A x)_free into dst (double or float-scaled), |r|^2 into red[0]
int residual64(const Ctx& c, const double* b, const double* x, double* dst) {
    ocmp_solver_s* sv = c.sv;
    launch_spmv64(sv->s, sv->mat->vals, x, sv->w, c.st);
    OCMP_LAUNCH(resid_kernel<double><<<sv->nb, kThreads, 0, c.st>>>(sv->n, b, sv->w, sv->s->d_free, dst, sv->part, sv->nb));
    OCMP_LAUNCH(reduce_kernel<<<1, kThreads, 0, c.st>>>(sv->nb, 1, sv->part, sv->red, nullptr, -1));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int read_flags(const Ctx& c) {
    OCMP_CUDA(cudaMemcpyAsync(c.sv->hflags, c.sv->flags, sizeof(int) * F_NFLAG * c.sv->B, cudaMemcpyDeviceToHost,
                              c.st));
    OCMP_CUDA(cudaStreamSynchronize(c.st));
    return OCMP_OK;
}

// GMRES lives in the fused section below (gm_*).

template <class T, class TM, class TX>
int cg_core(const Ctx& c, const TM* vals, const T* dinv, T* r, T* z, T* p, T* q, TX* x, int maxit, double tol,
            int* iters_out) {
    ocmp_solver_s* sv = c.sv;
    const int64_t n = sv->n;
    OCMP_LAUNCH(set_state<<<1, 1, 0, c.st>>>(sv->st, S_TOL, tol));
    OCMP_CUDA(cudaMemsetAsync(sv->flags, 0, sizeof(int) * F_NFLAG, c.st));
    OCMP_LAUNCH(cg_init<T><<<sv->nb, kThreads, 0, c.st>>>(n, r, dinv, z, p, sv->part, sv->nb));
    OCMP_LAUNCH(reduce_kernel<<<2, kThreads, 0, c.st>>>(sv->nb, 2, sv->part, sv->red, nullptr, -1));
    OCMP_LAUNCH(cg_scalars_init<<<1, 1, 0, c.st>>>(sv->red, sv->st, sv->flags));
    int it = 0;
    if (read_flags(c)) return OCMP_ERR_CUDA;
    if (!sv->hflags[F_CONV]) {
        const int nbs = spmv_blocks(c);
        while (it < maxit) {
            launch_spmv_masked<TM, T>(c, vals, p, q, sv->pspmv, sv->flags);
            OCMP_LAUNCH(reduce_kernel<<<1, kThreads, 0, c.st>>>(nbs, 1, sv->pspmv, sv->red, nullptr, -1));
            OCMP_LAUNCH(cg_alpha<<<1, 1, 0, c.st>>>(sv->red, sv->st, sv->flags));
            OCMP_LAUNCH(cg_update<T><<<sv->nb, kThreads, 0, c.st>>>(n, sv->st, x, r, p, q, dinv, z, sv->part, sv->nb, sv->flags));
            OCMP_LAUNCH(reduce_kernel<<<2, kThreads, 0, c.st>>>(sv->nb, 2, sv->part, sv->red, sv->flags, -1));
            OCMP_LAUNCH(cg_beta<<<1, 1, 0, c.st>>>(sv->red, sv->st, sv->flags));
            OCMP_LAUNCH(cg_pupdate<T><<<c.grid, kThreads, 0, c.st>>>(n, sv->st, z, p, sv->flags));
            it++;
            if ((it % std::max(1, sv->prm.check_every)) == 0 || it >= maxit) {
                if (read_flags(c)) return OCMP_ERR_CUDA;
                if (sv->hflags[F_CONV]) break;
            }
        }
    }
    OCMP_CUDA(cudaGetLastError());
    if (read_flags(c)) return OCMP_ERR_CUDA;
    *iters_out = sv->hflags[F_ITERS];
    return OCMP_OK;
}

// =============================================================================================
// Fused GMRES(m), right-preconditioned.
//
// The Krylov matrix is A D^-1 (point Jacobi folded into the values by gm_scale_matrix, refreshed
// by ocmp_solver_update) or A itself with an explicit block-Jacobi application. The basis is kept
// unnormalised: v_k = scale[k] * V[k], so no pass is spent normalising. One iteration is
//   gm_spmv       : w = A_s v_j, written into V[j+1] (the row-blocked CSR SpMV);
//   gm_dots       : all dot products V_k . w (k <= j) and |w|^2 in one pass over the basis;
//   gm_orth       : w -= sum_k h_k v_k, |w|^2, then Hessenberg column, Givens rotation, residual
//                   estimate, convergence and breakdown flags, scale[j+1] = 1/|w|;
//   gm_dots / gm_orth pass 2 : a second classical Gram-Schmidt pass, launched always and skipped
//                   on the device unless the first pass cancelled nearly all of |w|.
// Reductions end in the last block to finish (a counter taken with atomicAdd after the block's
// partials are written): that block sums the per-block partials in block order, so every result
// is deterministic. Cycle start, refinement residual and final residual are one FP64 kernel
// (gm_resid). FP64 restarts and the mixed-precision refinement share the same host loop.
// =============================================================================================
constexpr int kGridCap = 1216;  // 152 SMs x 8 resident blocks of 256 threads
constexpr double kTargetMargin = 0.9;  // a GMRES cycle stops at kTargetMargin x the outer tolerance

enum { S_TARGET = 11, S_INNER = 12, S_OUTERTOL = 13, S_ETA2 = 14 };
enum { F_OUTER = 6 };

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// true in every thread of the block that finishes last of nblocks; resets the counter for the next
// launch
__device__ __forceinline__ bool finish_last(unsigned* cnt, unsigned nblocks) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(cnt, 1u) == nblocks - 1;
    __syncthreads();
    if (last) {
        __threadfence();
        if (threadIdx.x == 0) *cnt = 0;
    }
    return last;
}

// out[k] = sum over blocks of part[k * nbp + b], k < nk, by the finishing block, warp per k
__device__ __forceinline__ void finish_sums(const double* __restrict__ part, int nbp, int nblocks, int nk,
                                            double* __restrict__ out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int k = warp; k < nk; k += nw) {
        double s = 0;
        for (int b = lane; b < nblocks; b += 32) s += __ldcg(part + (int64_t)k * nbp + b);
        s = warp_sum(s);
        if (lane == 0) out[k] = s;
    }
    __syncthreads();
}

// One Givens step on Hessenberg column j (thread 0 of the finishing block).
__device__ void givens_step(int m, int j, double hn, double* __restrict__ H, double* __restrict__ csg,
                            double* __restrict__ st, int* __restrict__ flags, double* __restrict__ scale) {
    double* cs = csg;
    double* sn = csg + m;
    double* g = csg + 2 * m;
    H[(j + 1) * m + j] = hn;
    for (int k = 0; k < j; k++) {
        const double a = H[k * m + j], b = H[(k + 1) * m + j];
        H[k * m + j] = cs[k] * a + sn[k] * b;
        H[(k + 1) * m + j] = -sn[k] * a + cs[k] * b;
    }
    const double a = H[j * m + j], b = H[(j + 1) * m + j];
    const double d = sqrt(a * a + b * b);
    flags[F_ITERS] += 1;
    if (!isfinite(d) || !isfinite(hn)) {
        flags[F_NONFIN] = 1;
        flags[F_CONV] = 1;
        return;  // column j is dropped (F_JDONE stays j)
    }
    if (d == 0.0) {
        flags[F_BREAK] = 1;
        flags[F_CONV] = 1;
        return;
    }
    cs[j] = a / d;
    sn[j] = b / d;
    H[j * m + j] = d;
    H[(j + 1) * m + j] = 0;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    flags[F_JDONE] = j + 1;
    st[S_RES] = fabs(g[j + 1]) / st[S_NB];
    scale[j + 1] = hn > 0 ? 1.0 / hn : 0.0;
    if (fabs(g[j + 1]) <= st[S_TARGET] || hn == 0.0 || j + 1 >= m) flags[F_CONV] = 1;
}

// Cycle start / residual: r = (b - A x)_free with the FP64 matrix; V0 = r (stored in T);
// mode 0: |(b - A x_D)_free| -> S_NB (x_D = x with free entries zeroed, V0 untouched)
// mode 1: start a cycle (outer convergence test, g = beta e1, scale[0] = 1/beta, target)
// mode 2: measure only (S_RES)
// mode 3: mode 0 and mode 1 in the same pass (the first cycle of a solve); the lift A_fD x_D is
//         summed over the precomputed lift list only
// (the kernel bodies below take the block's index bx within its instance and the instance's block
// count gx in place of blockIdx.x / gridDim.x: the batched kernels pass those, the group kernels
// an instance's share of a grid over several instances)
template <class T, int TPR, int U>
__device__ __forceinline__ void gm_resid_body(int bx, int gx, int64_t n, const int32_t* __restrict__ rp,
                                              const int32_t* __restrict__ col, const double* __restrict__ A,
                                              const uint8_t* __restrict__ freed, const double* __restrict__ b,
                                              const double* __restrict__ x, T* __restrict__ V0,
                                              double* __restrict__ part, unsigned* __restrict__ cnt, double* st,
                                              int* flags, double* scale, double* csg, int m, int mode,
                                              const int32_t* __restrict__ lift_ptr,
                                              const int32_t* __restrict__ lift_pos) {
    if (mode == 1 && flags[F_OUTER]) return;  // this instance has converged

    constexpr int RT = 256 / TPR;
    const int lane = threadIdx.x % TPR;
    double acc = 0, accd = 0;
    for (int64_t t0 = (int64_t)bx * RT; t0 < n; t0 += (int64_t)gx * RT) {
        const int64_t r = t0 + threadIdx.x / TPR;
        int32_t a = 0, e = 0;
        if (r < n) {
            a = __ldg(rp + r);
            e = __ldg(rp + r + 1);
        }
        double ax;
        if (mode == 0) {
            // A x_D: gather only constrained entries
            ax = 0;
            for (int32_t k = a + lane; k < e; k += TPR) {
                const int32_t c = __ldg(col + k);
                if (!freed[c]) ax += __ldg(A + k) * __ldg(x + c);
            }
#pragma unroll
            for (int o = TPR / 2; o > 0; o >>= 1) ax += __shfl_xor_sync(0xffffffffu, ax, o, TPR);
        } else {
            ax = row_dot<double, double, TPR, U>(a, e, col, A, x, lane);
        }
        if (r < n && lane == 0) {
            const double v = freed[r] ? b[r] - ax : 0.0;
            if (mode == 1 || mode == 3) V0[r] = (T)v;
            acc += v * v;
            if (mode == 3 && freed[r]) {
                double lift = 0;
                for (int32_t q = lift_ptr[r]; q < lift_ptr[r + 1]; q++) {
                    const int32_t k = lift_pos[q];
                    lift += A[k] * x[col[k]];
                }
                const double vd = b[r] - lift;
                accd += vd * vd;
            }
        }
    }
    __shared__ double sh[8], shd[8];
    {
        const double s1 = warp_sum(acc), s2 = warp_sum(accd);
        if ((threadIdx.x & 31) == 0) {
            sh[threadIdx.x >> 5] = s1;
            shd[threadIdx.x >> 5] = s2;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0, td = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            t += sh[w];
            td += shd[w];
        }
        part[bx] = t;
        part[gx + bx] = td;
    }
    if (!finish_last(cnt, gx)) return;
    __shared__ double tot, totd;
    if (threadIdx.x < 32) {
        double q = 0, qd = 0;
        for (int bb = threadIdx.x; bb < gx; bb += 32) {
            q += __ldcg(part + bb);
            qd += __ldcg(part + gx + bb);
        }
        q = warp_sum(q);
        qd = warp_sum(qd);
        if (threadIdx.x == 0) {
            tot = q;
            totd = qd;
        }
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double beta = isfinite(tot) ? sqrt(fmax(tot, 0.0)) : (double)NAN;
    if (mode == 0) {
        st[S_NB] = beta > 0 ? beta : 1.0;
        return;
    }
    if (mode == 3) {
        const double nb = isfinite(totd) ? sqrt(fmax(totd, 0.0)) : (double)NAN;
        st[S_NB] = (nb > 0 || !isfinite(nb)) ? nb : 1.0;
    }
    const double res = beta / st[S_NB];
    st[S_RES] = res;
    st[S_BETA] = beta;
    if (mode == 2) return;
    flags[F_JDONE] = 0;
    flags[F_REORTH] = 0;
    if (!isfinite(beta)) {
        flags[F_NONFIN] = 1;
        flags[F_CONV] = 1;
        flags[F_OUTER] = 1;
        return;
    }
    if (res <= st[S_OUTERTOL]) {
        flags[F_OUTER] = 1;
        flags[F_CONV] = 1;
        return;
    }
    flags[F_CONV] = 0;
    double* g = csg + 2 * m;
    for (int k = 0; k <= m; k++) g[k] = 0;
    g[0] = beta;
    scale[0] = beta > 0 ? 1.0 / beta : 0.0;
    // stop the cycle at the outer tolerance (with a 0.9 margin: the cycle's residual estimate is
    // accurate to far below it, and the FP64 residual of the result is checked after the cycle), or
    // at the inner reduction for mixed precision
    st[S_TARGET] = fmax(kTargetMargin * st[S_OUTERTOL] * st[S_NB], st[S_INNER] * beta);
}

template <class T, int TPR, int U>
__global__ void __launch_bounds__(256) gm_resid(int64_t n, const int32_t* __restrict__ rp,
                                                const int32_t* __restrict__ col, const double* __restrict__ A,
                                                const uint8_t* __restrict__ freed, const double* __restrict__ b,
                                                const double* __restrict__ x, T* __restrict__ V0,
                                                double* __restrict__ part, unsigned* __restrict__ cnt, double* st,
                                                int* flags, double* scale, double* csg, int m, int mode,
                                                const int32_t* __restrict__ lift_ptr,
                                                const int32_t* __restrict__ lift_pos, Bat bt) {
    const int64_t ib = blockIdx.y;
    gm_resid_body<T, TPR, U>(blockIdx.x, gridDim.x, n, rp, col, A + ib * bt.nnz, freed, b + ib * bt.n, x + ib * bt.n,
                             V0 ? V0 + ib * bt.V : nullptr, part + ib * bt.part, cnt + ib * bt.cnt, st + ib * bt.st,
                             flags + ib * bt.flags, scale + ib * bt.scale, csg + ib * bt.H, m, mode, lift_ptr, lift_pos);
}

// d_k = V_k . w for k <= j, and |w|^2 as d_{j+1} when with_norm; w = V[j+1]. The second
// Gram-Schmidt pass (gated = 1) runs only when F_REORTH is set.
template <class T>
__device__ __forceinline__ void gm_dots_body(int bx, int gx, int64_t n, int j, const T* __restrict__ V,
                                             double* __restrict__ part, int nbp, unsigned* __restrict__ cnt,
                                             double* __restrict__ red, const int* __restrict__ flags, int gated,
                                             int with_norm) {
    if (flags[F_CONV] || (gated && !flags[F_REORTH])) return;
    const T* __restrict__ w = V + (int64_t)(j + 1) * n;
    const int warp = threadIdx.x >> 5, lane32 = threadIdx.x & 31;
    const int nk = j + 1 + (with_norm ? 1 : 0);
    // a block sweeps a contiguous slab of rows; warp w owns k = w, w + 8, ...
    const int64_t slab = ((n + gx - 1) / gx + 31) / 32 * 32;
    const int64_t i0 = (int64_t)bx * slab, i1 = min(n, i0 + slab);
    for (int k = warp; k < nk; k += 8) {
        const T* __restrict__ vk = k <= j ? V + (int64_t)k * n : w;
        T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        int64_t i = i0 + lane32;
        for (; i + 96 < i1; i += 128) {
            s0 += vk[i] * w[i];
            s1 += vk[i + 32] * w[i + 32];
            s2 += vk[i + 64] * w[i + 64];
            s3 += vk[i + 96] * w[i + 96];
        }
        for (; i < i1; i += 32) s0 += vk[i] * w[i];
        const double sm = warp_sum((double)s0 + (double)s1 + (double)s2 + (double)s3);
        if (lane32 == 0) part[(int64_t)k * nbp + bx] = sm;
    }
    if (!finish_last(cnt, gx)) return;
    finish_sums(part, nbp, gx, nk, red);
}

template <class T>
__global__ void __launch_bounds__(256) gm_dots(int64_t n, int j, const T* __restrict__ V, double* __restrict__ part,
                                               int nbp, unsigned* __restrict__ cnt, double* __restrict__ red,
                                               const int* __restrict__ flags, int gated, int with_norm, Bat bt) {
    const int64_t ib = blockIdx.y;
    gm_dots_body<T>(blockIdx.x, gridDim.x, n, j, V + ib * bt.V, part + ib * bt.part, nbp, cnt + ib * bt.cnt,
                    red + ib * bt.red, flags + ib * bt.flags, gated, with_norm);
}

// plain masked SpMV of the Krylov matrix into the next basis slot: V[j+1] = sc * (A_s x_in)_free
template <class T, int TPR, int U>
__device__ __forceinline__ void gm_spmv_body(int bx, int64_t n, int j, const int32_t* __restrict__ rp,
                                             const int32_t* __restrict__ col, const T* __restrict__ A,
                                             const uint8_t* __restrict__ freed, const T* __restrict__ xin,
                                             int xin_is_basis, T* __restrict__ V, const double* __restrict__ scale) {
    const int64_t r = (bx * (int64_t)blockDim.x + threadIdx.x) / TPR;
    const int lane = threadIdx.x % TPR;
    int32_t a = 0, e = 0;
    if (r < n) {
        a = __ldg(rp + r);
        e = __ldg(rp + r + 1);
    }
    const T y = row_dot<T, T, TPR, U>(a, e, col, A, xin, lane);
    if (r < n && lane == 0) {
        const T sc = xin_is_basis ? (T)scale[j] : (T)1;
        V[(int64_t)(j + 1) * n + r] = freed[r] ? y * sc : (T)0;
    }
}

template <class T, int TPR, int U>
__global__ void __launch_bounds__(256) gm_spmv(int64_t n, int j, const int32_t* __restrict__ rp,
                                               const int32_t* __restrict__ col, const T* __restrict__ A,
                                               const uint8_t* __restrict__ freed, const T* __restrict__ xin,
                                               int xin_is_basis, T* __restrict__ V, const double* __restrict__ scale,
                                               const int* __restrict__ flags, Bat bt, int* __restrict__ worked) {
    const int64_t ib = blockIdx.y;
    const bool done = flags[ib * bt.flags + F_CONV] != 0;
    // timed launches log whether they did the product or returned at once past convergence
    if (worked && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *worked = done ? 0 : 1;
    if (done) return;
    gm_spmv_body<T, TPR, U>(blockIdx.x, n, j, rp, col, A + ib * bt.nnz, freed, xin + ib * (xin_is_basis ? bt.V : bt.n),
                            xin_is_basis, V + ib * bt.V, scale + ib * bt.scale);
}

// The same product from the SELL-32 copy: a warp per slice of 32 rows, a lane per row, 16-byte loads
// of column indices and values, two chunks (8 entries) in flight before their gathers. The grid is
// a fixed number of waves that stride over the slices, so that a launch queued past convergence
// retires at once.
__global__ void __launch_bounds__(256) gm_spmv_sell(int64_t n, int64_t nslices, int j, const int32_t* __restrict__ off,
                                                    const int32_t* __restrict__ scol, const float* __restrict__ sval,
                                                    const uint8_t* __restrict__ freed, const float* __restrict__ xin,
                                                    int xin_is_basis, float* __restrict__ V,
                                                    const double* __restrict__ scale, const int* __restrict__ flags,
                                                    int* __restrict__ worked) {
    const bool done = flags[F_CONV] != 0;
    if (worked && blockIdx.x == 0 && threadIdx.x == 0) *worked = done ? 0 : 1;
    if (done) return;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float sc = xin_is_basis ? (float)scale[j] : 1.f;
    for (int64_t sl = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; sl < nslices; sl += nw) {
        const int32_t o0 = off[sl], w = (off[sl + 1] - o0) >> 7;   // chunks of 4 entries per row
        const int4* C = reinterpret_cast<const int4*>(scol + o0) + lane;
        const float4* A = reinterpret_cast<const float4*>(sval + o0) + lane;
        float acc0 = 0.f, acc1 = 0.f;
        int c = 0;
        for (; c + 1 < w; c += 2) {
            const int4 c0 = __ldg(C + c * 32), c1 = __ldg(C + (c + 1) * 32);
            const float4 a0 = __ldg(A + c * 32), a1 = __ldg(A + (c + 1) * 32);
            acc0 = fmaf(a0.x, __ldg(xin + c0.x), acc0);
            acc1 = fmaf(a1.x, __ldg(xin + c1.x), acc1);
            acc0 = fmaf(a0.y, __ldg(xin + c0.y), acc0);
            acc1 = fmaf(a1.y, __ldg(xin + c1.y), acc1);
            acc0 = fmaf(a0.z, __ldg(xin + c0.z), acc0);
            acc1 = fmaf(a1.z, __ldg(xin + c1.z), acc1);
            acc0 = fmaf(a0.w, __ldg(xin + c0.w), acc0);
            acc1 = fmaf(a1.w, __ldg(xin + c1.w), acc1);
        }
        if (c < w) {
            const int4 c0 = __ldg(C + c * 32);
            const float4 a0 = __ldg(A + c * 32);
            acc0 = fmaf(a0.x, __ldg(xin + c0.x), acc0);
            acc0 = fmaf(a0.y, __ldg(xin + c0.y), acc0);
            acc0 = fmaf(a0.z, __ldg(xin + c0.z), acc0);
            acc0 = fmaf(a0.w, __ldg(xin + c0.w), acc0);
        }
        const int64_t r = sl * 32 + lane;
        if (r < n) V[(int64_t)(j + 1) * n + r] = freed[r] ? (acc0 + acc1) * sc : 0.f;
    }
}

// w -= sum_k h_k v_k; |w|^2; then (finishing block) Hessenberg column + Givens, or the request for
// a second pass. pass 1 reads h from red (d_k = V_k . w, |w|^2 in red[j+1]); pass 2 from red2.
template <class T>
__device__ __forceinline__ void gm_orth_body(int bx, int gx, int64_t n, int j, int m, T* __restrict__ V,
                                             const double* __restrict__ red, double* __restrict__ part,
                                             unsigned* __restrict__ cnt, double* __restrict__ H,
                                             double* __restrict__ csg, double* st, int* flags, double* scale,
                                             int pass) {
    if (flags[F_CONV] || (pass == 2 && !flags[F_REORTH])) return;
    __shared__ T coef[130];
    for (int k = threadIdx.x; k <= j; k += blockDim.x) coef[k] = (T)(red[k] * scale[k] * scale[k]);
    __syncthreads();
    T* __restrict__ w = V + (int64_t)(j + 1) * n;
    double acc = 0;
    for (int64_t i = bx * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gx * blockDim.x) {
        T wi = w[i];
        for (int k = 0; k <= j; k++) wi -= coef[k] * V[(int64_t)k * n + i];
        w[i] = wi;
        acc += (double)(wi * wi);
    }
    double s = warp_sum(acc);
    __shared__ double sh[8];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q];
        part[bx] = t;
    }
    if (!finish_last(cnt, gx)) return;
    __shared__ double hn2;
    if (threadIdx.x < 32) {
        double q = 0;
        for (int b = threadIdx.x; b < gx; b += 32) q += __ldcg(part + b);
        q = warp_sum(q);
        if (threadIdx.x == 0) hn2 = q;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int k = 0; k <= j; k++) {
        const double h = red[k] * scale[k];
        H[k * m + j] = pass == 1 ? h : H[k * m + j] + h;
    }
    if (pass == 1) {
        st[S_NW2] = red[j + 1];
        if (hn2 < st[S_ETA2] * red[j + 1]) {  // cancellation beyond the threshold: orthogonalise again
            flags[F_REORTH] = 1;
            return;
        }
    }
    flags[F_REORTH] = 0;
    givens_step(m, j, isfinite(hn2) ? sqrt(fmax(hn2, 0.0)) : (double)NAN, H, csg, st, flags, scale);
}

template <class T>
__global__ void __launch_bounds__(256) gm_orth(int64_t n, int j, int m, T* __restrict__ V,
                                               const double* __restrict__ red, double* __restrict__ part,
                                               unsigned* __restrict__ cnt, double* __restrict__ H,
                                               double* __restrict__ csg, double* st, int* flags, double* scale,
                                               int pass, Bat bt) {
    const int64_t ib = blockIdx.y;
    gm_orth_body<T>(blockIdx.x, gridDim.x, n, j, m, V + ib * bt.V, red + ib * bt.red, part + ib * bt.part,
                    cnt + ib * bt.cnt, H + ib * bt.H, csg + ib * bt.H, st + ib * bt.st, flags + ib * bt.flags,
                    scale + ib * bt.scale, pass);
}

// x += P (sum_k y_k v_k) with y = H^-1 g over the completed columns (each block solves the small
// triangular system itself). P = D^-1 (dinv != null), identity, or (u != null) the sum is written
// to u for a block-Jacobi application by the caller.
template <class T>
__device__ __forceinline__ void gm_combine_body(int bx, int gx, int64_t n, int m, const T* __restrict__ V,
                                                const double* __restrict__ scale, const double* __restrict__ H,
                                                const double* __restrict__ csg, const int* __restrict__ flags,
                                                const T* __restrict__ dinv, double* __restrict__ x,
                                                T* __restrict__ u) {
    __shared__ double y[130];
    __shared__ T c[130];
    const int jd = flags[F_JDONE];
    if (jd == 0) {
        // no completed column: the correction is zero (the preconditioner input must not keep the
        // last iteration's vector)
        if (u)
            for (int64_t i = bx * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gx * blockDim.x) u[i] = (T)0;
        return;
    }
    if (threadIdx.x == 0) {
        const double* g = csg + 2 * m;
        for (int k = jd - 1; k >= 0; k--) {
            double a = g[k];
            for (int l = k + 1; l < jd; l++) a -= H[k * m + l] * y[l];
            y[k] = a / H[k * m + k];
        }
        for (int k = 0; k < jd; k++) c[k] = (T)(y[k] * scale[k]);
    }
    __syncthreads();
    for (int64_t i = bx * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gx * blockDim.x) {
        T acc = 0;
        for (int k = 0; k < jd; k++) acc += c[k] * V[(int64_t)k * n + i];
        if (u) u[i] = acc;
        else x[i] += (double)(dinv ? dinv[i] * acc : acc);
    }
}

template <class T>
__global__ void __launch_bounds__(256) gm_combine(int64_t n, int m, const T* __restrict__ V,
                                                  const double* __restrict__ scale, const double* __restrict__ H,
                                                  const double* __restrict__ csg, const int* __restrict__ flags,
                                                  const T* __restrict__ dinv, double* __restrict__ x,
                                                  T* __restrict__ u, Bat bt) {
    const int64_t ib = blockIdx.y;
    gm_combine_body<T>(blockIdx.x, gridDim.x, n, m, V + ib * bt.V, scale + ib * bt.scale, H + ib * bt.H,
                       csg + ib * bt.H, flags + ib * bt.flags, dinv ? dinv + ib * bt.n : nullptr, x + ib * bt.n,
                       u ? u + ib * bt.n : nullptr);
}

template <class T, int L>
__global__ void gm_block_apply(int64_t ne, const T* __restrict__ Binv, const T* __restrict__ v, double sc_const,
                               const double* __restrict__ scale, int j, T* __restrict__ z, double* __restrict__ x,
                               const int* __restrict__ flags) {
    if (flags && flags[F_CONV]) return;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= ne * L) return;
    const int64_t e = t / L;
    const int i = (int)(t % L);
    const T sc = scale ? (T)scale[j] : (T)sc_const;
    T acc = 0;
#pragma unroll
    for (int k = 0; k < L; k++) acc += Binv[(e * L + i) * L + k] * v[e * L + k];
    if (x) x[t] += (double)(acc * sc);
    else z[t] = acc * sc;
}

// A_s = A D^-1 (Jacobi) or A, cast to T
template <class T>
__global__ void gm_scale_matrix(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                const double* __restrict__ A, const double* __restrict__ dinv64, T* __restrict__ As,
                                int64_t nnz) {
    A += blockIdx.y * nnz;
    As += blockIdx.y * nnz;
    if (dinv64) dinv64 += blockIdx.y * n;
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int32_t k = rp[r]; k < rp[r + 1]; k++) {
        const double d = dinv64 ? dinv64[col[k]] : 1.0;
        As[k] = (T)(A[k] * d);
    }
}

__global__ void gm_cast(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

__global__ void gm_set_tols(double* st, double tol, double inner, double eta2, int nb, int64_t stride) {
    for (int q = 0; q < nb; q++) {
        double* s = st + q * stride;
        s[S_OUTERTOL] = tol;
        s[S_INNER] = inner;
        s[S_TOL] = tol;
        s[S_ETA2] = eta2;
    }
}

// Cahouet-Chabard, part 1: z_u = sc D_u^-1 v_u, zp = sc v_p (the pressure solve's right-hand side)
template <class T>
__global__ void cc_pre1(int64_t nu, int64_t np, const T* __restrict__ v, const double* __restrict__ scale, int j,
                        const double* __restrict__ vdinv, T* __restrict__ z, T* __restrict__ zp,
                        const int* __restrict__ flags) {
    if (flags && flags[F_CONV]) return;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double sc = scale ? scale[j] : 1.0;
    if (i < nu) z[i] = (T)(sc * vdinv[i] * (double)v[i]);
    else if (i < nu + np) zp[i - nu] = (T)(sc * (double)v[i]);
}
// part 2: z_p = -(alpha S^-1 (sc v_p) + beta M^-1 (sc v_p)) / tc^2 (S^-1 applied in place on zp)
template <class T>
__global__ void cc_pre2(int64_t nu, int64_t np, const T* __restrict__ v, const double* __restrict__ scale, int j,
                        const double* __restrict__ mpinv, const T* __restrict__ zp, T* __restrict__ z, double alpha,
                        double beta, double tc, const int* __restrict__ flags) {
    if (flags && flags[F_CONV]) return;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    const double sc = scale ? scale[j] : 1.0;
    const double vp = sc * (double)v[nu + i];
    z[nu + i] = (T)(-(alpha * (double)zp[i] + beta * mpinv[i] * vp) / (tc * tc));
}

template <class T>
int cc_apply(CCPre* cc, const T* v, const double* scale, int j, T* z, const int* flags, cudaStream_t st) {
    T* zp = nullptr;
    if constexpr (std::is_same<T, float>::value) zp = cc->zp32;
    else zp = cc->zp64;
    OCMP_LAUNCH(cc_pre1<T><<<nblk(cc->nu + cc->np, kThreads), kThreads, 0, st>>>(cc->nu, cc->np, v, scale, j, cc->vdinv,
                                                                              z, zp, flags));
    int r = strip_apply<T>(cc->strip, cc->pop->space, cc->pop->vals, zp, nullptr, 0, zp, flags, st);
    if (r) return r;
    OCMP_LAUNCH(cc_pre2<T><<<nblk(cc->np, kThreads), kThreads, 0, st>>>(cc->nu, cc->np, v, scale, j, cc->mpinv, zp, z,
                                                                     cc->alpha, cc->beta, cc->tc, flags));
    return OCMP_OK;
}

template <class T>
struct GmBufs {
    const T* A;        // Krylov matrix (scaled or plain)
    const T* dinv;     // for the final x update (Jacobi), or null
    const T* Binv;     // block Jacobi, or null
    T* V;
    T* z;              // block Jacobi / strip workspace
    Strip* strip;      // strip direct preconditioner, or null
    CCPre* cc;         // Cahouet-Chabard preconditioner, or null
};

// Host driver of the fused GMRES over a batch of sv->B systems (B = 1 for a single solve).
// Without graphs the host reads the convergence flags every check_every iterations; with graphs
// one restart cycle (m iterations, the x update and the next FP64 residual) is captured once into
// a CUDA graph and replayed, the host reading the flags only between cycles. Converged instances
// return at the top of every kernel.
template <class T, int TPR, int U>
int gm_run(const Ctx& c, const GmBufs<T>& B, const double* b, double* x, int maxit, double inner_tol, int* iters,
           int* cycles, double* relres0) {
    ocmp_solver_s* sv = c.sv;
    const ocmp_space_s* s = sv->s;
    const int64_t n = sv->n;
    const int m = sv->m;
    const int G = sv->grid;
    const int NB = sv->B;
    const Bat bt = sv->bat;
    double* csg = sv->H + (size_t)(m + 1) * m;
    const int nbp = G;
    double* red2 = sv->red + (m + 4);
    const bool block = B.Binv != nullptr;
    const bool strip = B.strip != nullptr;
    const bool ccp = B.cc != nullptr;
    const int64_t ne = s->mesh->ne;
    const int L = s->nloc;
    const dim3 gg(G, NB), gs(nblk(n * TPR, 256), NB);
    // The FP64 residual is bound by the FP64 pipe (1/58 of the FP32 rate here), not by HBM: half the
    // lanes per row of the SpMV halves the FP64 shuffle-reduction adds it spends beside the FMAs.
    constexpr int RTPR = TPR > 2 ? TPR / 2 : TPR;
    cudaStream_t ls = c.st;  // launch stream of the lambdas below (switched while capturing)
    auto block_apply = [&](int j, double* xo) {
        const unsigned nbk = nblk(ne * L, kThreads);
        switch (L) {
        case 3: OCMP_LAUNCH(gm_block_apply<T, 3><<<nbk, kThreads, 0, ls>>>(ne, B.Binv, xo ? B.z : B.V + (int64_t)j * n, 1.0, xo ? nullptr : sv->scale, j, B.z, xo, xo ? nullptr : sv->flags)); break;
        case 6: OCMP_LAUNCH(gm_block_apply<T, 6><<<nbk, kThreads, 0, ls>>>(ne, B.Binv, xo ? B.z : B.V + (int64_t)j * n, 1.0, xo ? nullptr : sv->scale, j, B.z, xo, xo ? nullptr : sv->flags)); break;
        case 10: OCMP_LAUNCH(gm_block_apply<T, 10><<<nbk, kThreads, 0, ls>>>(ne, B.Binv, xo ? B.z : B.V + (int64_t)j * n, 1.0, xo ? nullptr : sv->scale, j, B.z, xo, xo ? nullptr : sv->flags)); break;
        default: break;
        }
    };
    auto iteration = [&](int j) {
        const T* xin = B.V + (int64_t)j * n;
        if (block) {
            block_apply(j, nullptr);
            xin = B.z;
        } else if (strip) {
            // z = M^-1 (scale_j V_j); every sweep kernel returns at once after convergence
            strip_apply<T>(B.strip, s, sv->mat->vals, B.V + (int64_t)j * n, sv->scale, j, B.z, sv->flags, ls);
            xin = B.z;
        } else if (ccp) {
            cc_apply<T>(B.cc, B.V + (int64_t)j * n, sv->scale, j, B.z, sv->flags, ls);
            xin = B.z;
        }
        const bool timing = sv->time_spmv && ls == c.st && sv->worklog && (int)(sv->tev_used / 2) < sv->worklog_cap;
        if (timing) {
            while (sv->tev.size() < sv->tev_used + 2) {
                cudaEvent_t e;
                cudaEventCreate(&e);
                sv->tev.push_back(e);
            }
            cudaEventRecord(sv->tev[sv->tev_used], ls);
        }
        int* wlog = timing ? sv->worklog + sv->tev_used / 2 : nullptr;
        bool done_sell = false;
        if constexpr (std::is_same<T, float>::value) {
            if (sv->sell && B.A == sv->K32 && NB == 1) {
                const unsigned gsl = (unsigned)std::min<int64_t>(nblk(s->sell_slices * 32, 256), 2 * kGridCap);
                OCMP_LAUNCH(gm_spmv_sell<<<gsl, 256, 0, ls>>>(n, s->sell_slices, j, s->d_sell_off, s->d_sell_col, B.A,
                                                              s->d_free, xin, (block || strip || ccp) ? 0 : 1, B.V, sv->scale,
                                                              sv->flags, wlog));
                done_sell = true;
            }
        }
        if (!done_sell)
            OCMP_LAUNCH(gm_spmv<T, TPR, U><<<gs, 256, 0, ls>>>(n, j, s->d_rowptr, s->d_col, B.A, s->d_free, xin,
                                                             (block || strip || ccp) ? 0 : 1, B.V, sv->scale, sv->flags, bt,
                                                             wlog));
        if (timing) {
            cudaEventRecord(sv->tev[sv->tev_used + 1], ls);
            sv->tev_used += 2;
        }
        OCMP_LAUNCH(gm_dots<T><<<gg, 256, 0, ls>>>(n, j, B.V, sv->part, nbp, sv->cnt, sv->red, sv->flags, 0, 1, bt));
        OCMP_LAUNCH(gm_orth<T><<<gg, 256, 0, ls>>>(n, j, m, B.V, sv->red, sv->part, sv->cnt + 1, sv->H, csg, sv->st, sv->flags,
                                         sv->scale, 1, bt));
        OCMP_LAUNCH(gm_dots<T><<<gg, 256, 0, ls>>>(n, j, B.V, sv->part, nbp, sv->cnt + 2, red2, sv->flags, 1, 0, bt));
        OCMP_LAUNCH(gm_orth<T><<<gg, 256, 0, ls>>>(n, j, m, B.V, red2, sv->part, sv->cnt + 3, sv->H, csg, sv->st, sv->flags,
                                         sv->scale, 2, bt));
    };
    auto finish_cycle = [&]() {
        if (block) {
            OCMP_LAUNCH(gm_combine<T><<<gg, 256, 0, ls>>>(n, m, B.V, sv->scale, sv->H, csg, sv->flags, nullptr, x, B.z, bt));
            block_apply(0, x);
        } else if (strip) {
            OCMP_LAUNCH(gm_combine<T><<<gg, 256, 0, ls>>>(n, m, B.V, sv->scale, sv->H, csg, sv->flags, nullptr, x, B.z, bt));
            strip_apply<T>(B.strip, s, sv->mat->vals, B.z, nullptr, 0, B.z, nullptr, ls);
            strip_add<T>(n, B.z, x, ls);
        } else if (ccp) {
            OCMP_LAUNCH(gm_combine<T><<<gg, 256, 0, ls>>>(n, m, B.V, sv->scale, sv->H, csg, sv->flags, nullptr, x, B.z, bt));
            cc_apply<T>(B.cc, B.z, nullptr, 0, B.z, nullptr, ls);
            strip_add<T>(n, B.z, x, ls);
        } else {
            OCMP_LAUNCH(gm_combine<T><<<gg, 256, 0, ls>>>(n, m, B.V, sv->scale, sv->H, csg, sv->flags, B.dinv, x, nullptr, bt));
        }
        OCMP_LAUNCH(gm_resid<T, RTPR, U><<<gg, 256, 0, ls>>>(n, s->d_rowptr, s->d_col, sv->mat->vals, s->d_free, b, x, B.V,
                                                  sv->part, sv->cnt, sv->st, sv->flags, sv->scale, csg, m, 1,
                                                  s->d_lift_ptr, s->d_lift_pos, bt));
    };
    auto all = [&](int f) {
        for (int q = 0; q < NB; q++)
            if (!sv->hflags[q * F_NFLAG + f] && !sv->hflags[q * F_NFLAG + F_NONFIN]) return false;
        return true;
    };
    // Classical Gram-Schmidt, repeated only when |w| lost more than 99.9% of its length to the
    // projection (|w_new|^2 < 1e-6 |w|^2); the mass-dominated systems here lose far less per step.
    OCMP_LAUNCH(gm_set_tols<<<1, 1, 0, c.st>>>(sv->st, sv->prm.tol, inner_tol, 1e-6, NB, bt.st));
    OCMP_CUDA(cudaMemsetAsync(sv->flags, 0, sizeof(int) * F_NFLAG * NB, c.st));
    OCMP_LAUNCH(gm_resid<T, RTPR, U><<<gg, 256, 0, c.st>>>(n, s->d_rowptr, s->d_col, sv->mat->vals, s->d_free, b, x, B.V, sv->part,
                                              sv->cnt, sv->st, sv->flags, sv->scale, csg, m, 3, s->d_lift_ptr,
                                              s->d_lift_pos, bt));
    {
        std::vector<double> sth((size_t)S_NSLOT * NB);
        OCMP_CUDA(cudaMemcpyAsync(sth.data(), sv->st, sizeof(double) * S_NSLOT * NB, cudaMemcpyDeviceToHost, c.st));
        if (read_flags(c)) return OCMP_ERR_CUDA;
        for (int q = 0; q < NB; q++) relres0[q] = sth[(size_t)q * S_NSLOT + S_RES];
    }
    int it = 0, cyc = 0;
    const bool graph = sv->use_graph;
    const bool adaptive = sv->prm.check_every < 0;
    int next_check = std::max(1, sv->last_iters - 1);
    // Stream capture is not allowed on the legacy default stream: capture and replay on the
    // solver's own stream instead, ordered after and before the caller's work with events.
    Ctx cg = c;
    if (graph && c.st == nullptr) {
        if (!sv->gstream) {
            OCMP_CUDA(cudaStreamCreateWithFlags(&sv->gstream, cudaStreamNonBlocking));
            OCMP_CUDA(cudaEventCreateWithFlags(&sv->gev[0], cudaEventDisableTiming));
            OCMP_CUDA(cudaEventCreateWithFlags(&sv->gev[1], cudaEventDisableTiming));
        }
        cg.st = sv->gstream;
    }
    if (graph && (sv->gexec == nullptr || sv->g_b != b || sv->g_x != x || sv->g_stream != cg.st)) {
        if (sv->gexec) {
            cudaGraphExecDestroy(sv->gexec);
            sv->gexec = nullptr;
        }
        cudaGraph_t gph;
        const unsigned long long l0 = g_launches.load();
        OCMP_CUDA(cudaStreamBeginCapture(cg.st, cudaStreamCaptureModeThreadLocal));
        ls = cg.st;
        for (int j = 0; j < m; j++) iteration(j);
        finish_cycle();
        ls = c.st;
        OCMP_CUDA(cudaStreamEndCapture(cg.st, &gph));
        // captured launches run at each replay, not now
        sv->graph_kernels = g_launches.load() - l0;
        g_launches.fetch_sub(sv->graph_kernels);
        cudaError_t e = cudaGraphInstantiate(&sv->gexec, gph, 0);
        cudaGraphDestroy(gph);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        sv->g_b = b;
        sv->g_x = x;
        sv->g_stream = cg.st;
    }
    while (true) {
        if (all(F_OUTER) || it >= maxit) break;
        if (graph) {
            if (cg.st != c.st) {
                OCMP_CUDA(cudaEventRecord(sv->gev[0], c.st));
                OCMP_CUDA(cudaStreamWaitEvent(cg.st, sv->gev[0], 0));
            }
            OCMP_CUDA(cudaGraphLaunch(sv->gexec, cg.st));
            g_launches.fetch_add(sv->graph_kernels);
            if (cg.st != c.st) {
                OCMP_CUDA(cudaEventRecord(sv->gev[1], cg.st));
                OCMP_CUDA(cudaStreamWaitEvent(c.st, sv->gev[1], 0));
            }
            it += m;
        } else {
            for (int j = 0; j < m; j++) {
                iteration(j);
                it++;
                // fixed interval, or (check_every < 0) the first check one iteration before the
                // previous solve's count and then after every iteration
                const bool check = adaptive ? it >= next_check : ((j + 1) % std::max(1, sv->prm.check_every)) == 0;
                if (check || it >= maxit) {
                    if (read_flags(c)) return OCMP_ERR_CUDA;
                    if (all(F_CONV) || it >= maxit) break;
                    next_check = it + 1;
                }
            }
            finish_cycle();
        }
        cyc++;
        if (read_flags(c)) return OCMP_ERR_CUDA;
    }
    OCMP_CUDA(cudaGetLastError());
    for (int q = 0; q < NB; q++) iters[q] = sv->hflags[q * F_NFLAG + F_ITERS];
    sv->last_iters = iters[0];
    *cycles = cyc;
    return OCMP_OK;
}

template <class T>
int gm_dispatch(const Ctx& c, const GmBufs<T>& B, const double* b, double* x, int maxit, double inner_tol,
                int* iters, int* cycles, double* relres0) {
    const RowCfg rc = row_cfg(c.sv->s);
    if (rc.tpr == 2) return gm_run<T, 2, 4>(c, B, b, x, maxit, inner_tol, iters, cycles, relres0);
    if (rc.tpr == 4 && rc.u == 4) return gm_run<T, 4, 4>(c, B, b, x, maxit, inner_tol, iters, cycles, relres0);
    if (rc.tpr == 4) return gm_run<T, 4, 8>(c, B, b, x, maxit, inner_tol, iters, cycles, relres0);
    if (rc.tpr == 8 && rc.u == 4) return gm_run<T, 8, 4>(c, B, b, x, maxit, inner_tol, iters, cycles, relres0);
    if (rc.tpr == 8) return gm_run<T, 8, 8>(c, B, b, x, maxit, inner_tol, iters, cycles, relres0);
    return gm_run<T, 16, 8>(c, B, b, x, maxit, inner_tol, iters, cycles, relres0);
}

// |(b - A x_D)_free| and |(b - A x)_free| / that, with the fused residual kernel
int gm_norms(const Ctx& c, const double* b, const double* x, int mode) {
    ocmp_solver_s* sv = c.sv;
    const ocmp_space_s* s = sv->s;
    const RowCfg rc = row_cfg(s);
    double* csg = sv->H + (size_t)(sv->m + 1) * sv->m;
    const dim3 gg(sv->grid, sv->B);
#define GM_R(TPR, U)                                                                                                  \
    OCMP_LAUNCH(gm_resid<double, TPR, U><<<gg, 256, 0, c.st>>>(sv->n, s->d_rowptr, s->d_col, sv->mat->vals, s->d_free, b, x,      \
                                                   (double*)nullptr, sv->part, sv->cnt, sv->st, sv->flags, sv->scale, \
                                                   csg, sv->m, mode, s->d_lift_ptr, s->d_lift_pos, sv->bat))
    if (rc.tpr == 2) GM_R(2, 4);
    else if (rc.tpr == 4 && rc.u == 4) GM_R(4, 4);
    else if (rc.tpr == 4) GM_R(4, 8);
    else if (rc.tpr == 8 && rc.u == 4) GM_R(8, 4);
    else if (rc.tpr == 8) GM_R(8, 8);
    else GM_R(16, 8);
#undef GM_R
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

// ---------------------------------------------------------------------------------------------
// Group kernels: the GMRES kernel bodies above over the (instance, block) pairs of a group's active
// instances, a fixed grid striding over the list (its length is read from the device, so one
// captured graph serves every active set). A barrier ends each pair: the bodies keep state in
// shared memory.
#define OCMP_GX_LOOP(list, which)                                                                                      \
    for (int vb = blockIdx.x; vb < nact[which]; vb += gridDim.x) {                                                     \
        const int2 e = list[vb];                                                                                       \
        const GInst& d = I[e.x];                                                                                       \
        const int bx = e.y;
#define OCMP_GX_END                                                                                                    \
        __syncthreads();                                                                                               \
    }

template <class T>
__global__ void __launch_bounds__(256) gx_resid(const GInst* __restrict__ I, const int2* __restrict__ list,
                                                const int* __restrict__ nact, int m, int mode) {
    OCMP_GX_LOOP(list, 0)
    T* V0 = (mode == 1 || mode == 3) ? (T*)d.V : nullptr;
    double* csg = d.H + (int64_t)(m + 1) * m;
#define OCMP_GX_RESID(TPR, U)                                                                                          \
    gm_resid_body<T, TPR, U>(bx, d.gbn, d.n, d.rp, d.col, d.A64, d.freed, d.b, d.x, V0, d.part, d.cnt, d.st, d.flags,   \
                             d.scale, csg, m, mode, d.lift_ptr, d.lift_pos)
    switch (d.cfg) {
    case 0:
    case 1: OCMP_GX_RESID(2, 4); break;
    case 2: OCMP_GX_RESID(2, 8); break;
    case 3: OCMP_GX_RESID(4, 4); break;
    case 4: OCMP_GX_RESID(4, 8); break;
    default: OCMP_GX_RESID(8, 8); break;
    }
#undef OCMP_GX_RESID
    OCMP_GX_END
}

template <class T>
__global__ void __launch_bounds__(256) gx_spmv(const GInst* __restrict__ I, const int2* __restrict__ list,
                                               const int* __restrict__ nact, int j) {
    OCMP_GX_LOOP(list, 1)
    if (!d.flags[F_CONV]) {
        T* V = (T*)d.V;
        const T* K = (const T*)d.K;
        const T* xin = V + (int64_t)j * d.n;
        switch (d.cfg) {
        case 0: gm_spmv_body<T, 2, 4>(bx, d.n, j, d.rp, d.col, K, d.freed, xin, 1, V, d.scale); break;
        case 1: gm_spmv_body<T, 4, 4>(bx, d.n, j, d.rp, d.col, K, d.freed, xin, 1, V, d.scale); break;
        case 2: gm_spmv_body<T, 4, 8>(bx, d.n, j, d.rp, d.col, K, d.freed, xin, 1, V, d.scale); break;
        case 3: gm_spmv_body<T, 8, 4>(bx, d.n, j, d.rp, d.col, K, d.freed, xin, 1, V, d.scale); break;
        case 4: gm_spmv_body<T, 8, 8>(bx, d.n, j, d.rp, d.col, K, d.freed, xin, 1, V, d.scale); break;
        default: gm_spmv_body<T, 16, 8>(bx, d.n, j, d.rp, d.col, K, d.freed, xin, 1, V, d.scale); break;
        }
    }
    }   // no barrier needed: the SpMV body keeps nothing in shared memory
}

// pass 1: dots into red (counter 0), pass 2: gated dots into red + m + 4 (counter 2)
template <class T>
__global__ void __launch_bounds__(256) gx_dots(const GInst* __restrict__ I, const int2* __restrict__ list,
                                               const int* __restrict__ nact, int j, int m, int pass) {
    OCMP_GX_LOOP(list, 0)
    gm_dots_body<T>(bx, d.gbn, d.n, j, (const T*)d.V, d.part, d.gbn, d.cnt + (pass == 1 ? 0 : 2),
                    d.red + (pass == 1 ? 0 : m + 4), d.flags, pass == 1 ? 0 : 1, pass == 1 ? 1 : 0);
    OCMP_GX_END
}

template <class T>
__global__ void __launch_bounds__(256) gx_orth(const GInst* __restrict__ I, const int2* __restrict__ list,
                                               const int* __restrict__ nact, int j, int m, int pass) {
    OCMP_GX_LOOP(list, 0)
    gm_orth_body<T>(bx, d.gbn, d.n, j, m, (T*)d.V, d.red + (pass == 1 ? 0 : m + 4), d.part,
                    d.cnt + (pass == 1 ? 1 : 3), d.H, d.H + (int64_t)(m + 1) * m, d.st, d.flags, d.scale, pass);
    OCMP_GX_END
}

template <class T>
__global__ void __launch_bounds__(256) gx_combine(const GInst* __restrict__ I, const int2* __restrict__ list,
                                                  const int* __restrict__ nact, int m) {
    OCMP_GX_LOOP(list, 0)
    gm_combine_body<T>(bx, d.gbn, d.n, m, (const T*)d.V, d.scale, d.H, d.H + (int64_t)(m + 1) * m, d.flags,
                       (const T*)d.dinv, d.x, nullptr);
    OCMP_GX_END
}
#undef OCMP_GX_LOOP
#undef OCMP_GX_END

constexpr int kGroupRows = 2048;   // rows per reduction block of a group instance

// Host driver of a group solve: the fused GMRES of gm_run over every instance of every member, one
// launch per kernel of the iteration for all of them; one restart cycle (m iterations, the x
// update and the next FP64 residual) is captured once into a CUDA graph and replayed (the kernels
// read the right-hand sides and solutions through the descriptors, so the graph serves every
// solve), the host reading the members' flags between cycles. Converged instances return at the
// top of every kernel.
template <class T>
int group_run(ocmp_group_s* g, cudaStream_t st, std::vector<int>& its, std::vector<double>& r0, int* cycles) {
    const int m = g->m;
    auto read_all = [&]() -> int {
        for (ocmp_solver_s* sv : g->members)
            OCMP_CUDA(cudaMemcpyAsync(sv->hflags, sv->flags, sizeof(int) * F_NFLAG * sv->B, cudaMemcpyDeviceToHost, st));
        OCMP_CUDA(cudaStreamSynchronize(st));
        return OCMP_OK;
    };
    auto all_outer = [&]() {
        for (ocmp_solver_s* sv : g->members)
            for (int q = 0; q < sv->B; q++)
                if (!sv->hflags[q * F_NFLAG + F_OUTER] && !sv->hflags[q * F_NFLAG + F_NONFIN]) return false;
        return true;
    };
    // each kernel's grid is what stays resident at once (a larger grid would leave a second wave
    // waiting for the first to stride through the whole list)
    const int* gr = g->grid[std::is_same<T, double>::value ? 1 : 0];
    auto G = [&](int k, int tot) { return (unsigned)std::max(1, std::min(gr[k], tot)); };
    auto cycle = [&](cudaStream_t ls) {
        for (int j = 0; j < m; j++) {
            OCMP_LAUNCH(gx_spmv<T><<<G(0, g->stot), 256, 0, ls>>>(g->d_inst, g->d_slist, g->d_nact, j));
            OCMP_LAUNCH(gx_dots<T><<<G(1, g->gtot), 256, 0, ls>>>(g->d_inst, g->d_glist, g->d_nact, j, m, 1));
            OCMP_LAUNCH(gx_orth<T><<<G(2, g->gtot), 256, 0, ls>>>(g->d_inst, g->d_glist, g->d_nact, j, m, 1));
            OCMP_LAUNCH(gx_dots<T><<<G(1, g->gtot), 256, 0, ls>>>(g->d_inst, g->d_glist, g->d_nact, j, m, 2));
            OCMP_LAUNCH(gx_orth<T><<<G(2, g->gtot), 256, 0, ls>>>(g->d_inst, g->d_glist, g->d_nact, j, m, 2));
        }
        OCMP_LAUNCH(gx_combine<T><<<G(3, g->gtot), 256, 0, ls>>>(g->d_inst, g->d_glist, g->d_nact, m));
        OCMP_LAUNCH(gx_resid<T><<<G(4, g->gtot), 256, 0, ls>>>(g->d_inst, g->d_glist, g->d_nact, m, 1));
    };
    // the (instance, block) lists of the instances still iterating, after the flags were read
    auto set_active = [&](bool all_inst) -> int {
        int ng = 0, ns = 0;
        for (size_t i = 0; i < g->members.size(); i++) {
            ocmp_solver_s* sv = g->members[i];
            for (int q = 0; q < sv->B; q++) {
                if (!all_inst && (sv->hflags[q * F_NFLAG + F_OUTER] || sv->hflags[q * F_NFLAG + F_NONFIN])) continue;
                const int k = g->first[i] + q;
                const GInst& d = g->h_inst[k];
                for (int bb = 0; bb < d.gbn; bb++) g->h_glist[ng++] = make_int2(k, bb);
                for (int bb = 0; bb < d.sbn; bb++) g->h_slist[ns++] = make_int2(k, bb);
            }
        }
        g->h_nact[0] = ng;
        g->h_nact[1] = ns;
        if (ng) OCMP_CUDA(cudaMemcpyAsync(g->d_glist, g->h_glist, sizeof(int2) * ng, cudaMemcpyHostToDevice, st));
        if (ns) OCMP_CUDA(cudaMemcpyAsync(g->d_slist, g->h_slist, sizeof(int2) * ns, cudaMemcpyHostToDevice, st));
        OCMP_CUDA(cudaMemcpyAsync(g->d_nact, g->h_nact, 2 * sizeof(int), cudaMemcpyHostToDevice, st));
        return OCMP_OK;
    };
    for (ocmp_solver_s* sv : g->members) {
        const double inner = g->mixed ? (sv->prm.inner_tol > 0 ? sv->prm.inner_tol : 1e-4) : 0.0;
        OCMP_LAUNCH(gm_set_tols<<<1, 1, 0, st>>>(sv->st, sv->prm.tol, inner, 1e-6, sv->B, sv->bat.st));
        OCMP_CUDA(cudaMemsetAsync(sv->flags, 0, sizeof(int) * F_NFLAG * sv->B, st));
    }
    if (set_active(true)) return OCMP_ERR_CUDA;
    OCMP_LAUNCH(gx_resid<T><<<G(4, g->gtot), 256, 0, st>>>(g->d_inst, g->d_glist, g->d_nact, m, 3));
    {
        if (read_all()) return OCMP_ERR_CUDA;
        for (size_t i = 0; i < g->members.size(); i++) {
            ocmp_solver_s* sv = g->members[i];
            std::vector<double> sth((size_t)S_NSLOT * sv->B);
            OCMP_CUDA(cudaMemcpy(sth.data(), sv->st, sizeof(double) * sth.size(), cudaMemcpyDeviceToHost));
            for (int q = 0; q < sv->B; q++) r0[g->first[i] + q] = sth[(size_t)q * S_NSLOT + S_RES];
        }
    }
    if (!g->gexec) {
        if (!g->gstream) OCMP_CUDA(cudaStreamCreateWithFlags(&g->gstream, cudaStreamNonBlocking));
        cudaGraph_t gph;
        const unsigned long long l0 = g_launches.load();
        OCMP_CUDA(cudaStreamBeginCapture(g->gstream, cudaStreamCaptureModeThreadLocal));
        cycle(g->gstream);
        OCMP_CUDA(cudaStreamEndCapture(g->gstream, &gph));
        g->graph_kernels = g_launches.load() - l0;
        g_launches.fetch_sub(g->graph_kernels);
        cudaError_t e = cudaGraphInstantiate(&g->gexec, gph, 0);
        cudaGraphDestroy(gph);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (group cycle)");
    }
    int it = 0, cyc = 0;
    while (!all_outer() && it < g->maxit) {
        if (set_active(false)) return OCMP_ERR_CUDA;
        OCMP_CUDA(cudaGraphLaunch(g->gexec, st));
        g_launches.fetch_add(g->graph_kernels);
        it += m;
        cyc++;
        if (read_all()) return OCMP_ERR_CUDA;
    }
    for (size_t i = 0; i < g->members.size(); i++) {
        ocmp_solver_s* sv = g->members[i];
        for (int q = 0; q < sv->B; q++) its[g->first[i] + q] = sv->hflags[q * F_NFLAG + F_ITERS];
    }
    *cycles = cyc;
    return set_active(true);   // every instance again, for the final residuals
}

}  // namespace
}  // namespace ocmp

using namespace ocmp;

static void free_solver(ocmp_solver_s* sv) {
    void* ps[] = {sv->udiag, sv->dinv, sv->Binv, sv->V,   sv->w,     sv->z,   sv->r,     sv->p,    sv->dinv32, sv->Binv32,
                  sv->V32,  sv->w32,  sv->z32, sv->r32,   sv->p32, sv->d32,   sv->part, sv->pspmv,  sv->red,
                  sv->st,   sv->H,    sv->flags, sv->As64, sv->As32, sv->scale, sv->cnt};
    for (void* q : ps) dfree(q);
    if (sv->strip) strip_destroy(sv->strip);
    if (sv->cc) {
        if (sv->cc->strip) strip_destroy(sv->cc->strip);
        dfree(sv->cc->vdinv);
        dfree(sv->cc->mpinv);
        dfree(sv->cc->zp64);
        dfree(sv->cc->zp32);
        delete sv->cc;
    }
    if (sv->hflags) cudaFreeHost(sv->hflags);
    if (sv->gexec) cudaGraphExecDestroy(sv->gexec);
    if (sv->gstream) cudaStreamDestroy(sv->gstream);
    for (cudaEvent_t e : sv->tev) cudaEventDestroy(e);
    dfree(sv->worklog);
    for (cudaEvent_t e : sv->gev)
        if (e) cudaEventDestroy(e);
}

extern "C" {

int ocmp_solver_create(ocmp_matrix_t mat, const ocmp_solve_params_t* prm, ocmp_solver_t* out) {
    if (!mat || !prm || !out) return fail(OCMP_ERR_ARG, "ocmp_solver_create: null argument");
    if (prm->method != OCMP_CG && prm->method != OCMP_GMRES) return fail(OCMP_ERR_ARG, "ocmp_solver_create: method");
    if (prm->precond < OCMP_PRE_NONE || prm->precond > OCMP_PRE_CAHOUET_CHABARD)
        return fail(OCMP_ERR_ARG, "ocmp_solver_create: precond");
    if (prm->precision == OCMP_MIXED && prm->method == OCMP_CG && !mat->vals32)
        return fail(OCMP_ERR_ARG, "ocmp_solver_create: mixed-precision CG needs a matrix created with OCMP_MAT_FP32");
    if (prm->method == OCMP_CG && prm->precond != OCMP_PRE_JACOBI && prm->precond != OCMP_PRE_USER)
        return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solver_create: CG is built with a diagonal preconditioner");
    ocmp_space_s* s = mat->space;
    if (prm->precond == OCMP_PRE_BLOCK_JACOBI && (s->kind != OCMP_L2 || (s->nloc != 3 && s->nloc != 6 && s->nloc != 10)))
        return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solver_create: block Jacobi is built for L2 element blocks");
    if ((prm->precond == OCMP_PRE_STRIP || prm->precond == OCMP_PRE_CAHOUET_CHABARD) &&
        (prm->method != OCMP_GMRES || mat->B != 1))
        return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solver_create: the strip and Cahouet-Chabard preconditioners are built "
                                          "for GMRES on one matrix");
    auto* sv = new ocmp_solver_s();
    sv->mat = mat;
    sv->s = s;
    sv->prm = *prm;
    if (sv->prm.check_every == 0) sv->prm.check_every = 8;
    // a strip-preconditioned iteration costs two full sweeps: read the flags after every one
    if (prm->precond == OCMP_PRE_STRIP) sv->prm.check_every = 1;
    const int64_t n = sv->n = s->ndof;
    const int NB = sv->B = mat->B;
    if (NB > 1 && (prm->method != OCMP_GMRES || prm->precond == OCMP_PRE_BLOCK_JACOBI)) {
        delete sv;
        return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solver_create: batches are solved with GMRES + point Jacobi");
    }
    sv->m = std::max(1, std::min(128, prm->restart > 0 ? prm->restart : 30));
    const int m = sv->m;
    sv->nb = (int)std::max<int64_t>(1, std::min<int64_t>(1216, (n + 1023) / 1024));
    const bool gm = prm->method == OCMP_GMRES, mixed = prm->precision == OCMP_MIXED;
    const bool blk = prm->precond == OCMP_PRE_BLOCK_JACOBI;
    const int tpr = pick_tpr(s);
    const int64_t nbs = (n * tpr + kThreads - 1) / kThreads;
    // one wave of the grid-stride reduction kernels: resident blocks per SM of the heaviest of them
    // (they share the partial-sum layout, so they share the grid) times the SM count
    {
        int dev = 0, sms = 152, bmin = 8;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        auto occ = [&](const void* k) {
            int nbk = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbk, k, kThreads, 0) == cudaSuccess && nbk > 0)
                bmin = std::min(bmin, nbk);
        };
        occ((const void*)gm_resid<double, 4, 8>);
        occ((const void*)gm_resid<float, 4, 8>);
        occ((const void*)gm_dots<double>);
        occ((const void*)gm_orth<double>);
        occ((const void*)gm_dots<float>);
        occ((const void*)gm_orth<float>);
        sv->grid = (int)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(kGridCap, (int64_t)bmin * sms), nbs));
    }
    const int64_t hsz = (int64_t)(m + 1) * m + 4 * m + 2;
    sv->bat = Bat{NB > 1 ? n : 0,
                  NB > 1 ? s->nnz : 0,
                  NB > 1 ? (int64_t)(m + 1) * n : 0,
                  NB > 1 ? (int64_t)(m + 4) * sv->grid : 0,
                  NB > 1 ? (int64_t)S_NSLOT : 0,
                  NB > 1 ? (int64_t)F_NFLAG : 0,
                  NB > 1 ? (int64_t)(m + 2) : 0,
                  NB > 1 ? hsz : 0,
                  NB > 1 ? (int64_t)(3 * m + 12) : 0,
                  NB > 1 ? (int64_t)8 : 0};
    int st = OCMP_OK;
    auto A = [&](auto** p, size_t cnt) {
        if (!st) st = dalloc(p, cnt);
    };
    A(&sv->dinv, (size_t)n * NB);
    if (prm->precond == OCMP_PRE_USER) A(&sv->udiag, (size_t)n * NB);
    A(&sv->w, n);
    A(&sv->z, n);
    A(&sv->r, n);
    if (!mixed) {
        if (gm) A(&sv->V, (size_t)(m + 1) * n * NB);
        else A(&sv->p, n);
    }
    if (blk) A(&sv->Binv, (size_t)s->mesh->ne * s->nloc * s->nloc);
    if (!st && prm->precond == OCMP_PRE_STRIP) st = strip_create(s, &sv->strip);
    if (mixed) {
        A(&sv->dinv32, (size_t)n * NB);
        A(&sv->w32, n);
        A(&sv->z32, n);
        A(&sv->d32, n);
        if (gm) A(&sv->V32, (size_t)(m + 1) * n * NB);
        else {
            A(&sv->r32, n);
            A(&sv->p32, n);
        }
        if (blk) A(&sv->Binv32, (size_t)s->mesh->ne * s->nloc * s->nloc);
    }
    A(&sv->part, (size_t)std::max<int64_t>((int64_t)(m + 4) * kGridCap, (int64_t)(m + 4) * sv->grid * NB));
    A(&sv->pspmv, (size_t)nbs);
    A(&sv->red, (size_t)(3 * m + 12) * NB);
    A(&sv->st, (size_t)S_NSLOT * NB);
    A(&sv->H, (size_t)hsz * NB);
    A(&sv->scale, (size_t)(m + 2) * NB);
    A(&sv->cnt, (size_t)8 * NB);
    sv->borrow = gm && prm->precond == OCMP_PRE_JACOBI && mat->dinv &&
                 (mixed ? mat->svals32 != nullptr : mat->svals64 != nullptr);
    if (gm && !sv->borrow) {
        if (mixed) A(&sv->As32, (size_t)s->nnz * NB);
        else A(&sv->As64, (size_t)s->nnz * NB);
    }
    sv->K64 = sv->borrow ? mat->svals64 : sv->As64;
    sv->K32 = sv->borrow ? mat->svals32 : sv->As32;
    sv->sell = sv->borrow && mixed && (mat->flags & OCMP_MAT_SELL32) && s->d_sell_off != nullptr;
    A(&sv->flags, (size_t)F_NFLAG * NB);
    if (!st && cudaMemset(sv->cnt, 0, sizeof(unsigned) * 8 * NB) != cudaSuccess) st = fail(OCMP_ERR_CUDA, "cudaMemset");
    if (!st && cudaMemset(sv->st, 0, sizeof(double) * S_NSLOT * NB) != cudaSuccess)
        st = fail(OCMP_ERR_CUDA, "cudaMemset");
    if (!st && cudaMallocHost((void**)&sv->hflags, sizeof(int) * F_NFLAG * NB) != cudaSuccess)
        st = fail(OCMP_ERR_NOMEM, "cudaMallocHost");
    if (st) {
        free_solver(sv);
        delete sv;
        return st;
    }
    // USER: after ocmp_solver_set_diag; STRIP: after the matrix is assembled (OpenCMP builds its
    // preconditioners before the first assembly and updates them after every one)
    if (prm->precond != OCMP_PRE_USER && prm->precond != OCMP_PRE_STRIP) st = ocmp_solver_update(sv, nullptr);
    if (st) {
        free_solver(sv);
        delete sv;
        return st;
    }
    OCMP_CUDA(cudaDeviceSynchronize());
    *out = sv;
    return OCMP_OK;
}

int ocmp_solver_destroy(ocmp_solver_t sv) {
    if (!sv) return OCMP_OK;
    free_solver(sv);
    delete sv;
    return OCMP_OK;
}

int ocmp_solver_update(ocmp_solver_t sv, void* stream) {
    if (!sv) return fail(OCMP_ERR_ARG, "ocmp_solver_update: null solver");
    cudaStream_t st = (cudaStream_t)stream;
    ocmp_space_s* s = sv->s;
    const int64_t n = sv->n;
    const int NB = sv->B;
    if (sv->prm.precond == OCMP_PRE_USER) {
        if (!sv->udiag_set) return fail(OCMP_ERR_ARG, "ocmp_solver_update: set the diagonal with ocmp_solver_set_diag");
        OCMP_CUDA(cudaMemcpyAsync(sv->dinv, sv->udiag, sizeof(double) * n * NB, cudaMemcpyDeviceToDevice, st));
        if (sv->dinv32) OCMP_LAUNCH(gm_cast<<<nblk(n * NB, kThreads), kThreads, 0, st>>>(n * NB, sv->dinv, sv->dinv32));
    } else if (sv->borrow) {
        // the assembly's D^-1 scaled the Krylov matrix: use the same one for x = D^-1 y
        OCMP_CUDA(cudaMemcpyAsync(sv->dinv, sv->mat->dinv, sizeof(double) * n * NB, cudaMemcpyDeviceToDevice, st));
        if (sv->dinv32) OCMP_LAUNCH(gm_cast<<<nblk(n * NB, kThreads), kThreads, 0, st>>>(n * NB, sv->mat->dinv, sv->dinv32));
    } else {
        for (int q = 0; q < NB; q++) {
            OCMP_LAUNCH(jacobi_setup<double><<<nblk(n, kThreads), kThreads, 0, st>>>(n, s->d_diag, sv->mat->vals + q * s->nnz,
                                                                        s->d_free, sv->dinv + q * n));
            if (sv->dinv32)
                OCMP_LAUNCH(jacobi_setup<float><<<nblk(n, kThreads), kThreads, 0, st>>>(n, s->d_diag, sv->mat->vals + q * s->nnz,
                                                                           s->d_free, sv->dinv32 + q * n));
        }
    }
    if (sv->Binv) {
        const int64_t ne = s->mesh->ne;
        switch (s->nloc) {
        case 3: OCMP_LAUNCH(block_jacobi_setup<3><<<nblk(ne, 128), 128, 0, st>>>(ne, s->d_rowptr, s->d_col, sv->mat->vals, sv->Binv, sv->Binv32)); break;
        case 6: OCMP_LAUNCH(block_jacobi_setup<6><<<nblk(ne, 128), 128, 0, st>>>(ne, s->d_rowptr, s->d_col, sv->mat->vals, sv->Binv, sv->Binv32)); break;
        case 10: OCMP_LAUNCH(block_jacobi_setup<10><<<nblk(ne, 128), 128, 0, st>>>(ne, s->d_rowptr, s->d_col, sv->mat->vals, sv->Binv, sv->Binv32)); break;
        default: break;
        }
    }
    if (sv->strip) {
        sv->strip_ready = false;
        const int r = strip_factor(sv->strip, s, sv->mat->vals, st);
        if (r) return r;
        sv->strip_ready = true;
    }
    if (sv->As64 || sv->As32) {
        const double* d = sv->prm.precond == OCMP_PRE_JACOBI || sv->prm.precond == OCMP_PRE_USER ? sv->dinv : nullptr;
        const dim3 g(nblk(n, kThreads), NB);
        if (sv->As64)
            OCMP_LAUNCH(gm_scale_matrix<double><<<g, kThreads, 0, st>>>(n, s->d_rowptr, s->d_col, sv->mat->vals, d, sv->As64, s->nnz));
        if (sv->As32)
            OCMP_LAUNCH(gm_scale_matrix<float><<<g, kThreads, 0, st>>>(n, s->d_rowptr, s->d_col, sv->mat->vals, d, sv->As32, s->nnz));
    }
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int ocmp_solver_set_diag(ocmp_solver_t sv, const double* dinv, void* stream) {
    if (!sv || !dinv) return fail(OCMP_ERR_ARG, "ocmp_solver_set_diag: null argument");
    if (sv->prm.precond != OCMP_PRE_USER) return fail(OCMP_ERR_ARG, "ocmp_solver_set_diag: solver not created with OCMP_PRE_USER");
    OCMP_CUDA(cudaMemcpyAsync(sv->udiag, dinv, sizeof(double) * sv->n * sv->B, cudaMemcpyDeviceToDevice,
                              (cudaStream_t)stream));
    sv->udiag_set = true;
    return OCMP_OK;
}

int ocmp_solver_spmv_timing(ocmp_solver_t sv, int32_t on) {
    if (!sv) return fail(OCMP_ERR_ARG, "ocmp_solver_spmv_timing: null solver");
    sv->time_spmv = on != 0;
    sv->spmv_launches = 0;
    sv->spmv_ms = 0;
    if (on && !sv->worklog) {
        const int st = dalloc(&sv->worklog, 4096);
        if (st) return st;
        sv->worklog_cap = 4096;
    }
    return OCMP_OK;
}

int ocmp_solver_spmv_stats(ocmp_solver_t sv, int64_t* launches, double* total_ms) {
    if (!sv || !launches || !total_ms) return fail(OCMP_ERR_ARG, "ocmp_solver_spmv_stats: null argument");
    *launches = sv->spmv_launches;
    *total_ms = sv->spmv_ms;
    return OCMP_OK;
}

int ocmp_solver_set_graph(ocmp_solver_t sv, int32_t on) {
    if (!sv) return fail(OCMP_ERR_ARG, "ocmp_solver_set_graph: null solver");
    if (on && sv->prm.method != OCMP_GMRES)
        return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solver_set_graph: graphs are built for GMRES");
    if (on && (sv->strip || sv->prm.precond == OCMP_PRE_CAHOUET_CHABARD))
        return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solver_set_graph: the strip preconditioners run without graphs");
    sv->use_graph = on != 0;
    if (!on && sv->gexec) {
        cudaGraphExecDestroy(sv->gexec);
        sv->gexec = nullptr;
    }
    return OCMP_OK;
}

int ocmp_solver_set_cahouet_chabard(ocmp_solver_t sv, ocmp_matrix_t pop, const double* vdinv, const double* mpinv,
                                    int64_t nu, double alpha, double beta, double tc, int32_t refactor,
                                    void* stream) {
    if (!sv || !pop || !vdinv || !mpinv) return fail(OCMP_ERR_ARG, "ocmp_solver_set_cahouet_chabard: null argument");
    if (sv->prm.precond != OCMP_PRE_CAHOUET_CHABARD)
        return fail(OCMP_ERR_ARG, "ocmp_solver_set_cahouet_chabard: solver not created with OCMP_PRE_CAHOUET_CHABARD");
    const int64_t np = pop->space->ndof;
    if (nu < 0 || nu + np != sv->n || pop->B != 1)
        return fail(OCMP_ERR_ARG, "ocmp_solver_set_cahouet_chabard: velocity + pressure dofs must make the system");
    if (!(tc != 0.0)) return fail(OCMP_ERR_ARG, "ocmp_solver_set_cahouet_chabard: tc must not be zero");
    cudaStream_t st = (cudaStream_t)stream;
    CCPre* cc = sv->cc;
    if (cc && cc->pop != pop) {
        if (cc->strip) strip_destroy(cc->strip);
        cc->strip = nullptr;
        cc->pop = pop;
        refactor = 1;
    }
    if (!cc) {
        cc = new CCPre();
        cc->pop = pop;
        cc->np = np;
        int r = dalloc(&cc->vdinv, (size_t)std::max<int64_t>(nu, 1));
        if (!r) r = dalloc(&cc->mpinv, (size_t)np);
        if (!r) r = dalloc(&cc->zp64, (size_t)np);
        if (!r) r = dalloc(&cc->zp32, (size_t)np);
        if (r) {
            dfree(cc->vdinv);
            dfree(cc->mpinv);
            dfree(cc->zp64);
            delete cc;
            return r;
        }
        sv->cc = cc;
        refactor = 1;
    }
    cc->nu = nu;
    cc->np = np;
    cc->alpha = alpha;
    cc->beta = beta;
    cc->tc = tc;
    if (nu) OCMP_CUDA(cudaMemcpyAsync(cc->vdinv, vdinv, sizeof(double) * nu, cudaMemcpyDeviceToDevice, st));
    OCMP_CUDA(cudaMemcpyAsync(cc->mpinv, mpinv, sizeof(double) * np, cudaMemcpyDeviceToDevice, st));
    if (!cc->strip) {
        const int r = strip_create(pop->space, &cc->strip);
        if (r) return r;
    }
    if (refactor) {
        const int r = strip_factor(cc->strip, pop->space, pop->vals, st);
        if (r) return r;
    }
    return OCMP_OK;
}

int ocmp_solver_strip_stats(ocmp_solver_t sv, ocmp_strip_stats_t* out) {
    if (!sv || !out) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_stats: null argument");
    if (!sv->strip) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_stats: solver not created with OCMP_PRE_STRIP");
    strip_stats(sv->strip, out);
    return OCMP_OK;
}

int ocmp_solver_strip_timing(ocmp_solver_t sv, int32_t on) {
    if (!sv) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_timing: null solver");
    if (!sv->strip) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_timing: solver not created with OCMP_PRE_STRIP");
    strip_set_timing(sv->strip, on != 0);
    return OCMP_OK;
}

int ocmp_solver_strip_gemm(ocmp_solver_t sv, int32_t kind) {
    if (!sv) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_gemm: null solver");
    if (!sv->strip) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_gemm: solver not created with OCMP_PRE_STRIP");
    if (kind != 0 && kind != 1) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_gemm: kind is 0 (SIMT) or 1 (tensor cores)");
    strip_set_gemm(sv->strip, kind);
    return OCMP_OK;
}

int ocmp_solver_strip_schulz(ocmp_solver_t sv, int32_t on) {
    if (!sv) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_schulz: null solver");
    if (!sv->strip) return fail(OCMP_ERR_ARG, "ocmp_solver_strip_schulz: solver not created with OCMP_PRE_STRIP");
    strip_set_schulz(sv->strip, on != 0);
    return OCMP_OK;
}

// Batched GMRES solve of all B systems of the solver's matrix: b and x hold B vectors of ndof.
int ocmp_solve_batch(ocmp_solver_t sv, const double* b, double* x, void* stream, ocmp_solve_info_t* infos) {
    if (!sv || !b || !x) return fail(OCMP_ERR_ARG, "ocmp_solve_batch: null argument");
    if (sv->prm.method != OCMP_GMRES) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solve_batch: GMRES only");
    Ctx c;
    c.sv = sv;
    c.st = (cudaStream_t)stream;
    c.tpr = pick_tpr(sv->s);
    c.grid = sv->nb;
    const int NB = sv->B;
    const ocmp_solve_params_t& P = sv->prm;
    const bool mixed = P.precision == OCMP_MIXED, jac = P.precond == OCMP_PRE_JACOBI || P.precond == OCMP_PRE_USER;
    std::vector<double> r0(NB, 0.0);
    std::vector<int> its(NB, 0);
    int cyc = 0, st;
    if (!mixed) {
        GmBufs<double> B{sv->K64, jac ? sv->dinv : nullptr, nullptr, sv->V, sv->z, nullptr, nullptr};
        st = gm_dispatch<double>(c, B, b, x, P.maxit, 0.0, its.data(), &cyc, r0.data());
    } else {
        GmBufs<float> B{sv->K32, jac ? sv->dinv32 : nullptr, nullptr, sv->V32, sv->z32, nullptr, nullptr};
        st = gm_dispatch<float>(c, B, b, x, P.maxit, P.inner_tol > 0 ? P.inner_tol : 1e-4, its.data(), &cyc,
                                r0.data());
    }
    if (st) return st;
    // the FP64 residual of each returned x: the last cycle start, or a fresh one
    st = gm_norms(c, b, x, 2);
    if (st) return st;
    std::vector<double> sth((size_t)S_NSLOT * NB);
    OCMP_CUDA(cudaMemcpyAsync(sth.data(), sv->st, sizeof(double) * S_NSLOT * NB, cudaMemcpyDeviceToHost, c.st));
    OCMP_CUDA(cudaStreamSynchronize(c.st));
    int worst = OCMP_OK;
    for (int q = 0; q < NB; q++) {
        const double rr = sth[(size_t)q * S_NSLOT + S_RES];
        int status = OCMP_OK;
        if (sv->hflags[q * F_NFLAG + F_NONFIN] || !std::isfinite(rr)) status = OCMP_ERR_NONFINITE;
        else if (rr > P.tol) status = sv->hflags[q * F_NFLAG + F_BREAK] ? OCMP_BREAKDOWN : OCMP_NOT_CONVERGED;
        if (infos) {
            infos[q].status = status;
            infos[q].iterations = its[q];
            infos[q].outer_iterations = cyc;
            infos[q].relres0 = r0[q];
            infos[q].relres = rr;
        }
        if (status != OCMP_OK && worst == OCMP_OK) worst = status;
    }
    if (worst != OCMP_OK) set_error("ocmp_solve_batch: at least one system did not reach the tolerance");
    return worst;
}

int ocmp_solve(ocmp_solver_t sv, const double* b, double* x, void* stream, ocmp_solve_info_t* info) {
    if (!sv || !b || !x) return fail(OCMP_ERR_ARG, "ocmp_solve: null argument");
    Ctx c;
    c.sv = sv;
    c.st = (cudaStream_t)stream;
    c.tpr = pick_tpr(sv->s);
    c.grid = sv->nb;
    const int64_t n = sv->n;
    const ocmp_solve_params_t& P = sv->prm;
    const bool gm = P.method == OCMP_GMRES, mixed = P.precision == OCMP_MIXED;
    int st = OCMP_OK;
    double hst[S_NSLOT];
    int iters = 0, outer = 0;
    bool nonfin = false, brk = false;
    double relres0 = 0, relres = 0;
    if (gm) {
        const bool jac = P.precond == OCMP_PRE_JACOBI || P.precond == OCMP_PRE_USER;
        if (sv->B != 1) return fail(OCMP_ERR_ARG, "ocmp_solve: batched matrix, use ocmp_solve_batch");
        if (sv->strip && !sv->strip_ready)
            return fail(OCMP_ERR_ARG, "ocmp_solve: the strip preconditioner is not factorised (call ocmp_solver_update "
                                      "after assembling the matrix)");
        if (!mixed) {
            if (P.precond == OCMP_PRE_CAHOUET_CHABARD && !sv->cc)
                return fail(OCMP_ERR_ARG, "ocmp_solve: set the Cahouet-Chabard data (ocmp_solver_set_cahouet_chabard)");
            GmBufs<double> B{sv->K64, jac ? sv->dinv : nullptr, sv->Binv, sv->V, sv->z, sv->strip, sv->cc};
            st = gm_dispatch<double>(c, B, b, x, P.maxit, 0.0, &iters, &outer, &relres0);
        } else {
            if (P.precond == OCMP_PRE_CAHOUET_CHABARD && !sv->cc)
                return fail(OCMP_ERR_ARG, "ocmp_solve: set the Cahouet-Chabard data (ocmp_solver_set_cahouet_chabard)");
            GmBufs<float> B{sv->K32, jac ? sv->dinv32 : nullptr, sv->Binv32, sv->V32, sv->z32, sv->strip, sv->cc};
            st = gm_dispatch<float>(c, B, b, x, P.maxit, P.inner_tol > 0 ? P.inner_tol : 1e-4, &iters, &outer,
                                    &relres0);
        }
        if (st) return st;
        nonfin = sv->hflags[F_NONFIN] != 0 || !std::isfinite(relres0);
        brk = sv->hflags[F_BREAK] != 0;
        if (sv->hflags[F_OUTER] && !nonfin) {
            // the last cycle-start residual is the FP64 residual of the returned x
            OCMP_CUDA(cudaMemcpyAsync(hst, sv->st, sizeof(hst), cudaMemcpyDeviceToHost, c.st));
            OCMP_CUDA(cudaStreamSynchronize(c.st));
            relres = hst[S_RES];
        } else {
            st = gm_norms(c, b, x, 2);
            if (st) return st;
            OCMP_CUDA(cudaMemcpyAsync(hst, sv->st, sizeof(hst), cudaMemcpyDeviceToHost, c.st));
            OCMP_CUDA(cudaStreamSynchronize(c.st));
            relres = hst[S_RES];
        }
        if (sv->tev_used) {
            // only the launches that did the product count (those queued past convergence return
            // at once and read no matrix)
            std::vector<int> wk(sv->tev_used / 2, 0);
            OCMP_CUDA(cudaMemcpyAsync(wk.data(), sv->worklog, sizeof(int) * wk.size(), cudaMemcpyDeviceToHost, c.st));
            OCMP_CUDA(cudaStreamSynchronize(c.st));
            for (size_t k = 0; k + 1 < sv->tev_used; k += 2) {
                if (!wk[k / 2]) continue;
                float ms = 0;
                OCMP_CUDA(cudaEventElapsedTime(&ms, sv->tev[k], sv->tev[k + 1]));
                sv->spmv_ms += ms;
                sv->spmv_launches++;
            }
        }
        sv->tev_used = 0;
    } else {
        st = rhs_norm(c, b, x);
        if (st) return st;
        st = residual64(c, b, x, sv->r);
        if (st) return st;
        double red0 = 0;
        OCMP_CUDA(cudaMemcpyAsync(&red0, sv->red, sizeof(double), cudaMemcpyDeviceToHost, c.st));
        OCMP_CUDA(cudaMemcpyAsync(hst, sv->st, sizeof(hst), cudaMemcpyDeviceToHost, c.st));
        OCMP_CUDA(cudaStreamSynchronize(c.st));
        const double nbv = hst[S_NB];
        relres0 = std::sqrt(std::max(red0, 0.0)) / nbv;
        nonfin = !std::isfinite(relres0);
        if (!nonfin && relres0 > P.tol) {
            if (!mixed) {
                st = cg_core<double, double, double>(c, sv->mat->vals, sv->dinv, sv->r, sv->z, sv->p, sv->w, x,
                                                     P.maxit, P.tol, &iters);
                if (st) return st;
                nonfin = sv->hflags[F_NONFIN] != 0;
                brk = sv->hflags[F_BREAK] != 0;
            } else {
                double beta = std::sqrt(std::max(red0, 0.0));
                while (iters < P.maxit) {
                    OCMP_LAUNCH(set_state<<<1, 1, 0, c.st>>>(sv->st, S_BETA, beta));
                    OCMP_LAUNCH(set_state<<<1, 1, 0, c.st>>>(sv->st, S_NB, 1.0));
                    const double itol = std::max(P.inner_tol > 0 ? P.inner_tol : 1e-4, kTargetMargin * P.tol * nbv / beta);
                    OCMP_CUDA(cudaMemsetAsync(sv->d32, 0, sizeof(float) * n, c.st));
                    int it_in = 0;
                    OCMP_LAUNCH(scale_to_float<<<c.grid, kThreads, 0, c.st>>>(n, sv->r, sv->st, sv->r32));
                    st = cg_core<float, float, float>(c, sv->mat->vals32, sv->dinv32, sv->r32, sv->z32, sv->p32,
                                                      sv->w32, sv->d32, P.maxit - iters, itol, &it_in);
                    if (st) return st;
                    iters += std::max(it_in, 1);
                    outer++;
                    if (sv->hflags[F_NONFIN]) {
                        nonfin = true;
                        break;
                    }
                    OCMP_LAUNCH(set_state<<<1, 1, 0, c.st>>>(sv->st, S_BETA, beta));
                    OCMP_LAUNCH(add_scaled_float<<<c.grid, kThreads, 0, c.st>>>(n, sv->d32, sv->st, x));
                    OCMP_LAUNCH(set_state<<<1, 1, 0, c.st>>>(sv->st, S_NB, nbv));
                    st = residual64(c, b, x, sv->r);
                    if (st) return st;
                    OCMP_CUDA(cudaMemcpyAsync(&red0, sv->red, sizeof(double), cudaMemcpyDeviceToHost, c.st));
                    OCMP_CUDA(cudaStreamSynchronize(c.st));
                    beta = std::sqrt(std::max(red0, 0.0));
                    if (!std::isfinite(beta)) {
                        nonfin = true;
                        break;
                    }
                    if (beta / nbv <= P.tol) break;
                }
            }
        }
        OCMP_LAUNCH(set_state<<<1, 1, 0, c.st>>>(sv->st, S_NB, nbv));
        st = residual64(c, b, x, (double*)nullptr);
        if (st) return st;
        OCMP_CUDA(cudaMemcpyAsync(&red0, sv->red, sizeof(double), cudaMemcpyDeviceToHost, c.st));
        OCMP_CUDA(cudaStreamSynchronize(c.st));
        relres = std::sqrt(std::max(red0, 0.0)) / nbv;
    }
    int status = OCMP_OK;
    if (nonfin || !std::isfinite(relres)) status = OCMP_ERR_NONFINITE;
    else if (relres > P.tol) status = brk ? OCMP_BREAKDOWN : OCMP_NOT_CONVERGED;
    if (info) {
        info->status = status;
        info->iterations = iters;
        info->outer_iterations = outer;
        info->relres0 = relres0;
        info->relres = relres;
    }
    if (status == OCMP_ERR_NONFINITE) set_error("ocmp_solve: non-finite value in the right-hand side or iteration");
    else if (status == OCMP_NOT_CONVERGED) set_error("ocmp_solve: iteration cap reached before the tolerance");
    else if (status == OCMP_BREAKDOWN) set_error("ocmp_solve: Krylov breakdown");
    return status;
}


int ocmp_group_create(const ocmp_solver_t* solvers, int32_t count, ocmp_group_t* out) {
    if (!solvers || count <= 0 || !out) return fail(OCMP_ERR_ARG, "ocmp_group_create: no solvers");
    *out = nullptr;
    auto* g = new ocmp_group_s();
    for (int i = 0; i < count; i++) {
        ocmp_solver_s* sv = solvers[i];
        const ocmp_solve_params_t& P = sv ? sv->prm : ocmp_solve_params_t{};
        const char* why = nullptr;
        if (!sv) why = "null solver";
        else if (P.method != OCMP_GMRES) why = "members must be GMRES solvers";
        else if (P.precond != OCMP_PRE_JACOBI && P.precond != OCMP_PRE_USER && P.precond != OCMP_PRE_NONE)
            why = "members must use point Jacobi (or no) preconditioning";
        else if (sv->sell) why = "members' FP32 Krylov matrices must be in CSR order (no OCMP_MAT_SELL32)";
        else if (i > 0 && (sv->m != g->m || (P.precision == OCMP_MIXED) != g->mixed || P.maxit != g->maxit))
            why = "members must share the restart, the precision and the iteration cap";
        if (why) {
            delete g;
            return fail(OCMP_ERR_UNSUPPORTED, std::string("ocmp_group_create: ") + why);
        }
        if (i == 0) {
            g->m = sv->m;
            g->mixed = P.precision == OCMP_MIXED;
            g->maxit = P.maxit;
        }
        g->members.push_back(sv);
        g->first.push_back(g->ninst);
        const ocmp_space_s* s = sv->s;
        const RowCfg rc = row_cfg(s);
        const int cfg = rc.tpr == 2 ? 0 : rc.tpr == 4 ? (rc.u == 4 ? 1 : 2) : rc.tpr == 8 ? (rc.u == 4 ? 3 : 4) : 5;
        const int tpr = cfg == 0 ? 2 : cfg <= 2 ? 4 : cfg <= 4 ? 8 : 16;
        const int64_t n = sv->n, m = sv->m;
        const Bat& bt = sv->bat;
        const size_t ts = g->mixed ? sizeof(float) : sizeof(double);
        const bool jac = P.precond == OCMP_PRE_JACOBI || P.precond == OCMP_PRE_USER;
        for (int q = 0; q < sv->B; q++) {
            GInst d{};
            d.n = n;
            d.rp = s->d_rowptr;
            d.col = s->d_col;
            d.freed = s->d_free;
            d.lift_ptr = s->d_lift_ptr;
            d.lift_pos = s->d_lift_pos;
            d.A64 = sv->mat->vals + q * s->nnz;
            const char* K = g->mixed ? (const char*)sv->K32 : (const char*)sv->K64;
            d.K = K + ts * q * s->nnz;
            const char* dv = jac ? (g->mixed ? (const char*)sv->dinv32 : (const char*)sv->dinv) : nullptr;
            d.dinv = dv ? dv + ts * q * n : nullptr;
            char* V = g->mixed ? (char*)sv->V32 : (char*)sv->V;
            d.V = V + ts * q * (m + 1) * n;
            d.part = sv->part + q * bt.part;
            d.cnt = sv->cnt + q * bt.cnt;
            d.st = sv->st + q * bt.st;
            d.flags = sv->flags + q * bt.flags;
            d.scale = sv->scale + q * bt.scale;
            d.H = sv->H + q * bt.H;
            d.red = sv->red + q * bt.red;
            // reduction blocks in proportion to the rows (the partial sums fit the member's layout,
            // sized for sv->grid blocks)
            d.gbn = (int)std::max<int64_t>(1, std::min<int64_t>(sv->grid, (n + kGroupRows - 1) / kGroupRows));
            d.sbn = (int)nblk(n * tpr, 256);
            d.cfg = cfg;
            g->gtot += d.gbn;
            g->stot += d.sbn;
            g->h_inst.push_back(d);
            g->ninst++;
        }
    }
    {
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const void* ks[2][5] = {{(const void*)gx_spmv<float>, (const void*)gx_dots<float>, (const void*)gx_orth<float>,
                                 (const void*)gx_combine<float>, (const void*)gx_resid<float>},
                                {(const void*)gx_spmv<double>, (const void*)gx_dots<double>,
                                 (const void*)gx_orth<double>, (const void*)gx_combine<double>,
                                 (const void*)gx_resid<double>}};
        for (int t = 0; t < 2; t++)
            for (int k = 0; k < 5; k++) {
                int nb = 0;
                if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ks[t][k], 256, 0) != cudaSuccess || nb < 1) nb = 1;
                g->grid[t][k] = nb * sms;
            }
    }
    int st = dalloc(&g->d_glist, (size_t)g->gtot);
    if (!st) st = dalloc(&g->d_slist, (size_t)g->stot);
    if (!st) st = dalloc(&g->d_nact, 2);
    if (!st) st = dalloc(&g->d_inst, (size_t)g->ninst);
    if (!st && (cudaMallocHost((void**)&g->h_glist, sizeof(int2) * g->gtot) != cudaSuccess ||
                cudaMallocHost((void**)&g->h_slist, sizeof(int2) * g->stot) != cudaSuccess ||
                cudaMallocHost((void**)&g->h_nact, 2 * sizeof(int)) != cudaSuccess))
        st = fail(OCMP_ERR_NOMEM, "ocmp_group_create: pinned lists");
    if (st) {
        ocmp_group_destroy(g);
        return st;
    }
    *out = g;
    return OCMP_OK;
}

int ocmp_group_destroy(ocmp_group_t g) {
    if (!g) return OCMP_OK;
    dfree(g->d_glist);
    dfree(g->d_slist);
    dfree(g->d_nact);
    dfree(g->d_inst);
    if (g->h_glist) cudaFreeHost(g->h_glist);
    if (g->h_slist) cudaFreeHost(g->h_slist);
    if (g->h_nact) cudaFreeHost(g->h_nact);
    if (g->gexec) cudaGraphExecDestroy(g->gexec);
    if (g->gstream) cudaStreamDestroy(g->gstream);
    delete g;
    return OCMP_OK;
}

int ocmp_group_solve(ocmp_group_t g, const double* const* b, double* const* x, void* stream, ocmp_solve_info_t* infos) {
    if (!g || !b || !x) return fail(OCMP_ERR_ARG, "ocmp_group_solve: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    for (size_t i = 0; i < g->members.size(); i++) {
        ocmp_solver_s* sv = g->members[i];
        if (!b[i] || !x[i]) return fail(OCMP_ERR_ARG, "ocmp_group_solve: null right-hand side or solution");
        for (int q = 0; q < sv->B; q++) {
            GInst& d = g->h_inst[g->first[i] + q];
            d.b = b[i] + q * sv->n;
            d.x = x[i] + q * sv->n;
        }
    }
    OCMP_CUDA(cudaMemcpyAsync(g->d_inst, g->h_inst.data(), sizeof(GInst) * g->ninst, cudaMemcpyHostToDevice, st));
    std::vector<int> its(g->ninst, 0);
    std::vector<double> r0(g->ninst, 0.0);
    int cyc = 0;
    int r = g->mixed ? group_run<float>(g, st, its, r0, &cyc) : group_run<double>(g, st, its, r0, &cyc);
    if (r) return r;
    // the FP64 residual of every returned x
    const unsigned gg = (unsigned)std::max(1, std::min(g->grid[g->mixed ? 0 : 1][4], g->gtot));
    if (g->mixed) OCMP_LAUNCH(gx_resid<float><<<gg, 256, 0, st>>>(g->d_inst, g->d_glist, g->d_nact, g->m, 2));
    else OCMP_LAUNCH(gx_resid<double><<<gg, 256, 0, st>>>(g->d_inst, g->d_glist, g->d_nact, g->m, 2));
    OCMP_CUDA(cudaGetLastError());
    int worst = OCMP_OK;
    for (size_t i = 0; i < g->members.size(); i++) {
        ocmp_solver_s* sv = g->members[i];
        std::vector<double> sth((size_t)S_NSLOT * sv->B);
        OCMP_CUDA(cudaMemcpyAsync(sth.data(), sv->st, sizeof(double) * sth.size(), cudaMemcpyDeviceToHost, st));
        OCMP_CUDA(cudaStreamSynchronize(st));
        for (int q = 0; q < sv->B; q++) {
            const int k = g->first[i] + q;
            const double rr = sth[(size_t)q * S_NSLOT + S_RES];
            int status = OCMP_OK;
            if (sv->hflags[q * F_NFLAG + F_NONFIN] || !std::isfinite(rr)) status = OCMP_ERR_NONFINITE;
            else if (rr > sv->prm.tol) status = sv->hflags[q * F_NFLAG + F_BREAK] ? OCMP_BREAKDOWN : OCMP_NOT_CONVERGED;
            if (infos) {
                infos[k].status = status;
                infos[k].iterations = its[k];
                infos[k].outer_iterations = cyc;
                infos[k].relres0 = r0[k];
                infos[k].relres = rr;
            }
            if (status != OCMP_OK && worst == OCMP_OK) worst = status;
        }
    }
    if (worst != OCMP_OK) set_error("ocmp_group_solve: at least one system did not reach the tolerance");
    return worst;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Allocation-free CG. Some callers cannot call cudaMalloc at the moment they need a solve: hosts
// whose device memory belongs to another allocator's fixed pool (cudaMalloc would take memory that
// pool has already claimed, or fail), and loops that cannot take the implicit device-wide
// synchronisation of cudaFree. ocmp_solve_cg_noalloc serves them: it runs the
// same FP64 Jacobi-preconditioned CG as ocmp_solve with method OCMP_CG, but its workspace (five
// n-vectors, reduction partials, scalars and flags) lives in the file-scope device arrays below,
// which the CUDA driver allocates once per device when this library is loaded and keeps until exit.
// The caller passes only the assembled matrix, the right-hand side and the initial guess/result.
namespace {

constexpr int64_t kNoAllocMaxN = OCMP_NOALLOC_MAX_NDOF;      // 1,048,576 dofs
constexpr int64_t kNoAllocRed = int64_t(1) << 17;            // reduction partials
constexpr int64_t kNoAllocState = 256;                        // reduced values + scalars
constexpr int64_t kNoAllocDoubles = 5 * kNoAllocMaxN + kNoAllocRed + kNoAllocState;  // 41 MiB

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];
static __device__ __align__(256) int g_noalloc_flags[64];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[128] = {};
int* g_noalloc_fptr[128] = {};

// Device addresses of the scratch arrays for the current device. Host code must not use the
// arrays' names as pointers (they name host-side shadows); cudaGetSymbolAddress gives the device
// address. Done once per device, under a lock, with that device current.
int noalloc_scratch(double** scratch, int** flags) {
    int dev = 0;
    OCMP_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return fail(OCMP_ERR_ARG, "ocmp_solve_cg_noalloc: device index out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        double* p = nullptr;
        int* f = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        e = cudaGetSymbolAddress((void**)&f, g_noalloc_flags);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_flags)");
        g_noalloc_ptr[dev] = p;
        g_noalloc_fptr[dev] = f;
    }
    *scratch = g_noalloc_ptr[dev];
    *flags = g_noalloc_fptr[dev];
    return OCMP_OK;
}

}  // namespace

extern "C" int ocmp_solve_cg_noalloc(ocmp_matrix_t mat, const double* b, double* x, double tol, int32_t maxit,
                                     void* stream, ocmp_solve_info_t* info) {
    if (!mat || !b || !x) return fail(OCMP_ERR_ARG, "ocmp_solve_cg_noalloc: null argument");
    if (mat->B != 1) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solve_cg_noalloc: batched matrices are not supported");
    {
        // the solve reads its convergence flags on the host (stream synchronisation, device-to-host
        // copies); on a stream under capture those calls would invalidate the caller's capture
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        OCMP_CUDA(cudaStreamIsCapturing((cudaStream_t)stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(OCMP_ERR_UNSUPPORTED, "ocmp_solve_cg_noalloc: the stream is being captured; the solve "
                                              "synchronises with the host and cannot run under capture");
    }
    ocmp_space_s* s = mat->space;
    const int64_t n = s->ndof;
    if (n > kNoAllocMaxN)
        return fail(OCMP_ERR_ARG, "ocmp_solve_cg_noalloc: " + std::to_string(n) + " dofs exceed the " +
                                      std::to_string(kNoAllocMaxN) + "-dof limit of its static workspace");
    const int tpr = pick_tpr(s);
    if ((n * tpr + kThreads - 1) / kThreads > kNoAllocRed)
        return fail(OCMP_ERR_ARG, "ocmp_solve_cg_noalloc: SpMV partials exceed the static workspace");
    double* scr = nullptr;
    int* flg = nullptr;
    int st = noalloc_scratch(&scr, &flg);
    if (st) return st;
    // A solver view over the static workspace: nothing here touches the allocator.
    ocmp_solver_s sv;
    sv.mat = mat;
    sv.s = s;
    sv.prm.method = OCMP_CG;
    sv.prm.precond = OCMP_PRE_JACOBI;
    sv.prm.precision = OCMP_FP64;
    sv.prm.tol = tol;
    sv.prm.maxit = maxit;
    sv.prm.check_every = 8;
    sv.n = n;
    sv.m = 1;
    sv.nb = (int)std::max<int64_t>(1, std::min<int64_t>(1216, (n + 1023) / 1024));
    sv.dinv = scr;
    sv.r = scr + n;
    sv.z = scr + 2 * n;
    sv.p = scr + 3 * n;
    sv.w = scr + 4 * n;
    double* tail = scr + 5 * kNoAllocMaxN;
    sv.pspmv = tail;
    sv.part = tail;  // CG partials (2 x nb) never overlap a live SpMV partial
    sv.red = tail + kNoAllocRed;
    sv.st = sv.red + 64;
    sv.flags = flg;
    int hflags[F_NFLAG] = {0};
    sv.hflags = hflags;
    Ctx c;
    c.sv = &sv;
    c.st = (cudaStream_t)stream;
    c.tpr = tpr;
    c.grid = sv.nb;
    // the workspace keeps the previous call's contents: reset the flags and scalars
    OCMP_CUDA(cudaMemsetAsync(flg, 0, sizeof(int) * 64, c.st));
    OCMP_CUDA(cudaMemsetAsync(sv.red, 0, sizeof(double) * kNoAllocState, c.st));
    OCMP_LAUNCH(jacobi_setup<double><<<nblk(n, kThreads), kThreads, 0, c.st>>>(n, s->d_diag, mat->vals, s->d_free, sv.dinv));
    st = rhs_norm(c, b, x);
    if (st) return st;
    st = residual64(c, b, x, sv.r);
    if (st) return st;
    double red0 = 0, nbv = 1;
    OCMP_CUDA(cudaMemcpyAsync(&red0, sv.red, sizeof(double), cudaMemcpyDeviceToHost, c.st));
    OCMP_CUDA(cudaMemcpyAsync(&nbv, sv.st + S_NB, sizeof(double), cudaMemcpyDeviceToHost, c.st));
    OCMP_CUDA(cudaStreamSynchronize(c.st));
    const double relres0 = std::sqrt(std::max(red0, 0.0)) / nbv;
    int iters = 0;
    bool nonfin = !std::isfinite(relres0), brk = false;
    if (!nonfin && relres0 > tol) {
        st = cg_core<double, double, double>(c, mat->vals, sv.dinv, sv.r, sv.z, sv.p, sv.w, x, maxit, tol, &iters);
        if (st) return st;
        nonfin = hflags[F_NONFIN] != 0;
        brk = hflags[F_BREAK] != 0;
    }
    st = residual64(c, b, x, (double*)nullptr);
    if (st) return st;
    OCMP_CUDA(cudaMemcpyAsync(&red0, sv.red, sizeof(double), cudaMemcpyDeviceToHost, c.st));
    OCMP_CUDA(cudaStreamSynchronize(c.st));
    const double relres = std::sqrt(std::max(red0, 0.0)) / nbv;
    int status = OCMP_OK;
    if (nonfin || !std::isfinite(relres)) status = OCMP_ERR_NONFINITE;
    else if (relres > tol) status = brk ? OCMP_BREAKDOWN : OCMP_NOT_CONVERGED;
    if (info) {
        info->status = status;
        info->iterations = iters;
        info->outer_iterations = 0;
        info->relres0 = relres0;
        info->relres = relres;
    }
    if (status != OCMP_OK) set_error("ocmp_solve_cg_noalloc: did not reach the tolerance (status " +
                                     std::to_string(status) + ")");
    return status;
}
