// Internal declarations shared by the host setup (ocmp_host.cpp) and the CUDA kernels (*.cu).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/opencmp_gpu.h"

namespace ocmp {

constexpr int kMaxLoc = 20;     // largest nloc built: H1 order 3 on tetrahedra
constexpr int kMaxNg = 27;      // element factors: 1 mass + 10 stiffness + 16 per-vertex wind (3D)
constexpr int kMaxFq = 25;      // facet quadrature points

// Kernels this library has launched (ocmp_launch_count); every launch site goes through OCMP_LAUNCH,
// and graph replays add the launches captured in the graph.
extern std::atomic<unsigned long long> g_launches;
#define OCMP_LAUNCH(...)                                                   \
    do {                                                                   \
        ::ocmp::g_launches.fetch_add(1, std::memory_order_relaxed);        \
        __VA_ARGS__;                                                       \
    } while (0)

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define OCMP_CUDA(call)                                         \
    do {                                                        \
        cudaError_t _e = (call);                                \
        if (_e != cudaSuccess) return ::ocmp::cuda_fail(_e, #call); \
    } while (0)

template <class T>
int dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    return OCMP_OK;
}
template <class T>
int upload(T** p, const T* h, size_t n) {
    int st = dalloc(p, n);
    if (st) return st;
    if (n) OCMP_CUDA(cudaMemcpy(*p, h, n * sizeof(T), cudaMemcpyHostToDevice));
    return OCMP_OK;
}
void dfree(void* p);

}  // namespace ocmp

struct ocmp_mesh_s {
    int dim = 0;
    int64_t nv = 0, ne = 0, nbf = 0;
    std::vector<double> X;          // nv*dim
    std::vector<int32_t> conn;      // ne*(dim+1), vertices ascending per element
    std::vector<int32_t> bfac;      // nbf*dim
    std::vector<int32_t> blab;      // nbf
    double* dX = nullptr;
    int32_t* dconn = nullptr;
};

// Reference-element tables of one space (host copies; device copies in ocmp_space_s).
struct ocmp_tables {
    int nloc = 0, nq = 0, nfq = 0, ng_const = 0, ng_vtx = 0;
    std::vector<double> R_const;    // ng_const * nloc^2 : mass, stiffness (k<=l), wind (k)
    std::vector<double> R_vtx;      // ng_vtx * nloc^2   : mass, stiffness, wind (k, vertex v)
    std::vector<double> qw;         // nq
    std::vector<double> qphi;       // nq * nloc  basis values at element quadrature points
    std::vector<double> qxi;        // nq * dim   reference quadrature points
    std::vector<double> mvec;       // nloc       integral of each basis function on the reference element
    std::vector<double> fw;         // nfq        facet rule weights (sum 1 in 2D, 1/2 in 3D)
    std::vector<double> fphi;       // (dim+1) * nfq * nloc       basis values on local facet f
    std::vector<double> fdphi;      // (dim+1) * nfq * nloc * dim reference gradients on local facet f
    std::vector<double> flam;       // (dim+1) * nfq * (dim+1)    barycentrics on local facet f
    // Sparse element-matrix terms in barycentric form (build_terms in ocmp_host.cpp), organised by
    // symmetric slot (i <= j): per slot, offsets into the term arrays of [mass | stiffness |
    // convection (i,j) | convection (j,i)]; one table for a constant wind, one for a per-vertex wind
    // (they differ only in the convection terms). K_ij = sym + conv_ij, K_ji = sym + conv_ji.
    int nsym = 0;
    std::vector<int32_t> slot_off[2];   // [wind variant] nsym * 5 offsets (+1 sentinel)
    std::vector<uint8_t> term_g[2];
    std::vector<double> term_coef[2];
    int nterms[2] = {0, 0};
};

struct ocmp_space_s {
    ocmp_mesh_s* mesh = nullptr;
    int kind = 0, order = 0, nloc = 0, dim = 0;
    uint32_t dirichlet_mask = 0;
    int64_t ndof = 0, nnz = 0, nif = 0, nbf = 0, ncontrib = 0;
    std::vector<int32_t> dofs;      // ne*nloc
    std::vector<int64_t> rowptr;    // ndof+1
    std::vector<int32_t> col;       // nnz
    std::vector<uint8_t> freed;     // ndof
    std::vector<int32_t> ifac;      // nif*4 : eL, fL, eR, fR
    std::vector<int32_t> bfac;      // nbf*3 : e, f, label  (only facets matched to an element)
    ocmp_tables T;
    // device
    int32_t* d_dofs = nullptr;
    int32_t* d_rowptr = nullptr;
    int32_t* d_col = nullptr;
    uint8_t* d_free = nullptr;
    int32_t* d_diag = nullptr;      // ndof: position of the diagonal entry in each row
    uint8_t* d_slot = nullptr;      // ne*nloc*slot_stride: column slot of dof(e,j) in row dof(e,i)
    uint8_t* d_fslot = nullptr;     // nif*2*nloc*2nloc: column slots of interior-facet matrix rows
    int32_t* d_efac_ptr = nullptr;  // ne+1: element -> interior facets (L2)
    int32_t* d_efac = nullptr;      // facet*2 + side
    int32_t* d_slot_off[2] = {nullptr, nullptr};
    uint8_t* d_term_g[2] = {nullptr, nullptr};
    double* d_term_coef[2] = {nullptr, nullptr};
    float2* d_term_coef_ff[2] = {nullptr, nullptr};  // the same coefficients as (hi, lo) float pairs
    int slot_stride = 0;            // bytes per (element, local row) in d_slot (nloc rounded to 16)
    int maxrow = 0;                 // longest CSR row
    int tuned_tpr = 0, tuned_u = 0; // SpMV row configuration chosen by ocmp_matrix_autotune (0: default)
    std::vector<int64_t> row_ranges;  // row ranges of similar length (vertex rows, the rest)
    std::vector<int> range_maxrow;
    int32_t* d_inc_ptr = nullptr;   // ndof+1: dof -> (element, local) incidence
    int32_t* d_inc = nullptr;       // ne*nloc: e*nloc + i
    int32_t* d_ifac = nullptr;
    int32_t* d_bfac = nullptr;
    int32_t* d_ebf_ptr = nullptr;   // ne+1: element -> boundary facets
    int32_t* d_ebf = nullptr;
    int32_t* d_lift_ptr = nullptr;  // ndof+1: per free row, CSR positions whose column is constrained
    int32_t* d_lift_pos = nullptr;
    int32_t* d_tpos = nullptr;      // nnz: position of the mirror entry (col, row), built on first use
    double* d_Rc = nullptr;         // R_const
    float2* d_Rm_ff = nullptr;      // reference mass matrix as (hi, lo) float pairs
    float2* d_geo_ff = nullptr;     // static element geometry for the double-float element kernel
    float2* d_Kd = nullptr;         // ne*nloc: element-matrix diagonals (double-float element kernel)
    float2* d_u2 = nullptr;         // ndof: a vector split into (hi, lo) float pairs (right-hand sides)
    int32_t* d_cseg = nullptr;      // nnz+1: per CSR entry, its run in d_csrc (built on first use)
    int32_t* d_csrc = nullptr;      // ne*nloc^2: element-matrix entries (e*nloc + i)*nloc + j per CSR entry,
                                    // in incidence order
    double* d_Rv = nullptr;         // R_vtx
    double* d_qw = nullptr;
    double* d_qphi = nullptr;
    double* d_mvec = nullptr;
    double* d_fw = nullptr;
    double* d_fphi = nullptr;
    double* d_fdphi = nullptr;
    double* d_flam = nullptr;
    // scratch owned by the space
    double* d_K = nullptr;          // ne*nloc^2 element matrices (FP64, or (hi, lo) float pairs)
    double* d_facetK = nullptr;     // nif*(2 nloc)^2 + nbf*nloc^2 facet matrices
    double* d_Fe = nullptr;         // ne*nloc element right-hand sides
    // SELL-32 layout of the pattern (built on first use by a matrix with OCMP_MAT_SELL32): slices of
    // 32 rows, each row padded to its slice's width in 4-entry chunks; entry (slice s, chunk c, row
    // lane l, e) at sell_off[s] + (c * 32 + l) * 4 + e
    int64_t sell_slices = 0, sell_nent = 0;
    int32_t* d_sell_off = nullptr;  // slices + 1
    int32_t* d_sell_col = nullptr;  // sell_nent columns (padding: the row itself, or 0 past the last row)
    int32_t* d_sell_pos = nullptr;  // nnz: the SELL position of each CSR entry
};

// Matrix outputs selected at creation (ocmp_matrix_create's flags): the FP64 values always; an FP32
// copy; the point-Jacobi right-scaled values A D^-1 in FP64 and/or FP32 (the Krylov matrices of
// the GMRES path) with D^-1 itself. The scaled outputs are written by the same assembly pass.
struct ocmp_matrix_s {
    ocmp_space_s* space = nullptr;
    int flags = 0;
    int B = 1;                      // instances (independent matrices on the same pattern)
    double* vals = nullptr;
    float* vals32 = nullptr;
    double* svals64 = nullptr;
    float* svals32 = nullptr;
    double* dinv = nullptr;
    float* dinv32 = nullptr;        // FP32 copy of D^-1 (double-float assembly with FP32 scaled output)
};

namespace ocmp {
// reference basis values/gradients (ocmp_host.cpp) and the collapsed simplex rule
int tabulate(int kind, int D, int p, int npts, const double* xi, double* val, double* grad);
int quad_rule(int D, int n, std::vector<double>& pts, std::vector<double>& wts);
// kernels (ocmp_assemble.cu)
int launch_assemble_matrix(ocmp_matrix_s* m, const ocmp_form_t* f, cudaStream_t st);
int launch_assemble_rhs(ocmp_space_s* s, const ocmp_form_t* f, const ocmp_rhs_t* r, double* b, cudaStream_t st);
int launch_set_boundary(ocmp_space_s* s, uint32_t mask, const double* gval, double* u, cudaStream_t st);
int launch_scatter_values(const std::vector<int32_t>& idx, const std::vector<double>& v, double* u, cudaStream_t st);
int launch_l2_error(ocmp_space_s* s, const double* u, const double* fq, double fconst, double* result, cudaStream_t st);
int launch_spmv64(const ocmp_space_s* s, const double* vals, const double* x, double* y, cudaStream_t st);
int launch_spmv_axpby(const ocmp_space_s* s, const double* vals, double alpha, const double* x, double beta, double* y,
                      cudaStream_t st);
// strip direct preconditioner (ocmp_strip.cu)
struct Strip;
int strip_create(const ocmp_space_s* s, Strip** out);
void strip_destroy(Strip* p);
int strip_factor(Strip* p, const ocmp_space_s* s, const double* vals, cudaStream_t st);
// z = M^-1 (sc v), sc = scale[j] (scale != null) or 1; z may alias v; kernels return at once when
// flags[0] (the solver's convergence flag) is set
template <class T>
int strip_apply(Strip* p, const ocmp_space_s* s, const double* vals, const T* v, const double* scale, int j, T* z,
                const int* flags, cudaStream_t st);
template <class T>
int strip_add(int64_t n, const T* z, double* x, cudaStream_t st);
void strip_stats(const Strip* p, ocmp_strip_stats_t* out);
void strip_set_timing(Strip* p, bool on);
void strip_set_gemm(Strip* p, int kind);
void strip_set_schulz(Strip* p, bool on);
// C = beta C + alpha A B^T on the tensor cores (ocmp_tcgemm.cu): FP32 operands, 3xTF32 products;
// M, N multiples of 128, K of 32; *err set when a bounded wait gave up
int tc_gemm_nt(int M, int N, int K, const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
               float alpha, float beta, int* err, cudaStream_t st);
int space_build_sell(ocmp_space_s* s);
int autotune_spmv(ocmp_space_s* s, const double* vals, const double* x, double* y, cudaStream_t st, int reps,
                  int* best_tpr, int* best_u, float* best_ms);
}  // namespace ocmp
