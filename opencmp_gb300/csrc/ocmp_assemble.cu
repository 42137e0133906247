// Assembly kernels of libopencmp_gpu.so (sm_103a).
//
// Matrix assembly is two launches (plus one for facet terms when the form has any):
//   1. elem_factors   one thread per element: Jacobian, |det J| and J^-1 in FP64, reduced to the
//                     ng geometric/coefficient factors F[g][e] of the element matrix
//                     K_e = sum_g F[g][e] R_g (R_g = reference-element tensors, exact quadrature);
//   2. scatter        one thread per CSR entry: walks its segment of the precomputed, sorted
//                     contribution list and sums F[.][e] . R[.][ij] for element entries and the
//                     precomputed facet-matrix entries for facet contributions. Every CSR value
//                     is written exactly once, in a fixed order: the result is bit-reproducible
//                     and needs no atomics and no zeroing pass.
// Facet matrices (DG skeleton terms, boundary terms) are computed by quadrature because their
// integrands (max(w.n, 0)) are not polynomial.
#include <cuda_runtime.h>

#include "ocmp_internal.h"

namespace ocmp {
namespace {

struct Geo {
    double Ji[3][3];
    double adet;
};

template <int D>
__device__ __forceinline__ void element_geo(const double* __restrict__ X, const int32_t* __restrict__ conn, int64_t e,
                                            Geo& g, double x0[3]) {
    double J[3][3];
    int32_t v0 = conn[e * (D + 1)];
#pragma unroll
    for (int r = 0; r < D; r++) x0[r] = X[(int64_t)v0 * D + r];
#pragma unroll
    for (int c = 0; c < D; c++) {
        int32_t vc = conn[e * (D + 1) + c + 1];
#pragma unroll
        for (int r = 0; r < D; r++) J[r][c] = X[(int64_t)vc * D + r] - x0[r];
    }
    if (D == 2) {
        double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        double id = 1.0 / det;
        g.Ji[0][0] = J[1][1] * id;
        g.Ji[0][1] = -J[0][1] * id;
        g.Ji[1][0] = -J[1][0] * id;
        g.Ji[1][1] = J[0][0] * id;
        g.adet = fabs(det);
    } else {
        double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        double id = 1.0 / det;
        g.Ji[0][0] = c00 * id;
        g.Ji[1][0] = c01 * id;
        g.Ji[2][0] = c02 * id;
        g.Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        g.Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        g.Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        g.Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        g.Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        g.Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
        g.adet = fabs(det);
    }
}

struct FormArgs {
    double mass, diff, dt, ipc, w0, w1, w2;
    const double* wind_vtx;
    int wind_kind;
    uint32_t outflow, wn, nitsche;
    int dg, order;
};

// F layout: g-major, F[g * ne + e].  g = 0 mass; 1..S stiffness (k <= l); then wind factors.
template <int D>
__global__ void elem_factors(int64_t ne, const double* __restrict__ X, const int32_t* __restrict__ conn,
                             FormArgs a, double* __restrict__ F) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    Geo g;
    double x0[3];
    element_geo<D>(X, conn, e, g, x0);
    int k = 0;
    F[(k++) * ne + e] = a.mass * g.adet;
    const double sd = a.dt * a.diff * g.adet;
#pragma unroll
    for (int r = 0; r < D; r++)
#pragma unroll
        for (int c = r; c < D; c++) {
            double m = 0;
#pragma unroll
            for (int t = 0; t < D; t++) m += g.Ji[r][t] * g.Ji[c][t];
            F[(k++) * ne + e] = sd * m;
        }
    const double sw = -a.dt * g.adet;
    if (a.wind_kind == OCMP_WIND_CONST) {
        const double w[3] = {a.w0, a.w1, a.w2};
#pragma unroll
        for (int r = 0; r < D; r++) {
            double t = 0;
#pragma unroll
            for (int c = 0; c < D; c++) t += g.Ji[r][c] * w[c];
            F[(k++) * ne + e] = sw * t;
        }
    } else if (a.wind_kind == OCMP_WIND_VERTEX) {
        double wv[D + 1][3];
#pragma unroll
        for (int v = 0; v <= D; v++) {
            int32_t gv = conn[e * (D + 1) + v];
#pragma unroll
            for (int c = 0; c < D; c++) wv[v][c] = a.wind_vtx[(int64_t)gv * D + c];
        }
#pragma unroll
        for (int r = 0; r < D; r++)
#pragma unroll
            for (int v = 0; v <= D; v++) {
                double t = 0;
#pragma unroll
                for (int c = 0; c < D; c++) t += g.Ji[r][c] * wv[v][c];
                F[(k++) * ne + e] = sw * t;
            }
    }
}

// Facet geometry on local facet lf of element e: outward unit normal, measure factor (length in
// 2D, |cross| = 2 area in 3D, matching rule weights that sum to 1 and 1/2).
template <int D>
__device__ __forceinline__ void facet_geo(const double* __restrict__ X, const int32_t* __restrict__ conn, int64_t e,
                                          int lf, double nrm[3], double& meas) {
    int fv[3], c = 0;
#pragma unroll
    for (int v = 0; v <= D; v++)
        if (v != lf) fv[c++] = conn[e * (D + 1) + v];
    int32_t vo = conn[e * (D + 1) + lf];
    const double* P0 = X + (int64_t)fv[0] * D;
    const double* P1 = X + (int64_t)fv[1] * D;
    const double* Po = X + (int64_t)vo * D;
    if (D == 2) {
        double tx = P1[0] - P0[0], ty = P1[1] - P0[1];
        double L = sqrt(tx * tx + ty * ty);
        nrm[0] = ty / L;
        nrm[1] = -tx / L;
        nrm[2] = 0;
        if ((Po[0] - P0[0]) * nrm[0] + (Po[1] - P0[1]) * nrm[1] > 0) {
            nrm[0] = -nrm[0];
            nrm[1] = -nrm[1];
        }
        meas = L;
    } else {
        const double* P2 = X + (int64_t)fv[2] * 3;
        double u[3], w[3], cr[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            u[k] = P1[k] - P0[k];
            w[k] = P2[k] - P0[k];
        }
        cr[0] = u[1] * w[2] - u[2] * w[1];
        cr[1] = u[2] * w[0] - u[0] * w[2];
        cr[2] = u[0] * w[1] - u[1] * w[0];
        double L = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        double dd = 0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            nrm[k] = cr[k] / L;
            dd += (Po[k] - P0[k]) * nrm[k];
        }
        if (dd > 0)
#pragma unroll
            for (int k = 0; k < 3; k++) nrm[k] = -nrm[k];
        meas = L;
    }
}

template <int D>
__device__ __forceinline__ double wind_dot_n(const FormArgs& a, const int32_t* __restrict__ conn, int64_t e,
                                             const double* __restrict__ lam, const double nrm[3]) {
    double w[3] = {0, 0, 0};
    if (a.wind_kind == OCMP_WIND_CONST) {
        w[0] = a.w0;
        w[1] = a.w1;
        w[2] = a.w2;
    } else if (a.wind_kind == OCMP_WIND_VERTEX) {
#pragma unroll
        for (int v = 0; v <= D; v++) {
            int32_t gv = conn[e * (D + 1) + v];
#pragma unroll
            for (int c = 0; c < D; c++) w[c] += lam[v] * a.wind_vtx[(int64_t)gv * D + c];
        }
    }
    double wn = 0;
#pragma unroll
    for (int c = 0; c < D; c++) wn += w[c] * nrm[c];
    return wn;
}

// Interior facets (SIPG + upwind, multi_component_ins.py:178-197 / poisson.py:103-121):
// one thread per (facet, test row i in [0, 2L)); writes row i of the 2L x 2L facet matrix.
template <int D, int L>
__global__ void interior_facet_kernel(int64_t nif, const double* __restrict__ X, const int32_t* __restrict__ conn,
                                      const int32_t* __restrict__ ifac, FormArgs a, int nfq,
                                      const double* __restrict__ fw, const double* __restrict__ fphi,
                                      const double* __restrict__ fdphi, const double* __restrict__ flam,
                                      double* __restrict__ K) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nif * 2 * L) return;
    const int64_t fi = t / (2 * L);
    const int i = (int)(t % (2 * L));
    const int64_t eL = ifac[4 * fi], eR = ifac[4 * fi + 2];
    const int fL = ifac[4 * fi + 1], fR = ifac[4 * fi + 3];
    Geo gL, gR;
    double x0[3];
    element_geo<D>(X, conn, eL, gL, x0);
    element_geo<D>(X, conn, eR, gR, x0);
    double nrm[3], meas;
    facet_geo<D>(X, conn, eL, fL, nrm, meas);
    const double h = D == 2 ? sqrt(gL.adet) : cbrt(gL.adet);
    const double alpha = a.ipc * a.order * a.order / h;
    double row[2 * L];
#pragma unroll
    for (int j = 0; j < 2 * L; j++) row[j] = 0;
    const bool iL = i < L;
    const int il = iL ? i : i - L;
    const Geo& gi = iL ? gL : gR;
    const int fi_loc = iL ? fL : fR;
    for (int q = 0; q < nfq; q++) {
        // test function i
        double vi = fphi[((size_t)fi_loc * nfq + q) * L + il];
        double dni = 0;
#pragma unroll
        for (int r = 0; r < D; r++) {
            double gr = 0;
#pragma unroll
            for (int c = 0; c < D; c++) gr += gi.Ji[c][r] * fdphi[(((size_t)fi_loc * nfq + q) * L + il) * D + c];
            dni += gr * nrm[r];
        }
        const double jv = iL ? vi : -vi;
        const double avn = 0.5 * dni;
        const double wn = wind_dot_n<D>(a, conn, eL, flam + ((size_t)fL * nfq + q) * (D + 1), nrm);
        const double wq = fw[q] * meas * a.dt;
#pragma unroll
        for (int j = 0; j < 2 * L; j++) {
            const bool jL = j < L;
            const int jl = jL ? j : j - L;
            const int fj = jL ? fL : fR;
            const Geo& gj = jL ? gL : gR;
            double vj = fphi[((size_t)fj * nfq + q) * L + jl];
            double dnj = 0;
#pragma unroll
            for (int r = 0; r < D; r++) {
                double gr = 0;
#pragma unroll
                for (int c = 0; c < D; c++) gr += gj.Ji[c][r] * fdphi[(((size_t)fj * nfq + q) * L + jl) * D + c];
                dnj += gr * nrm[r];
            }
            const double ju = jL ? vj : -vj;
            const double aun = 0.5 * dnj;
            double tt = a.diff * (alpha * ju * jv - aun * jv - avn * ju);
            tt += jv * (jL ? vj * fmax(wn, 0.0) : vj * fmin(wn, 0.0));
            row[j] += wq * tt;
        }
    }
    double* out = K + fi * 4 * L * L + (int64_t)i * 2 * L;
#pragma unroll
    for (int j = 0; j < 2 * L; j++) out[j] = row[j];
}

// Boundary facets: outflow upwind, (w.n) Neumann half, DG Nitsche (multi_component_ins.py:254-301,
// poisson.py:83-91); one thread per (facet, test row).
template <int D, int L>
__global__ void boundary_facet_kernel(int64_t nbf, const double* __restrict__ X, const int32_t* __restrict__ conn,
                                      const int32_t* __restrict__ bfac, FormArgs a, int is_l2, int nfq,
                                      const double* __restrict__ fw, const double* __restrict__ fphi,
                                      const double* __restrict__ fdphi, const double* __restrict__ flam,
                                      double* __restrict__ K) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nbf * L) return;
    const int64_t b = t / L;
    const int i = (int)(t % L);
    const int64_t e = bfac[3 * b];
    const int lf = bfac[3 * b + 1], lab = bfac[3 * b + 2];
    double row[L];
#pragma unroll
    for (int j = 0; j < L; j++) row[j] = 0;
    const uint32_t bit = (lab >= 0 && lab < 32) ? (1u << lab) : 0u;
    const bool has_out = a.outflow & bit, has_wn = a.wn & bit, has_nit = is_l2 && (a.nitsche & bit);
    if (has_out || has_wn || has_nit) {
        Geo g;
        double x0[3];
        element_geo<D>(X, conn, e, g, x0);
        double nrm[3], meas;
        facet_geo<D>(X, conn, e, lf, nrm, meas);
        const double h = D == 2 ? sqrt(g.adet) : cbrt(g.adet);
        const double alpha = a.ipc * a.order * a.order / h;
        for (int q = 0; q < nfq; q++) {
            const size_t base = ((size_t)lf * nfq + q) * L;
            const double vi = fphi[base + i];
            double dni = 0;
#pragma unroll
            for (int r = 0; r < D; r++) {
                double gr = 0;
#pragma unroll
                for (int c = 0; c < D; c++) gr += g.Ji[c][r] * fdphi[(base + i) * D + c];
                dni += gr * nrm[r];
            }
            const double wn = wind_dot_n<D>(a, conn, e, flam + ((size_t)lf * nfq + q) * (D + 1), nrm);
            const double wq = fw[q] * meas * a.dt;
#pragma unroll
            for (int j = 0; j < L; j++) {
                const double vj = fphi[base + j];
                double dnj = 0;
#pragma unroll
                for (int r = 0; r < D; r++) {
                    double gr = 0;
#pragma unroll
                    for (int c = 0; c < D; c++) gr += g.Ji[c][r] * fdphi[(base + j) * D + c];
                    dnj += gr * nrm[r];
                }
                double tt = 0;
                if (has_out) tt += vi * vj * fmax(wn, 0.0);
                if (has_wn) tt += vi * vj * wn;
                if (has_nit) tt += a.diff * (alpha * vi * vj - vi * dnj - vj * dni) + vi * vj * fmax(wn, 0.0);
                row[j] += wq * tt;
            }
        }
    }
    double* out = K + b * L * L + (int64_t)i * L;
#pragma unroll
    for (int j = 0; j < L; j++) out[j] = row[j];
}

// The sorted segmented reduction. R (ng x L^2) is staged in shared memory.
template <int L>
__global__ void __launch_bounds__(256) scatter_kernel(int64_t nnz, int64_t ne, int ng, const uint32_t* __restrict__ seg,
                                                      const uint32_t* __restrict__ contrib,
                                                      const double* __restrict__ F, const double* __restrict__ R,
                                                      const double* __restrict__ facetK, uint64_t E, int use_facets,
                                                      double* __restrict__ vals, float* __restrict__ vals32) {
    extern __shared__ double sR[];
    for (int k = threadIdx.x; k < ng * L * L; k += blockDim.x) sR[k] = R[k];
    __syncthreads();
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= nnz) return;
    const uint32_t c0 = seg[p], c1 = seg[p + 1];
    double acc = 0.0;
    for (uint32_t c = c0; c < c1; c++) {
        const uint32_t id = __ldg(contrib + c);
        if (id < E) {
            const uint32_t e = id / (L * L), ij = id - e * (L * L);
            double v = 0.0;
            for (int g = 0; g < ng; g++) v += __ldg(F + (int64_t)g * ne + e) * sR[g * L * L + ij];
            acc += v;
        } else if (use_facets) {
            acc += __ldg(facetK + (id - E));
        }
    }
    vals[p] = acc;
    if (vals32) vals32[p] = (float)acc;
}

// Element right-hand sides: dt (f, phi_i) + mass (u_prev, phi_i) + boundary data.
template <int D, int L>
__global__ void rhs_elem_kernel(int64_t ne, const double* __restrict__ X, const int32_t* __restrict__ conn,
                                const int32_t* __restrict__ dofs, FormArgs a, double dt, int src_kind, double src_const,
                                const double* __restrict__ src_qp, double mass, const double* __restrict__ uprev,
                                int nq, const double* __restrict__ qw, const double* __restrict__ qphi,
                                const double* __restrict__ mvec, const double* __restrict__ Rm,
                                const int32_t* __restrict__ ebf_ptr, const int32_t* __restrict__ ebf,
                                const int32_t* __restrict__ bfac, const double* __restrict__ bval, uint32_t bval_mask,
                                const double* __restrict__ gval, int is_l2, int nfq, const double* __restrict__ fw,
                                const double* __restrict__ fphi, const double* __restrict__ fdphi,
                                const double* __restrict__ flam, double* __restrict__ Fe) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    Geo g;
    double x0[3];
    element_geo<D>(X, conn, e, g, x0);
    double out[L];
#pragma unroll
    for (int i = 0; i < L; i++) out[i] = 0;
    if (src_kind == OCMP_SRC_CONST) {
#pragma unroll
        for (int i = 0; i < L; i++) out[i] = dt * src_const * g.adet * mvec[i];
    } else if (src_kind == OCMP_SRC_QP) {
        for (int q = 0; q < nq; q++) {
            const double fq = dt * src_qp[e * nq + q] * qw[q] * g.adet;
#pragma unroll
            for (int i = 0; i < L; i++) out[i] += fq * qphi[q * L + i];
        }
    }
    if (uprev) {
        double u[L];
#pragma unroll
        for (int j = 0; j < L; j++) u[j] = uprev[dofs[e * L + j]];
        const double s = mass * g.adet;
#pragma unroll
        for (int i = 0; i < L; i++) {
            double acc = 0;
#pragma unroll
            for (int j = 0; j < L; j++) acc += Rm[i * L + j] * u[j];
            out[i] += s * acc;
        }
    }
    for (int k = ebf_ptr[e]; k < ebf_ptr[e + 1]; k++) {
        const int b = ebf[k];
        const int lf = bfac[3 * b + 1], lab = bfac[3 * b + 2];
        if (lab < 0 || lab >= 32) continue;
        const uint32_t bit = 1u << lab;
        const bool hb = bval_mask & bit, hg = is_l2 && (a.nitsche & bit);
        if (!hb && !hg) continue;
        double nrm[3], meas;
        facet_geo<D>(X, conn, e, lf, nrm, meas);
        const double h = D == 2 ? sqrt(g.adet) : cbrt(g.adet);
        const double alpha = a.ipc * a.order * a.order / h;
        for (int q = 0; q < nfq; q++) {
            const size_t base = ((size_t)lf * nfq + q) * L;
            const double wq = fw[q] * meas * dt;
            const double wn = hg ? wind_dot_n<D>(a, conn, e, flam + ((size_t)lf * nfq + q) * (D + 1), nrm) : 0.0;
#pragma unroll
            for (int i = 0; i < L; i++) {
                const double vi = fphi[base + i];
                double t = 0;
                if (hb) t += bval[lab] * vi;
                if (hg) {
                    double dni = 0;
#pragma unroll
                    for (int r = 0; r < D; r++) {
                        double gr = 0;
#pragma unroll
                        for (int c = 0; c < D; c++) gr += g.Ji[c][r] * fdphi[(base + i) * D + c];
                        dni += gr * nrm[r];
                    }
                    const double gv = gval[lab];
                    t += a.diff * gv * (alpha * vi - dni) - vi * gv * fmin(wn, 0.0);
                }
                out[i] += wq * t;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < L; i++) Fe[e * L + i] = out[i];
}

__global__ void rhs_gather_kernel(int64_t ndof, const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                  const double* __restrict__ Fe, double* __restrict__ b) {
    int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (d >= ndof) return;
    double acc = 0;
    for (int k = inc_ptr[d]; k < inc_ptr[d + 1]; k++) acc += Fe[inc[k]];
    b[d] = acc;
}

__global__ void set_values_kernel(int64_t n, const int32_t* __restrict__ idx, const double* __restrict__ v,
                                  double* __restrict__ u) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) u[idx[k]] = v[k];
}

// CSR SpMV, TPR threads per row (TPR in {2,4,8,16,32}), FP64 values and accumulation.
template <int TPR>
__global__ void __launch_bounds__(256) spmv64_kernel(int64_t n, const int32_t* __restrict__ rp,
                                                     const int32_t* __restrict__ col, const double* __restrict__ val,
                                                     const double* __restrict__ x, double* __restrict__ y) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t r = t / TPR;
    int lane = threadIdx.x % TPR;
    double acc = 0;
    if (r < n) {
        int32_t a = rp[r], b = rp[r + 1];
        for (int32_t k = a + lane; k < b; k += TPR) acc += __ldg(val + k) * __ldg(x + __ldg(col + k));
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, TPR);
    if (r < n && lane == 0) y[r] = acc;
}

FormArgs make_args(const ocmp_space_s* s, const ocmp_form_t* f) {
    FormArgs a;
    a.mass = f->mass;
    a.diff = f->diff;
    a.dt = f->dt;
    a.ipc = f->ipc;
    a.w0 = f->wind[0];
    a.w1 = f->wind[1];
    a.w2 = f->wind[2];
    a.wind_vtx = f->wind_vtx;
    a.wind_kind = f->wind_kind;
    a.outflow = f->outflow_mask;
    a.wn = f->wn_mask;
    a.nitsche = f->nitsche_mask;
    a.dg = f->dg;
    a.order = s->order;
    return a;
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

template <int D, int L>
int assemble_impl(ocmp_matrix_s* m, const ocmp_form_t* f, cudaStream_t st) {
    ocmp_space_s* s = m->space;
    const ocmp_mesh_s* mesh = s->mesh;
    const int64_t ne = mesh->ne;
    FormArgs a = make_args(s, f);
    const int S = D * (D + 1) / 2;
    int ng = 1 + S;
    const double* R = s->d_Rc;
    if (f->wind_kind == OCMP_WIND_CONST) ng += D;
    if (f->wind_kind == OCMP_WIND_VERTEX) {
        ng += D * (D + 1);
        R = s->d_Rv;
    }
    elem_factors<D><<<nblk(ne, 128), 128, 0, st>>>(ne, mesh->dX, mesh->dconn, a, s->d_F);
    const bool is_l2 = s->kind == OCMP_L2;
    const bool interior = is_l2 && f->dg && s->nif > 0;
    const uint32_t bmask = f->outflow_mask | f->wn_mask | (is_l2 ? f->nitsche_mask : 0u);
    const bool boundary = bmask != 0 && s->nbf > 0;
    const bool use_facets = interior || boundary;
    if (use_facets) {
        double* Ki = s->d_facetK;
        double* Kb = s->d_facetK + s->nif * 4 * L * L;
        if (is_l2 && s->nif > 0) {
            if (interior)
                interior_facet_kernel<D, L><<<nblk(s->nif * 2 * L, 128), 128, 0, st>>>(
                    s->nif, mesh->dX, mesh->dconn, s->d_ifac, a, s->T.nfq, s->d_fw, s->d_fphi, s->d_fdphi, s->d_flam, Ki);
            else
                OCMP_CUDA(cudaMemsetAsync(Ki, 0, sizeof(double) * s->nif * 4 * L * L, st));
        }
        if (s->nbf > 0)
            boundary_facet_kernel<D, L><<<nblk(s->nbf * L, 128), 128, 0, st>>>(
                s->nbf, mesh->dX, mesh->dconn, s->d_bfac, a, is_l2, s->T.nfq, s->d_fw, s->d_fphi, s->d_fdphi,
                s->d_flam, Kb);
    }
    const size_t smem = sizeof(double) * ng * L * L;
    if (smem > 48 * 1024)
        OCMP_CUDA(cudaFuncSetAttribute(scatter_kernel<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    scatter_kernel<L><<<nblk(s->nnz, 256), 256, smem, st>>>(s->nnz, ne, ng, s->d_seg, s->d_contrib, s->d_F, R,
                                                            s->d_facetK, s->elem_entries, use_facets ? 1 : 0, m->vals,
                                                            m->vals32);
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

template <int D, int L>
int rhs_impl(ocmp_space_s* s, const ocmp_form_t* f, const ocmp_rhs_t* r, double* b, cudaStream_t st) {
    const ocmp_mesh_s* mesh = s->mesh;
    const int64_t ne = mesh->ne;
    FormArgs a = make_args(s, f);
    // per-label data travels by value through a small device buffer owned by the call's stream
    double* dvals = nullptr;
    OCMP_CUDA(cudaMallocAsync((void**)&dvals, sizeof(double) * 64, st));
    double hv[64];
    for (int k = 0; k < 32; k++) {
        hv[k] = r->bval[k];
        hv[32 + k] = r->gval[k];
    }
    OCMP_CUDA(cudaMemcpyAsync(dvals, hv, sizeof(hv), cudaMemcpyHostToDevice, st));
    rhs_elem_kernel<D, L><<<nblk(ne, 128), 128, 0, st>>>(
        ne, mesh->dX, mesh->dconn, s->d_dofs, a, r->dt, r->src_kind, r->src_const, r->src_qp, r->mass, r->uprev,
        s->T.nq, s->d_qw, s->d_qphi, s->d_mvec, s->d_Rc, s->d_ebf_ptr, s->d_ebf, s->d_bfac, dvals, r->bval_mask,
        dvals + 32, s->kind == OCMP_L2, s->T.nfq, s->d_fw, s->d_fphi, s->d_fdphi, s->d_flam, s->d_Fe);
    rhs_gather_kernel<<<nblk(s->ndof, 256), 256, 0, st>>>(s->ndof, s->d_inc_ptr, s->d_inc, s->d_Fe, b);
    OCMP_CUDA(cudaFreeAsync(dvals, st));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

}  // namespace

#define OCMP_DISPATCH(FN, ...)                                                   \
    do {                                                                         \
        const int D_ = s->dim, L_ = s->nloc;                                     \
        if (D_ == 2 && L_ == 3) return FN<2, 3>(__VA_ARGS__);                    \
        if (D_ == 2 && L_ == 6) return FN<2, 6>(__VA_ARGS__);                    \
        if (D_ == 2 && L_ == 10) return FN<2, 10>(__VA_ARGS__);                  \
        if (D_ == 3 && L_ == 4) return FN<3, 4>(__VA_ARGS__);                    \
        if (D_ == 3 && L_ == 10) return FN<3, 10>(__VA_ARGS__);                  \
        if (D_ == 3 && L_ == 20) return FN<3, 20>(__VA_ARGS__);                  \
        return fail(OCMP_ERR_UNSUPPORTED, "no kernel built for this element");   \
    } while (0)

int launch_assemble_matrix(ocmp_matrix_s* m, const ocmp_form_t* f, cudaStream_t st) {
    ocmp_space_s* s = m->space;
    OCMP_DISPATCH(assemble_impl, m, f, st);
}

int launch_assemble_rhs(ocmp_space_s* s, const ocmp_form_t* f, const ocmp_rhs_t* r, double* b, cudaStream_t st) {
    OCMP_DISPATCH(rhs_impl, s, f, r, b, st);
}

// Dirichlet values (base_model.py:321-341): vertex dofs of every facet with a label in `mask` take
// the label's constant g; the higher-order dofs on those facets are set to 0 (exact for data that
// is linear along each facet). Where facets of different labels share a dof, the facet that comes
// last in the mesh's boundary list wins. The owner table is built on the host.
int launch_set_boundary(ocmp_space_s* s, uint32_t mask, const double* gval, double* u, cudaStream_t st) {
    if (s->kind != OCMP_H1) return OCMP_OK;
    const int D = s->dim, nvp = D + 1, L = s->nloc, p = s->order;
    std::vector<int32_t> owner(s->ndof, -1);
    std::vector<double> val(s->ndof, 0.0);
    for (int64_t b = 0; b < s->nbf; b++) {
        const int lab = s->bfac[3 * b + 2];
        if (lab < 0 || lab >= 32 || !((mask >> lab) & 1u)) continue;
        const int64_t e = s->bfac[3 * b];
        const int f = s->bfac[3 * b + 1];
        const int32_t* d = &s->dofs[e * L];
        int c = 0;
        for (int a = 0; a < nvp; a++, c++)
            if (a != f) {
                owner[d[c]] = 1;
                val[d[c]] = gval[lab];
            }
        if (p >= 2)
            for (int a = 0; a < nvp; a++)
                for (int bb = a + 1; bb < nvp; bb++)
                    for (int k = 0; k < p - 1; k++, c++)
                        if (a != f && bb != f) {
                            owner[d[c]] = 1;
                            val[d[c]] = 0.0;
                        }
        if (p >= 3)
            for (int a = 0; a < nvp; a++)
                for (int bb = a + 1; bb < nvp; bb++)
                    for (int cc = bb + 1; cc < nvp; cc++, c++)
                        if (a != f && bb != f && cc != f) {
                            owner[d[c]] = 1;
                            val[d[c]] = 0.0;
                        }
    }
    std::vector<int32_t> idx;
    std::vector<double> v;
    for (int64_t i = 0; i < s->ndof; i++)
        if (owner[i] >= 0) {
            idx.push_back((int32_t)i);
            v.push_back(val[i]);
        }
    if (idx.empty()) return OCMP_OK;
    int32_t* didx = nullptr;
    double* dv = nullptr;
    OCMP_CUDA(cudaMallocAsync((void**)&didx, idx.size() * sizeof(int32_t), st));
    OCMP_CUDA(cudaMallocAsync((void**)&dv, v.size() * sizeof(double), st));
    OCMP_CUDA(cudaMemcpyAsync(didx, idx.data(), idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    OCMP_CUDA(cudaMemcpyAsync(dv, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    set_values_kernel<<<nblk((int64_t)idx.size(), 256), 256, 0, st>>>((int64_t)idx.size(), didx, dv, u);
    OCMP_CUDA(cudaFreeAsync(didx, st));
    OCMP_CUDA(cudaFreeAsync(dv, st));
    // the host vectors must outlive the async copies
    OCMP_CUDA(cudaStreamSynchronize(st));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int launch_spmv64(const ocmp_space_s* s, const double* vals, const double* x, double* y, cudaStream_t st) {
    const double avg = (double)s->nnz / (double)s->ndof;
    const int64_t n = s->ndof;
    if (avg <= 6)
        spmv64_kernel<2><<<nblk(n * 2, 256), 256, 0, st>>>(n, s->d_rowptr, s->d_col, vals, x, y);
    else if (avg <= 14)
        spmv64_kernel<4><<<nblk(n * 4, 256), 256, 0, st>>>(n, s->d_rowptr, s->d_col, vals, x, y);
    else if (avg <= 40)
        spmv64_kernel<8><<<nblk(n * 8, 256), 256, 0, st>>>(n, s->d_rowptr, s->d_col, vals, x, y);
    else
        spmv64_kernel<16><<<nblk(n * 16, 256), 256, 0, st>>>(n, s->d_rowptr, s->d_col, vals, x, y);
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

}  // namespace ocmp
