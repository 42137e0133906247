// Taylor-Hood velocity/pressure system of OpenCMP's incompressible Navier-Stokes model
// (opencmp/models/ins.py) on triangles: velocity H1 order k per component, pressure H1 order k-1,
// compound vector [u_x (n_u) | u_y (n_u) | p (n_p)].
//
// Bilinear form (ins.py:178-251 with the time-derivative mass term of base_model.py:418-497):
//   mass (u, v) + dt nu (grad u, grad v) - dt (u (x) w, grad v) - dt (div u, q) - dt (div v, p)
//   - dt eps_p (p, q)
// Linear form (ins.py:253-314): dt (f, v) + mass (u_prev, v) - dt ((grad u^n) u^n, v) [IMEX].
//
// Assembly: one thread per element writes the element's blocks in structure-of-arrays order
// (entry l of element e at Ke[l * ne + e]: coalesced across the warp) - K_uu (k_u x k_u, shared by
// both velocity components), B_x, B_y (pressure rows x velocity columns) and K_pp - from reference
// tensors contracted with the element's inverse Jacobian; the Oseen convection term is a quadrature
// sum with the wind evaluated at the points. A gather kernel then sums, for each CSR entry, its
// contributions in a fixed order (a per-entry list built once on the host), so the values are
// deterministic without atomics.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "ocmp_internal.h"

namespace ocmp {
namespace {

inline unsigned nblk_s(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct ThTabs {
    const double* M;    // Lu*Lu      int phi_i phi_j              (reference element)
    const double* S;    // 3*Lu*Lu    int d0phi_i d0phi_j, (d0 d1 + d1 d0), d1 d1
    const double* T;    // 2*Lp*Lu    int psi_i d_d phi_j
    const double* Mp;   // Lp*Lp      int psi_i psi_j
    const double* R;    // nq*2*Lu*Lu w_q d_d phi_i(x_q) phi_j(x_q)
    const double* phi;  // nq*Lu
    const double* gref; // nq*Lu*2
    const double* psi;  // nq*Lp
    const double* qw;   // nq
};

struct ThGeo {
    double adet, Ji[2][2];  // Ji[c][r] = d xi_c / d x_r
};

__device__ __forceinline__ void th_geo(const double* __restrict__ X, const int32_t* __restrict__ conn, int64_t e,
                                       ThGeo& g, double x0[2]) {
    const int32_t a = conn[3 * e], b = conn[3 * e + 1], c = conn[3 * e + 2];
    x0[0] = X[2 * a];
    x0[1] = X[2 * a + 1];
    const double j00 = X[2 * b] - x0[0], j10 = X[2 * b + 1] - x0[1];
    const double j01 = X[2 * c] - x0[0], j11 = X[2 * c + 1] - x0[1];
    const double det = j00 * j11 - j01 * j10;
    const double id = 1.0 / det;
    g.adet = fabs(det);
    g.Ji[0][0] = j11 * id;
    g.Ji[0][1] = -j01 * id;
    g.Ji[1][0] = -j10 * id;
    g.Ji[1][1] = j00 * id;
}

template <int LU, int LP, int NQ>
__global__ void __launch_bounds__(128) th_elem_kernel(int64_t ne, const double* __restrict__ X,
                                                      const int32_t* __restrict__ conn,
                                                      const int32_t* __restrict__ vdofs, ThTabs t, double mass,
                                                      double nu, double dt, double tcoef, double eps_p,
                                                      const double* __restrict__ wind, int64_t nu_dofs,
                                                      double* __restrict__ Ke) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    ThGeo g;
    double x0[2];
    th_geo(X, conn, e, g, x0);
    const double G00 = g.Ji[0][0] * g.Ji[0][0] + g.Ji[0][1] * g.Ji[0][1];
    const double G01 = g.Ji[0][0] * g.Ji[1][0] + g.Ji[0][1] * g.Ji[1][1];
    const double G11 = g.Ji[1][0] * g.Ji[1][0] + g.Ji[1][1] * g.Ji[1][1];
    const double sm = mass * g.adet, sk = dt * nu * g.adet;
    // Oseen wind: a[q][d] = sum_r w_r(x_q) Ji[d][r] (the rule weight is folded into R)
    double a[NQ][2];
    const bool osn = wind != nullptr;
    if (osn) {
        double wx[LU], wy[LU];
#pragma unroll
        for (int j = 0; j < LU; j++) {
            const int32_t d = vdofs[e * LU + j];
            wx[j] = wind[d];
            wy[j] = wind[nu_dofs + d];
        }
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            double u0 = 0, u1 = 0;
#pragma unroll
            for (int j = 0; j < LU; j++) {
                const double p = __ldg(t.phi + q * LU + j);
                u0 += wx[j] * p;
                u1 += wy[j] * p;
            }
            a[q][0] = u0 * g.Ji[0][0] + u1 * g.Ji[0][1];
            a[q][1] = u0 * g.Ji[1][0] + u1 * g.Ji[1][1];
        }
    }
    const double sc = -dt * g.adet;
    // K_uu
#pragma unroll 1
    for (int ij = 0; ij < LU * LU; ij++) {
        double v = sm * __ldg(t.M + ij) +
                   sk * (G00 * __ldg(t.S + ij) + G01 * __ldg(t.S + LU * LU + ij) + G11 * __ldg(t.S + 2 * LU * LU + ij));
        if (osn) {
            double c = 0;
#pragma unroll
            for (int q = 0; q < NQ; q++)
                c += a[q][0] * __ldg(t.R + (q * 2) * LU * LU + ij) + a[q][1] * __ldg(t.R + (q * 2 + 1) * LU * LU + ij);
            v += sc * c;
        }
        Ke[ij * ne + e] = v;
    }
    // B_c(i, j) = -tcoef |det| sum_d Ji[d][c] T_d(i, j)
    const double sb = -tcoef * g.adet;
#pragma unroll 1
    for (int c = 0; c < 2; c++)
#pragma unroll 1
        for (int ij = 0; ij < LP * LU; ij++) {
            const double v = sb * (g.Ji[0][c] * __ldg(t.T + ij) + g.Ji[1][c] * __ldg(t.T + LP * LU + ij));
            Ke[(LU * LU + c * LP * LU + ij) * ne + e] = v;
        }
    const double sp = -tcoef * eps_p * g.adet;
#pragma unroll 1
    for (int ij = 0; ij < LP * LP; ij++) Ke[(LU * LU + 2 * LP * LU + ij) * ne + e] = sp * __ldg(t.Mp + ij);
}

// vals[k] = sum of the element entries listed for CSR entry k, in list order
__global__ void th_gather_kernel(int64_t nnz, const int32_t* __restrict__ seg, const int32_t* __restrict__ src,
                                 const double* __restrict__ Ke, double* __restrict__ vals) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    double acc = 0;
    for (int32_t s = seg[k]; s < seg[k + 1]; s++) acc += Ke[src[s]];
    vals[k] = acc;
}

// Element right-hand sides per velocity component: Fe[c][e*LU + i]
template <int LU, int NQ>
__global__ void __launch_bounds__(128) th_rhs_kernel(int64_t ne, const double* __restrict__ X,
                                                     const int32_t* __restrict__ conn,
                                                     const int32_t* __restrict__ vdofs, ThTabs t, double dt,
                                                     double f0, double f1, const double* __restrict__ fq,
                                                     double mass, const double* __restrict__ uprev,
                                                     const double* __restrict__ imex, double imex_coef,
                                                     int64_t nu_dofs, double* __restrict__ Fe) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    ThGeo g;
    double x0[2];
    th_geo(X, conn, e, g, x0);
    double up[2][LU], un[2][LU];
#pragma unroll
    for (int j = 0; j < LU; j++) {
        const int32_t d = vdofs[e * LU + j];
        up[0][j] = uprev ? uprev[d] : 0.0;
        up[1][j] = uprev ? uprev[nu_dofs + d] : 0.0;
        un[0][j] = imex ? imex[d] : 0.0;
        un[1][j] = imex ? imex[nu_dofs + d] : 0.0;
    }
    double F[2][LU];
#pragma unroll
    for (int i = 0; i < LU; i++) F[0][i] = F[1][i] = 0.0;
#pragma unroll 1
    for (int q = 0; q < NQ; q++) {
        double val[2];
        val[0] = dt * (fq ? fq[(e * NQ + q) * 2] : f0);
        val[1] = dt * (fq ? fq[(e * NQ + q) * 2 + 1] : f1);
        if (uprev) {
#pragma unroll
            for (int c = 0; c < 2; c++) {
                double s = 0;
#pragma unroll
                for (int j = 0; j < LU; j++) s += up[c][j] * __ldg(t.phi + q * LU + j);
                val[c] += mass * s;
            }
        }
        if (imex) {
            double u[2] = {0, 0}, gr[2][2] = {{0, 0}, {0, 0}};  // gr[c][d] = d u_c / d xi_d
#pragma unroll
            for (int j = 0; j < LU; j++) {
                const double p = __ldg(t.phi + q * LU + j);
                const double g0 = __ldg(t.gref + (q * LU + j) * 2), g1 = __ldg(t.gref + (q * LU + j) * 2 + 1);
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    u[c] += un[c][j] * p;
                    gr[c][0] += un[c][j] * g0;
                    gr[c][1] += un[c][j] * g1;
                }
            }
#pragma unroll
            for (int c = 0; c < 2; c++) {
                // (grad u) u: sum_r d u_c / d x_r u_r, d/dx_r = sum_d Ji[d][r] d/dxi_d
                double s = 0;
#pragma unroll
                for (int r = 0; r < 2; r++) s += (gr[c][0] * g.Ji[0][r] + gr[c][1] * g.Ji[1][r]) * u[r];
                val[c] -= imex_coef * dt * s;
            }
        }
        const double w = __ldg(t.qw + q) * g.adet;
#pragma unroll
        for (int i = 0; i < LU; i++) {
            const double p = w * __ldg(t.phi + q * LU + i);
            F[0][i] += p * val[0];
            F[1][i] += p * val[1];
        }
    }
#pragma unroll
    for (int i = 0; i < LU; i++) {
        Fe[e * LU + i] = F[0][i];
        Fe[ne * LU + e * LU + i] = F[1][i];
    }
}

__global__ void th_rhs_gather_kernel(int64_t nu_dofs, int64_t ndof, int64_t ne_lu, const int32_t* __restrict__ inc_ptr,
                                     const int32_t* __restrict__ inc, const double* __restrict__ Fe,
                                     double* __restrict__ b, int accumulate) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= ndof) return;
    if (r >= 2 * nu_dofs) {
        if (!accumulate) b[r] = 0.0;
        return;
    }
    const int c = r >= nu_dofs ? 1 : 0;
    const int64_t d = r - c * nu_dofs;
    const double* F = Fe + c * ne_lu;
    double acc = 0;
    for (int k = inc_ptr[d]; k < inc_ptr[d + 1]; k++) acc += F[inc[k]];
    b[r] = accumulate ? b[r] + acc : acc;
}

// Inverse block-diagonal preconditioner: velocity rows 1/a_ii; pressure rows
// -1/(sum_j a_ij^2 / a_jj + |a_ii|) over free velocity columns j; constrained rows 0.
__global__ void th_block_diag_kernel(int64_t nu_dofs, int64_t ndof, const int32_t* __restrict__ rp,
                                     const int32_t* __restrict__ col, const int32_t* __restrict__ diag,
                                     const uint8_t* __restrict__ freed, const double* __restrict__ vals,
                                     double* __restrict__ dinv) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= ndof) return;
    if (!freed[r]) {
        dinv[r] = 0.0;
        return;
    }
    const double arr = vals[diag[r]];
    if (r < 2 * nu_dofs) {
        dinv[r] = arr != 0.0 ? 1.0 / arr : 0.0;
        return;
    }
    double s = fabs(arr);
    for (int32_t k = rp[r]; k < rp[r + 1]; k++) {
        const int32_t c = col[k];
        if (c >= 2 * nu_dofs || !freed[c]) continue;
        const double ajj = vals[diag[c]];
        if (ajj != 0.0) s += vals[k] * vals[k] / fabs(ajj);
    }
    dinv[r] = s > 0.0 ? -1.0 / s : 0.0;
}

// per element: sum_q w |u_h - ref|^2 and sum_q w (div u_h)^2
template <int LU, int NQ>
__global__ void th_errors_kernel(int64_t ne, const double* __restrict__ X, const int32_t* __restrict__ conn,
                                 const int32_t* __restrict__ vdofs, ThTabs t, const double* __restrict__ u,
                                 int64_t nu_dofs, const double* __restrict__ ref, double* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    ThGeo g;
    double x0[2];
    th_geo(X, conn, e, g, x0);
    double ue[2][LU];
#pragma unroll
    for (int j = 0; j < LU; j++) {
        const int32_t d = vdofs[e * LU + j];
        ue[0][j] = u[d];
        ue[1][j] = u[nu_dofs + d];
    }
    double el = 0, ed = 0;
#pragma unroll 1
    for (int q = 0; q < NQ; q++) {
        double v[2] = {0, 0}, gr[2][2] = {{0, 0}, {0, 0}};
#pragma unroll
        for (int j = 0; j < LU; j++) {
            const double p = __ldg(t.phi + q * LU + j);
            const double g0 = __ldg(t.gref + (q * LU + j) * 2), g1 = __ldg(t.gref + (q * LU + j) * 2 + 1);
#pragma unroll
            for (int c = 0; c < 2; c++) {
                v[c] += ue[c][j] * p;
                gr[c][0] += ue[c][j] * g0;
                gr[c][1] += ue[c][j] * g1;
            }
        }
        const double w = __ldg(t.qw + q) * g.adet;
        const double d0 = v[0] - (ref ? ref[(e * NQ + q) * 2] : 0.0), d1 = v[1] - (ref ? ref[(e * NQ + q) * 2 + 1] : 0.0);
        el += w * (d0 * d0 + d1 * d1);
        // div u = d u_0 / d x_0 + d u_1 / d x_1
        const double dv = gr[0][0] * g.Ji[0][0] + gr[0][1] * g.Ji[1][0] + gr[1][0] * g.Ji[0][1] + gr[1][1] * g.Ji[1][1];
        ed += w * dv * dv;
    }
    out[2 * e] = el;
    out[2 * e + 1] = ed;
}

}  // namespace
}  // namespace ocmp

using namespace ocmp;

struct ocmp_th_s {
    ocmp_mesh_s* mesh = nullptr;
    int k = 2, Lu = 6, Lp = 3, nq = 0, ES = 0;
    ocmp_space_s* V = nullptr;
    ocmp_space_s* Q = nullptr;
    ocmp_space_s* C = nullptr;
    int64_t nu = 0, np = 0;
    std::vector<double> xq, wq;
    ThTabs tabs{};
    double* d_tab = nullptr;        // one buffer holding every table of `tabs`
    double* d_Ke = nullptr;         // ES * ne
    double* d_Fe = nullptr;         // 2 * ne * Lu
    int32_t* d_seg = nullptr;       // nnz + 1
    int32_t* d_src = nullptr;       // contributions
    double* d_err = nullptr;        // 2 * ne
};

namespace {

int th_build(ocmp_th_s* th) {
    ocmp_mesh_s* m = th->mesh;
    ocmp_space_s *V = th->V, *Q = th->Q;
    const int Lu = th->Lu, Lp = th->Lp, k = th->k;
    const int64_t ne = m->ne, nu = V->ndof, np = Q->ndof, nd = 2 * nu + np;
    th->nu = nu;
    th->np = np;
    th->ES = Lu * Lu + 2 * Lp * Lu + Lp * Lp;
    // ---- reference tables
    th->nq = quad_rule(2, k + 2, th->xq, th->wq);
    const int nq = th->nq;
    std::vector<double> phi(nq * Lu), gref(nq * Lu * 2), psi(nq * Lp), gpsi(nq * Lp * 2);
    tabulate(OCMP_H1, 2, k, nq, th->xq.data(), phi.data(), gref.data());
    tabulate(OCMP_H1, 2, k - 1, nq, th->xq.data(), psi.data(), gpsi.data());
    std::vector<double> M(Lu * Lu, 0.0), S(3 * Lu * Lu, 0.0), T(2 * Lp * Lu, 0.0), Mp(Lp * Lp, 0.0),
        R((size_t)nq * 2 * Lu * Lu, 0.0);
    for (int q = 0; q < nq; q++) {
        const double w = th->wq[q];
        for (int i = 0; i < Lu; i++)
            for (int j = 0; j < Lu; j++) {
                const double* gi = &gref[(q * Lu + i) * 2];
                const double* gj = &gref[(q * Lu + j) * 2];
                M[i * Lu + j] += w * phi[q * Lu + i] * phi[q * Lu + j];
                S[i * Lu + j] += w * gi[0] * gj[0];
                S[Lu * Lu + i * Lu + j] += w * (gi[0] * gj[1] + gi[1] * gj[0]);
                S[2 * Lu * Lu + i * Lu + j] += w * gi[1] * gj[1];
                for (int d = 0; d < 2; d++) R[((size_t)(q * 2 + d) * Lu + i) * Lu + j] = w * gi[d] * phi[q * Lu + j];
            }
        for (int i = 0; i < Lp; i++) {
            for (int j = 0; j < Lu; j++)
                for (int d = 0; d < 2; d++) T[(d * Lp + i) * Lu + j] += w * psi[q * Lp + i] * gref[(q * Lu + j) * 2 + d];
            for (int j = 0; j < Lp; j++) Mp[i * Lp + j] += w * psi[q * Lp + i] * psi[q * Lp + j];
        }
    }
    std::vector<double> all;
    std::vector<size_t> off;
    for (auto* v : {&M, &S, &T, &Mp, &R, &phi, &gref, &psi, &th->wq}) {
        off.push_back(all.size());
        all.insert(all.end(), v->begin(), v->end());
    }
    int st = upload(&th->d_tab, all.data(), all.size());
    if (st) return st;
    const double* b0 = th->d_tab;
    th->tabs = ThTabs{b0 + off[0], b0 + off[1], b0 + off[2], b0 + off[3], b0 + off[4],
                      b0 + off[5], b0 + off[6], b0 + off[7], b0 + off[8]};

    // ---- compound pattern: rows [u_x | u_y | p]
    const int32_t* vd = V->dofs.data();
    const int32_t* qd = Q->dofs.data();
    auto incidence = [&](const int32_t* dofs, int L, int64_t n, std::vector<int32_t>& ptr, std::vector<int32_t>& el) {
        ptr.assign(n + 1, 0);
        for (int64_t e = 0; e < ne; e++)
            for (int i = 0; i < L; i++) ptr[dofs[e * L + i] + 1]++;
        for (int64_t i = 0; i < n; i++) ptr[i + 1] += ptr[i];
        el.resize(ptr[n]);
        std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
        for (int64_t e = 0; e < ne; e++)
            for (int i = 0; i < L; i++) el[fill[dofs[e * L + i]]++] = (int32_t)e;
    };
    std::vector<int32_t> vptr, vel, qptr, qel;
    incidence(vd, Lu, nu, vptr, vel);
    incidence(qd, Lp, np, qptr, qel);
    std::vector<std::vector<int32_t>> vp(nu), qv(np);   // velocity row -> pressure cols; pressure row -> velocity cols
    for (int64_t d = 0; d < nu; d++) {
        auto& c = vp[d];
        for (int32_t s = vptr[d]; s < vptr[d + 1]; s++)
            for (int i = 0; i < Lp; i++) c.push_back(qd[(int64_t)vel[s] * Lp + i]);
        std::sort(c.begin(), c.end());
        c.erase(std::unique(c.begin(), c.end()), c.end());
    }
    for (int64_t d = 0; d < np; d++) {
        auto& c = qv[d];
        for (int32_t s = qptr[d]; s < qptr[d + 1]; s++)
            for (int i = 0; i < Lu; i++) c.push_back(vd[(int64_t)qel[s] * Lu + i]);
        std::sort(c.begin(), c.end());
        c.erase(std::unique(c.begin(), c.end()), c.end());
    }
    ocmp_space_s* C = th->C;
    C->rowptr.assign(nd + 1, 0);
    for (int comp = 0; comp < 2; comp++)
        for (int64_t d = 0; d < nu; d++)
            C->rowptr[comp * nu + d + 1] = (V->rowptr[d + 1] - V->rowptr[d]) + (int64_t)vp[d].size();
    for (int64_t d = 0; d < np; d++)
        C->rowptr[2 * nu + d + 1] = 2 * (int64_t)qv[d].size() + (Q->rowptr[d + 1] - Q->rowptr[d]);
    for (int64_t r = 0; r < nd; r++) C->rowptr[r + 1] += C->rowptr[r];
    const int64_t nnz = C->rowptr[nd];
    if (nnz >= (int64_t)INT32_MAX) return fail(OCMP_ERR_ARG, "ocmp_th_create: nnz too large for 32-bit indices");
    C->col.resize(nnz);
    for (int comp = 0; comp < 2; comp++)
        for (int64_t d = 0; d < nu; d++) {
            int64_t o = C->rowptr[comp * nu + d];
            for (int64_t s = V->rowptr[d]; s < V->rowptr[d + 1]; s++) C->col[o++] = (int32_t)(comp * nu + V->col[s]);
            for (int32_t c : vp[d]) C->col[o++] = (int32_t)(2 * nu + c);
        }
    for (int64_t d = 0; d < np; d++) {
        int64_t o = C->rowptr[2 * nu + d];
        for (int comp = 0; comp < 2; comp++)
            for (int32_t c : qv[d]) C->col[o++] = (int32_t)(comp * nu + c);
        for (int64_t s = Q->rowptr[d]; s < Q->rowptr[d + 1]; s++) C->col[o++] = (int32_t)(2 * nu + Q->col[s]);
    }
    C->ndof = nd;
    C->nnz = nnz;
    C->freed.assign(nd, 1);
    for (int64_t d = 0; d < nu; d++) C->freed[d] = C->freed[nu + d] = V->freed[d];
    int maxrow = 0;
    for (int64_t r = 0; r < nd; r++) maxrow = std::max(maxrow, (int)(C->rowptr[r + 1] - C->rowptr[r]));
    C->maxrow = maxrow;

    // ---- contribution lists: for each CSR entry, the element entries that sum into it
    auto pos = [&](int64_t r, int64_t c) -> int64_t {
        const int32_t* b = C->col.data() + C->rowptr[r];
        const int32_t* e = C->col.data() + C->rowptr[r + 1];
        const int32_t* it = std::lower_bound(b, e, (int32_t)c);
        return C->rowptr[r] + (it - b);
    };
    const int ES = th->ES;
    const int per = 2 * Lu * Lu + 4 * Lp * Lu + Lp * Lp;
    if ((int64_t)ES * ne >= (int64_t)INT32_MAX || (int64_t)per * ne >= (int64_t)INT32_MAX)
        return fail(OCMP_ERR_ARG, "ocmp_th_create: too many element entries for 32-bit indices");
    std::vector<int64_t> cpos((size_t)per * ne);
    std::vector<int32_t> csrc((size_t)per * ne);
    {
        size_t w = 0;
        for (int64_t e = 0; e < ne; e++) {
            const int32_t* dv = vd + e * Lu;
            const int32_t* dq = qd + e * Lp;
            for (int i = 0; i < Lu; i++)
                for (int j = 0; j < Lu; j++) {
                    const int32_t l = (int32_t)((int64_t)(i * Lu + j) * ne + e);
                    for (int comp = 0; comp < 2; comp++) {
                        cpos[w] = pos(comp * nu + dv[i], comp * nu + dv[j]);
                        csrc[w++] = l;
                    }
                }
            for (int comp = 0; comp < 2; comp++)
                for (int i = 0; i < Lp; i++)
                    for (int j = 0; j < Lu; j++) {
                        const int32_t l = (int32_t)((int64_t)(Lu * Lu + comp * Lp * Lu + i * Lu + j) * ne + e);
                        cpos[w] = pos(2 * nu + dq[i], comp * nu + dv[j]);      // B
                        csrc[w++] = l;
                        cpos[w] = pos(comp * nu + dv[j], 2 * nu + dq[i]);      // B^T
                        csrc[w++] = l;
                    }
            for (int i = 0; i < Lp; i++)
                for (int j = 0; j < Lp; j++) {
                    cpos[w] = pos(2 * nu + dq[i], 2 * nu + dq[j]);
                    csrc[w++] = (int32_t)((int64_t)(Lu * Lu + 2 * Lp * Lu + i * Lp + j) * ne + e);
                }
        }
    }
    std::vector<int32_t> seg(nnz + 1, 0), src(cpos.size());
    for (int64_t p : cpos) seg[p + 1]++;
    for (int64_t i = 0; i < nnz; i++) seg[i + 1] += seg[i];
    {
        std::vector<int32_t> fill(seg.begin(), seg.end() - 1);
        for (size_t s = 0; s < cpos.size(); s++) src[fill[cpos[s]]++] = csrc[s];
    }
    C->ncontrib = (int64_t)src.size();
    std::vector<int32_t> diag(nd), rp32(nd + 1);
    for (int64_t r = 0; r <= nd; r++) rp32[r] = (int32_t)C->rowptr[r];
    for (int64_t r = 0; r < nd; r++) diag[r] = (int32_t)pos(r, r);
    std::vector<int32_t> lift_ptr(nd + 1, 0), lift_pos;
    for (int64_t r = 0; r < nd; r++) {
        if (C->freed[r])
            for (int64_t q = C->rowptr[r]; q < C->rowptr[r + 1]; q++)
                if (!C->freed[C->col[q]]) lift_pos.push_back((int32_t)q);
        lift_ptr[r + 1] = (int32_t)lift_pos.size();
    }
    if ((st = upload(&C->d_rowptr, rp32.data(), rp32.size()))) return st;
    if ((st = upload(&C->d_col, C->col.data(), C->col.size()))) return st;
    if ((st = upload(&C->d_free, C->freed.data(), C->freed.size()))) return st;
    if ((st = upload(&C->d_diag, diag.data(), diag.size()))) return st;
    if ((st = upload(&C->d_lift_ptr, lift_ptr.data(), lift_ptr.size()))) return st;
    if ((st = upload(&C->d_lift_pos, lift_pos.data(), lift_pos.size()))) return st;
    if ((st = upload(&th->d_seg, seg.data(), seg.size()))) return st;
    if ((st = upload(&th->d_src, src.data(), src.size()))) return st;
    if ((st = dalloc(&th->d_Ke, (size_t)ES * ne))) return st;
    if ((st = dalloc(&th->d_Fe, (size_t)2 * ne * Lu))) return st;
    if ((st = dalloc(&th->d_err, (size_t)2 * ne))) return st;
    return OCMP_OK;
}

template <int LU, int LP, int NQ>
int th_assemble_impl(ocmp_th_s* th, ocmp_matrix_s* mat, const ocmp_th_form_t* f, cudaStream_t st) {
    const int64_t ne = th->mesh->ne;
    OCMP_LAUNCH(th_elem_kernel<LU, LP, NQ><<<nblk_s(ne, 128), 128, 0, st>>>(ne, th->mesh->dX, th->mesh->dconn, th->V->d_dofs,
                                                               th->tabs, f->mass, f->nu, f->dt, f->tcoef, f->eps_p, f->wind,
                                                               th->nu, th->d_Ke));
    OCMP_LAUNCH(th_gather_kernel<<<nblk_s(th->C->nnz, 256), 256, 0, st>>>(th->C->nnz, th->d_seg, th->d_src, th->d_Ke, mat->vals));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

template <int LU, int NQ>
int th_rhs_impl(ocmp_th_s* th, const ocmp_th_rhs_t* r, double* b, cudaStream_t st) {
    const int64_t ne = th->mesh->ne;
    OCMP_LAUNCH(th_rhs_kernel<LU, NQ><<<nblk_s(ne, 128), 128, 0, st>>>(ne, th->mesh->dX, th->mesh->dconn, th->V->d_dofs, th->tabs,
                                                          r->dt, r->src[0], r->src[1], r->src_qp, r->mass, r->uprev,
                                                          r->imex, r->imex_coef, th->nu, th->d_Fe));
    OCMP_LAUNCH(th_rhs_gather_kernel<<<nblk_s(th->C->ndof, 256), 256, 0, st>>>(th->nu, th->C->ndof, ne * LU, th->V->d_inc_ptr,
                                                                  th->V->d_inc, th->d_Fe, b, r->accumulate));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

template <int LU, int NQ>
int th_errors_impl(ocmp_th_s* th, const double* u, const double* ref, double* l2, double* dv, cudaStream_t st) {
    const int64_t ne = th->mesh->ne;
    OCMP_LAUNCH(th_errors_kernel<LU, NQ><<<nblk_s(ne, 128), 128, 0, st>>>(ne, th->mesh->dX, th->mesh->dconn, th->V->d_dofs,
                                                             th->tabs, u, th->nu, ref, th->d_err));
    std::vector<double> h(2 * ne);
    OCMP_CUDA(cudaMemcpyAsync(h.data(), th->d_err, sizeof(double) * 2 * ne, cudaMemcpyDeviceToHost, st));
    OCMP_CUDA(cudaStreamSynchronize(st));
    double a = 0, c = 0;
    for (int64_t e = 0; e < ne; e++) {
        a += h[2 * e];
        c += h[2 * e + 1];
    }
    *l2 = std::sqrt(a);
    *dv = std::sqrt(c);
    return OCMP_OK;
}

void th_free(ocmp_th_s* th) {
    if (th->C) ocmp_space_destroy(th->C);
    if (th->V) ocmp_space_destroy(th->V);
    if (th->Q) ocmp_space_destroy(th->Q);
    void* ps[] = {th->d_tab, th->d_Ke, th->d_Fe, th->d_seg, th->d_src, th->d_err};
    for (void* p : ps) dfree(p);
}

}  // namespace

extern "C" {

int ocmp_th_create(ocmp_mesh_t mesh, int32_t order_u, uint32_t dirichlet_mask, ocmp_th_t* out) {
    if (!mesh || !out) return fail(OCMP_ERR_ARG, "ocmp_th_create: null argument");
    if (mesh->dim != 2) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_th_create: Taylor-Hood is built for triangles");
    if (order_u != 2 && order_u != 3) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_th_create: velocity order 2 or 3");
    auto* th = new ocmp_th_s();
    th->mesh = mesh;
    th->k = order_u;
    th->Lu = (order_u + 1) * (order_u + 2) / 2;
    th->Lp = order_u * (order_u + 1) / 2;
    int st = ocmp_space_create(mesh, OCMP_H1, order_u, dirichlet_mask, &th->V);
    if (!st) st = ocmp_space_create(mesh, OCMP_H1, order_u - 1, 0, &th->Q);
    if (!st) {
        th->C = new ocmp_space_s();
        th->C->mesh = mesh;
        th->C->kind = OCMP_COMPOUND;
        th->C->order = order_u;
        th->C->dim = 2;
        th->C->nloc = 2 * th->Lu + th->Lp;
        th->C->dirichlet_mask = dirichlet_mask;
        st = th_build(th);
    }
    if (st) {
        th_free(th);
        delete th;
        return st;
    }
    *out = th;
    return OCMP_OK;
}

int ocmp_th_destroy(ocmp_th_t th) {
    if (!th) return OCMP_OK;
    th_free(th);
    delete th;
    return OCMP_OK;
}

int ocmp_th_spaces(ocmp_th_t th, ocmp_space_t* velocity, ocmp_space_t* pressure, ocmp_space_t* compound) {
    if (!th) return fail(OCMP_ERR_ARG, "ocmp_th_spaces: null argument");
    if (velocity) *velocity = th->V;
    if (pressure) *pressure = th->Q;
    if (compound) *compound = th->C;
    return OCMP_OK;
}

int ocmp_th_nq(ocmp_th_t th) { return th ? th->nq : 0; }

int ocmp_th_quad_points(ocmp_th_t th, double* xyz) {
    if (!th || !xyz) return fail(OCMP_ERR_ARG, "ocmp_th_quad_points: null argument");
    const ocmp_mesh_s* m = th->mesh;
    for (int64_t e = 0; e < m->ne; e++) {
        const int32_t* v = &m->conn[e * 3];
        for (int q = 0; q < th->nq; q++)
            for (int r = 0; r < 2; r++) {
                const double x0 = m->X[(int64_t)v[0] * 2 + r];
                xyz[(e * th->nq + q) * 2 + r] = x0 + (m->X[(int64_t)v[1] * 2 + r] - x0) * th->xq[q * 2] +
                                               (m->X[(int64_t)v[2] * 2 + r] - x0) * th->xq[q * 2 + 1];
            }
    }
    return OCMP_OK;
}

int ocmp_th_assemble(ocmp_th_t th, ocmp_matrix_t mat, const ocmp_th_form_t* f, void* stream) {
    if (!th || !mat || !f) return fail(OCMP_ERR_ARG, "ocmp_th_assemble: null argument");
    if (mat->space != th->C) return fail(OCMP_ERR_ARG, "ocmp_th_assemble: matrix not on the compound space");
    if (mat->B != 1 || mat->flags != 0)
        return fail(OCMP_ERR_UNSUPPORTED, "ocmp_th_assemble: plain FP64 matrices only (the solver keeps its own "
                                          "scaled FP32 copy)");
    cudaStream_t st = (cudaStream_t)stream;
    if (th->k == 2) return th_assemble_impl<6, 3, 16>(th, mat, f, st);
    return th_assemble_impl<10, 6, 25>(th, mat, f, st);
}

int ocmp_th_assemble_rhs(ocmp_th_t th, const ocmp_th_rhs_t* r, double* b, void* stream) {
    if (!th || !r || !b) return fail(OCMP_ERR_ARG, "ocmp_th_assemble_rhs: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (th->k == 2) return th_rhs_impl<6, 16>(th, r, b, st);
    return th_rhs_impl<10, 25>(th, r, b, st);
}

int ocmp_th_block_diag(ocmp_th_t th, ocmp_matrix_t mat, double* dinv, void* stream) {
    if (!th || !mat || !dinv) return fail(OCMP_ERR_ARG, "ocmp_th_block_diag: null argument");
    ocmp_space_s* C = th->C;
    OCMP_LAUNCH(th_block_diag_kernel<<<nblk_s(C->ndof, 256), 256, 0, (cudaStream_t)stream>>>(
        th->nu, C->ndof, C->d_rowptr, C->d_col, C->d_diag, C->d_free, mat->vals, dinv));
    OCMP_CUDA(cudaGetLastError());
    return OCMP_OK;
}

int ocmp_th_errors(ocmp_th_t th, const double* u, const double* ref_qp, double* l2, double* div, void* stream) {
    if (!th || !u || !l2 || !div) return fail(OCMP_ERR_ARG, "ocmp_th_errors: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (th->k == 2) return th_errors_impl<6, 16>(th, u, ref_qp, l2, div, st);
    return th_errors_impl<10, 25>(th, u, ref_qp, l2, div, st);
}

}  // extern "C"
