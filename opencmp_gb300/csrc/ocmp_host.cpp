// Host side of libopencmp_gpu.so: handles, error reporting, and the one-off set-up of each space
// (DOF numbering, CSR pattern, sorted scatter plan, reference-element tables), uploaded once to
// HBM. Everything per time step runs on the GPU (ocmp_assemble.cu, ocmp_krylov.cu).
//
// Space conventions (the documented numbering this library and its CPU oracle share):
//  * element vertices are stored in ascending global order, so every edge/face is oriented from
//    its lower to its higher global vertex in every element that shares it;
//  * H1 order p: dofs [0, nv) are the vertex functions lam_v; then p-1 functions per edge, edges
//    sorted by (lower, upper) vertex; then (p=3) one bubble per triangle face, faces sorted by
//    vertex triple; the local order is vertices, edges (a<b) lexicographic, faces (a<b<c);
//  * L2 order p (triangles): Dubiner basis, dof = element * nloc + local.
// NGSolve (opencmp/models/poisson.py:60-65) numbers vertex dofs first too, then edge, face and
// cell dofs; its edge enumeration comes from netgen and is not reproduced here.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <mutex>
#include <numeric>
#include <thread>

#include "ocmp_internal.h"

namespace ocmp {

std::atomic<unsigned long long> g_launches{0};
static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? OCMP_ERR_NOMEM : OCMP_ERR_CUDA;
}
void dfree(void* p) {
    if (p) cudaFree(p);
}

static void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)>& fn) {
    int nt = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 4096 || nt == 1) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> th;
    int64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        int64_t a = t * chunk, b = std::min(n, a + chunk);
        if (a >= b) break;
        th.emplace_back(fn, a, b);
    }
    for (auto& x : th) x.join();
}

// ---------------------------------------------------------------- reference basis (host)
struct Dn {
    double v, d[3];
};
static Dn dconst(double c) { return Dn{c, {0, 0, 0}}; }
static Dn operator+(Dn a, Dn b) { return Dn{a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}}; }
static Dn operator-(Dn a, Dn b) { return Dn{a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}}; }
static Dn operator*(Dn a, double s) { return Dn{a.v * s, {a.d[0] * s, a.d[1] * s, a.d[2] * s}}; }
static Dn operator*(Dn a, Dn b) {
    return Dn{a.v * b.v, {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1], a.d[2] * b.v + a.v * b.d[2]}};
}

// scaled Legendre L_k(x,t) = t^k P_k(x/t)
static void sleg(int n, Dn x, Dn t, Dn* out) {
    out[0] = dconst(1);
    if (n >= 1) out[1] = x;
    Dn t2 = t * t;
    for (int k = 1; k < n; k++) out[k + 1] = ((x * out[k]) * (2.0 * k + 1) - (t2 * out[k - 1]) * (double)k) * (1.0 / (k + 1));
}
// Jacobi P_j^{(a,0)}
static void jac(int n, double a, Dn s, Dn* out) {
    out[0] = dconst(1);
    if (n >= 1) out[1] = (s * (a + 2) + dconst(a)) * 0.5;
    for (int k = 2; k <= n; k++) {
        double A = 2.0 * k * (k + a) * (2.0 * k + a - 2);
        double B = 2.0 * k + a - 1;
        double C1 = (2.0 * k + a) * (2.0 * k + a - 2), C0 = a * a;
        double Dd = 2.0 * (k + a - 1) * (k - 1) * (2.0 * k + a);
        out[k] = (((s * C1 + dconst(C0)) * out[k - 1]) * B - out[k - 2] * Dd) * (1.0 / A);
    }
}

static int nloc_of(int kind, int D, int p) {
    (void)kind;
    return D == 2 ? (p + 1) * (p + 2) / 2 : (p + 1) * (p + 2) * (p + 3) / 6;
}

static void bary(int D, const double* xi, Dn* lam) {
    lam[0] = dconst(1);
    for (int k = 0; k < D; k++) {
        lam[0].v -= xi[k];
        lam[0].d[k] = -1;
        lam[k + 1] = dconst(xi[k]);
        lam[k + 1].d[k] = 1;
    }
}

static int basis(int kind, int D, int p, const double* xi, Dn* out) {
    Dn lam[4];
    bary(D, xi, lam);
    int c = 0;
    if (kind == OCMP_H1) {
        for (int v = 0; v <= D; v++) out[c++] = lam[v];
        if (p >= 2)
            for (int a = 0; a <= D; a++)
                for (int b = a + 1; b <= D; b++) {
                    Dn L[4];
                    sleg(p - 2, lam[b] - lam[a], lam[a] + lam[b], L);
                    Dn base = lam[a] * lam[b];
                    for (int k = 0; k <= p - 2; k++) out[c++] = base * L[k];
                }
        if (p >= 3)
            for (int a = 0; a <= D; a++)
                for (int b = a + 1; b <= D; b++)
                    for (int cc = b + 1; cc <= D; cc++) out[c++] = lam[a] * lam[b] * lam[cc];
    } else {
        Dn L[8];
        sleg(p, lam[1] - lam[0], lam[0] + lam[1], L);
        for (int i = 0; i <= p; i++) {
            Dn P[8];
            jac(p - i, 2.0 * i + 1, lam[2] * 2.0 - dconst(1), P);
            for (int j = 0; j <= p - i; j++) out[c++] = L[i] * P[j];
        }
    }
    return c;
}

// Gauss-Legendre on [0,1] and the collapsed simplex rule with n points per direction.
static void gauss01(int n, double* x, double* w) {
    for (int i = 0; i < n; i++) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1, p1 = 0;
            for (int k = 1; k <= n; k++) {
                double p2 = p1;
                p1 = p0;
                p0 = ((2.0 * k - 1) * z * p1 - (k - 1.0) * p2) / k;
            }
            pp = n * (z * p0 - p1) / (z * z - 1);
            double dz = p0 / pp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[i] = 0.5 * (1 - z);
        w[i] = 1.0 / ((1 - z * z) * pp * pp);
    }
}
static int simplex_rule(int D, int n, std::vector<double>& pts, std::vector<double>& wts) {
    double x[32], w[32];
    gauss01(n, x, w);
    pts.clear();
    wts.clear();
    if (D == 1) {
        for (int i = 0; i < n; i++) { pts.push_back(x[i]); wts.push_back(w[i]); }
    } else if (D == 2) {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                pts.push_back(x[i]);
                pts.push_back(x[j] * (1 - x[i]));
                wts.push_back(w[i] * w[j] * (1 - x[i]));
            }
    } else {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++) {
                    pts.push_back(x[i]);
                    pts.push_back(x[j] * (1 - x[i]));
                    pts.push_back(x[k] * (1 - x[i]) * (1 - x[j]));
                    wts.push_back(w[i] * w[j] * w[k] * (1 - x[i]) * (1 - x[i]) * (1 - x[j]));
                }
    }
    return (int)wts.size();
}

int tabulate(int kind, int D, int p, int npts, const double* xi, double* val, double* grad) {
    Dn b[kMaxLoc];
    int L = 0;
    for (int q = 0; q < npts; q++) {
        L = basis(kind, D, p, xi + (size_t)q * D, b);
        for (int i = 0; i < L; i++) {
            val[(size_t)q * L + i] = b[i].v;
            for (int k = 0; k < D; k++) grad[((size_t)q * L + i) * D + k] = b[i].d[k];
        }
    }
    return L;
}
int quad_rule(int D, int n, std::vector<double>& pts, std::vector<double>& wts) { return simplex_rule(D, n, pts, wts); }

// Basis as polynomials in independent barycentric variables: values and d/d lam_a (a = 0..D).
// Every function of both spaces is such a polynomial, so grad phi = sum_a dphi/dlam_a grad lam_a.
struct DL {
    double v, d[4];
};
static DL lc(double c) { return DL{c, {0, 0, 0, 0}}; }
static DL operator+(DL a, DL b) {
    DL r{a.v + b.v, {}};
    for (int k = 0; k < 4; k++) r.d[k] = a.d[k] + b.d[k];
    return r;
}
static DL operator-(DL a, DL b) {
    DL r{a.v - b.v, {}};
    for (int k = 0; k < 4; k++) r.d[k] = a.d[k] - b.d[k];
    return r;
}
static DL operator*(DL a, double s) {
    DL r{a.v * s, {}};
    for (int k = 0; k < 4; k++) r.d[k] = a.d[k] * s;
    return r;
}
static DL operator*(DL a, DL b) {
    DL r{a.v * b.v, {}};
    for (int k = 0; k < 4; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
static void sleg_l(int n, DL x, DL t, DL* out) {
    out[0] = lc(1);
    if (n >= 1) out[1] = x;
    DL t2 = t * t;
    for (int k = 1; k < n; k++) out[k + 1] = ((x * out[k]) * (2.0 * k + 1) - (t2 * out[k - 1]) * (double)k) * (1.0 / (k + 1));
}
static void jac_l(int n, double a, DL s, DL* out) {
    out[0] = lc(1);
    if (n >= 1) out[1] = (s * (a + 2) + lc(a)) * 0.5;
    for (int k = 2; k <= n; k++) {
        double A = 2.0 * k * (k + a) * (2.0 * k + a - 2);
        double B = 2.0 * k + a - 1;
        double C1 = (2.0 * k + a) * (2.0 * k + a - 2), C0 = a * a;
        double Dd = 2.0 * (k + a - 1) * (k - 1) * (2.0 * k + a);
        out[k] = (((s * C1 + lc(C0)) * out[k - 1]) * B - out[k - 2] * Dd) * (1.0 / A);
    }
}
static int basis_lam(int kind, int D, int p, const double* lamv, DL* out) {
    DL lam[4];
    for (int a = 0; a <= D; a++) {
        lam[a] = lc(lamv[a]);
        lam[a].d[a] = 1;
    }
    int c = 0;
    if (kind == OCMP_H1) {
        for (int v = 0; v <= D; v++) out[c++] = lam[v];
        if (p >= 2)
            for (int a = 0; a <= D; a++)
                for (int b = a + 1; b <= D; b++) {
                    DL L[4];
                    sleg_l(p - 2, lam[b] - lam[a], lam[a] + lam[b], L);
                    DL base = lam[a] * lam[b];
                    for (int k = 0; k <= p - 2; k++) out[c++] = base * L[k];
                }
        if (p >= 3)
            for (int a = 0; a <= D; a++)
                for (int b = a + 1; b <= D; b++)
                    for (int cc = b + 1; cc <= D; cc++) out[c++] = lam[a] * lam[b] * lam[cc];
    } else {
        DL L[8];
        sleg_l(p, lam[1] - lam[0], lam[0] + lam[1], L);
        for (int i = 0; i <= p; i++) {
            DL P[8];
            jac_l(p - i, 2.0 * i + 1, lam[2] * 2.0 - lc(1), P);
            for (int j = 0; j <= p - i; j++) out[c++] = L[i] * P[j];
        }
    }
    return c;
}

// Element-matrix terms. With G_ab = grad lam_a . grad lam_b and wt_a = w . grad lam_a:
//   mass       K_ij  = (mass |det J|)              * int phi_i phi_j
//   stiffness  K_ij += (dt diff |det J| G_ab)       * int (d_a phi_i d_b phi_j + d_b phi_i d_a phi_j) / (1 + [a==b])
//   convection K_ij += (-dt |det J| wt_a)           * int d_a phi_i phi_j          (constant wind)
//              K_ij += (-dt |det J| w_v . grad lam_a) * int lam_v d_a phi_i phi_j  (per-vertex wind)
// Integrals over the reference simplex (exact rule); symmetric parts are kept for i <= j only.
// Terms below 1e-14 of their group's largest are dropped: for the hierarchical P2 tetrahedron the
// element matrix takes 510 products instead of 1000 for dense Cartesian reference tensors.
static void build_terms(int kind, int D, int p, ocmp_tables& T) {
    const int L = T.nloc, NP = D + 1, NS = NP * (NP + 1) / 2;
    T.nsym = L * (L + 1) / 2;
    auto sym = [&](int i, int j) { return i * L - i * (i - 1) / 2 + (j - i); };
    std::vector<double> msum((size_t)L * L, 0.0), ssum((size_t)NS * L * L, 0.0), csum((size_t)NP * L * L, 0.0),
        vsum((size_t)NP * NP * L * L, 0.0);
    DL b[kMaxLoc];
    for (int q = 0; q < T.nq; q++) {
        double lam[4] = {1, 0, 0, 0};
        for (int k = 0; k < D; k++) {
            lam[k + 1] = T.qxi[q * D + k];
            lam[0] -= lam[k + 1];
        }
        basis_lam(kind, D, p, lam, b);
        const double w = T.qw[q];
        for (int i = 0; i < L; i++)
            for (int j = 0; j < L; j++) {
                msum[i * L + j] += w * b[i].v * b[j].v;
                int pi = 0;
                for (int a = 0; a < NP; a++)
                    for (int c = a; c < NP; c++, pi++) {
                        double t = b[i].d[a] * b[j].d[c];
                        if (a != c) t += b[i].d[c] * b[j].d[a];
                        ssum[((size_t)pi * L + i) * L + j] += w * t;
                    }
                for (int a = 0; a < NP; a++) {
                    csum[((size_t)a * L + i) * L + j] += w * b[i].d[a] * b[j].v;
                    for (int v = 0; v < NP; v++)
                        vsum[(((size_t)a * NP + v) * L + i) * L + j] += w * lam[v] * b[i].d[a] * b[j].v;
                }
            }
    }
    const double mmax = *std::max_element(msum.begin(), msum.end(), [](double x, double y) { return std::fabs(x) < std::fabs(y); });
    auto absmax = [](const std::vector<double>& v) {
        double m = 0;
        for (double x : v) m = std::max(m, std::fabs(x));
        return m;
    };
    const double tol_m = 1e-14 * std::fabs(mmax), tol_s = 1e-14 * absmax(ssum), tol_c = 1e-14 * absmax(csum),
                 tol_v = 1e-14 * absmax(vsum);
    for (int var = 0; var < 2; var++) {
        auto& off = T.slot_off[var];
        auto& tg = T.term_g[var];
        auto& tc = T.term_coef[var];
        off.clear();
        tg.clear();
        tc.clear();
        auto conv = [&](int i, int j) {
            if (var == 0) {
                for (int a = 0; a < NP; a++) {
                    const double v = csum[((size_t)a * L + i) * L + j];
                    if (std::fabs(v) > tol_c) { tg.push_back((uint8_t)(1 + NS + a)); tc.push_back(v); }
                }
            } else {
                for (int a = 0; a < NP; a++)
                    for (int vv = 0; vv < NP; vv++) {
                        const double v = vsum[(((size_t)a * NP + vv) * L + i) * L + j];
                        if (std::fabs(v) > tol_v) { tg.push_back((uint8_t)(1 + NS + a * NP + vv)); tc.push_back(v); }
                    }
            }
        };
        for (int i = 0; i < L; i++)
            for (int j = i; j < L; j++) {
                off.push_back((int32_t)tc.size());
                const double mv = msum[i * L + j];
                if (std::fabs(mv) > tol_m) { tg.push_back(0); tc.push_back(mv); }
                off.push_back((int32_t)tc.size());
                for (int f = 0; f < NS; f++) {
                    const double v = ssum[((size_t)f * L + i) * L + j];
                    if (std::fabs(v) > tol_s) { tg.push_back((uint8_t)(1 + f)); tc.push_back(v); }
                }
                off.push_back((int32_t)tc.size());
                conv(i, j);
                off.push_back((int32_t)tc.size());
                if (j != i) conv(j, i);
            }
        off.push_back((int32_t)tc.size());
        T.nterms[var] = (int)tc.size();
    }
    (void)sym;
}

static void build_tables(int kind, int D, int p, ocmp_tables& T) {
    int L = nloc_of(kind, D, p);
    T.nloc = L;
    std::vector<double> qp, qw;
    T.nq = simplex_rule(D, p + 2, qp, qw);
    T.qw = qw;
    T.qxi = qp;
    int S = D * (D + 1) / 2;
    T.ng_const = 1 + S + D;
    T.ng_vtx = 1 + S + D * (D + 1);
    T.R_const.assign((size_t)T.ng_const * L * L, 0.0);
    T.R_vtx.assign((size_t)T.ng_vtx * L * L, 0.0);
    T.qphi.assign((size_t)T.nq * L, 0.0);
    T.mvec.assign(L, 0.0);
    Dn b[kMaxLoc];
    for (int q = 0; q < T.nq; q++) {
        const double* xi = &qp[q * D];
        basis(kind, D, p, xi, b);
        double lam[4];
        lam[0] = 1;
        for (int k = 0; k < D; k++) { lam[k + 1] = xi[k]; lam[0] -= xi[k]; }
        double w = qw[q];
        for (int i = 0; i < L; i++) {
            T.qphi[q * L + i] = b[i].v;
            T.mvec[i] += w * b[i].v;
            for (int j = 0; j < L; j++) {
                size_t ij = (size_t)i * L + j;
                double m = w * b[i].v * b[j].v;
                T.R_const[ij] += m;
                T.R_vtx[ij] += m;
                int g = 1;
                for (int k = 0; k < D; k++)
                    for (int l = k; l < D; l++, g++) {
                        double s = w * b[i].d[k] * b[j].d[l];
                        if (k != l) s += w * b[i].d[l] * b[j].d[k];
                        T.R_const[(size_t)g * L * L + ij] += s;
                        T.R_vtx[(size_t)g * L * L + ij] += s;
                    }
                for (int k = 0; k < D; k++) T.R_const[(size_t)(1 + S + k) * L * L + ij] += w * b[i].d[k] * b[j].v;
                for (int k = 0; k < D; k++)
                    for (int v = 0; v <= D; v++)
                        T.R_vtx[(size_t)(1 + S + k * (D + 1) + v) * L * L + ij] += w * lam[v] * b[i].d[k] * b[j].v;
            }
        }
    }
    // facet tables: local facet f = the facet opposite local vertex f; its vertices in ascending
    // local order a0 < a1 (< a2) with lam_{a0} = 1 - s (- t), lam_{a1} = s, lam_{a2} = t.
    std::vector<double> fp, fw;
    T.nfq = simplex_rule(D - 1, p + 2, fp, fw);
    T.fw = fw;
    int nf = D + 1;
    T.fphi.assign((size_t)nf * T.nfq * L, 0.0);
    T.fdphi.assign((size_t)nf * T.nfq * L * D, 0.0);
    T.flam.assign((size_t)nf * T.nfq * (D + 1), 0.0);
    for (int f = 0; f < nf; f++) {
        int av[3], c = 0;
        for (int v = 0; v <= D; v++)
            if (v != f) av[c++] = v;
        for (int q = 0; q < T.nfq; q++) {
            double lam[4] = {0, 0, 0, 0};
            if (D == 2) {
                lam[av[0]] = 1 - fp[q];
                lam[av[1]] = fp[q];
            } else {
                lam[av[0]] = 1 - fp[2 * q] - fp[2 * q + 1];
                lam[av[1]] = fp[2 * q];
                lam[av[2]] = fp[2 * q + 1];
            }
            double xi[3];
            for (int k = 0; k < D; k++) xi[k] = lam[k + 1];
            basis(kind, D, p, xi, b);
            for (int v = 0; v <= D; v++) T.flam[((size_t)f * T.nfq + q) * (D + 1) + v] = lam[v];
            for (int i = 0; i < L; i++) {
                T.fphi[((size_t)f * T.nfq + q) * L + i] = b[i].v;
                for (int k = 0; k < D; k++) T.fdphi[(((size_t)f * T.nfq + q) * L + i) * D + k] = b[i].d[k];
            }
        }
    }
}

}  // namespace ocmp

using namespace ocmp;

namespace ocmp {
// SELL-32 layout of the space's pattern (see ocmp_space_s), built once on the host
int space_build_sell(ocmp_space_s* s) {
    if (s->d_sell_off) return OCMP_OK;
    const int64_t n = s->ndof, ns = (n + 31) / 32;
    std::vector<int32_t> off(ns + 1), pos(s->nnz);
    int64_t tot = 0;
    for (int64_t sl = 0; sl < ns; sl++) {
        int64_t w = 0;
        for (int64_t r = sl * 32; r < std::min(n, sl * 32 + 32); r++)
            w = std::max<int64_t>(w, (s->rowptr[r + 1] - s->rowptr[r] + 3) / 4);
        off[sl] = (int32_t)tot;
        tot += w * 128;
        if (tot >= (int64_t)INT32_MAX) return fail(OCMP_ERR_UNSUPPORTED, "SELL-32 layout: too many entries");
    }
    off[ns] = (int32_t)tot;
    std::vector<int32_t> colv(tot, 0);
    for (int64_t sl = 0; sl < ns; sl++) {
        const int64_t w = (off[sl + 1] - off[sl]) / 128;
        for (int lane = 0; lane < 32; lane++) {
            const int64_t r = sl * 32 + lane;
            if (r >= n) continue;                           // past the last row: column 0, value 0
            for (int64_t e = 0; e < 4 * w; e++) {
                const int64_t q = off[sl] + ((e / 4) * 32 + lane) * 4 + e % 4;
                const int64_t k = s->rowptr[r] + e;
                if (k < s->rowptr[r + 1]) {
                    colv[q] = s->col[k];
                    pos[k] = (int32_t)q;
                } else {
                    colv[q] = (int32_t)r;                   // padding: the row itself, value 0
                }
            }
        }
    }
    int st = upload(&s->d_sell_off, off.data(), off.size());
    if (!st) st = upload(&s->d_sell_col, colv.data(), colv.size());
    if (!st) st = upload(&s->d_sell_pos, pos.data(), pos.size());
    if (st) {
        dfree(s->d_sell_off);
        dfree(s->d_sell_col);
        dfree(s->d_sell_pos);
        s->d_sell_off = s->d_sell_col = s->d_sell_pos = nullptr;
        return st;
    }
    s->sell_slices = ns;
    s->sell_nent = tot;
    return OCMP_OK;
}
}  // namespace ocmp

extern "C" {

int ocmp_abi_version(void) { return OCMP_ABI_VERSION; }

uint64_t ocmp_launch_count(void) { return (uint64_t)g_launches.load(); }

int ocmp_last_error(char* buf, int len) {
    if (!buf || len <= 0) return OCMP_ERR_ARG;
    std::strncpy(buf, g_err.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
    return OCMP_OK;
}

int ocmp_device_sync(void* stream) {
    OCMP_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return OCMP_OK;
}

int ocmp_mesh_create(const double* coords, int64_t nv, int32_t dim, const int32_t* elements, int64_t ne,
                     const int32_t* bfacets, const int32_t* blabels, int64_t nbf, ocmp_mesh_t* out) {
    if (!out || !coords || !elements || (dim != 2 && dim != 3) || nv <= 0 || ne <= 0 || nbf < 0 ||
        (nbf > 0 && (!bfacets || !blabels)))
        return fail(OCMP_ERR_ARG, "ocmp_mesh_create: bad arguments");
    if (nv >= (int64_t)1 << 31 || ne * (dim + 1) >= (int64_t)1 << 31)
        return fail(OCMP_ERR_ARG, "ocmp_mesh_create: mesh too large for 32-bit indices");
    auto* m = new ocmp_mesh_s();
    m->dim = dim;
    m->nv = nv;
    m->ne = ne;
    m->nbf = nbf;
    m->X.assign(coords, coords + nv * dim);
    m->conn.assign(elements, elements + ne * (dim + 1));
    for (int64_t i = 0; i < ne * (dim + 1); i++)
        if (m->conn[i] < 0 || m->conn[i] >= nv) {
            delete m;
            return fail(OCMP_ERR_ARG, "ocmp_mesh_create: element vertex index out of range");
        }
    for (int64_t e = 0; e < ne; e++) std::sort(m->conn.begin() + e * (dim + 1), m->conn.begin() + (e + 1) * (dim + 1));
    if (nbf) {
        m->bfac.assign(bfacets, bfacets + nbf * dim);
        m->blab.assign(blabels, blabels + nbf);
    }
    int st = upload(&m->dX, m->X.data(), m->X.size());
    if (!st) st = upload(&m->dconn, m->conn.data(), m->conn.size());
    if (st) {
        dfree(m->dX);
        dfree(m->dconn);
        delete m;
        return st;
    }
    *out = m;
    return OCMP_OK;
}

int ocmp_mesh_destroy(ocmp_mesh_t m) {
    if (!m) return OCMP_OK;
    dfree(m->dX);
    dfree(m->dconn);
    delete m;
    return OCMP_OK;
}

static void free_space_device(ocmp_space_s* s) {
    void* ps[] = {s->d_dofs,     s->d_rowptr,   s->d_col,       s->d_free,     s->d_diag,      s->d_slot,
                  s->d_fslot,    s->d_efac_ptr, s->d_efac,      s->d_slot_off[0], s->d_term_g[0], s->d_term_coef[0],
                  s->d_slot_off[1], s->d_term_g[1], s->d_term_coef[1], s->d_term_coef_ff[0], s->d_term_coef_ff[1],
                  s->d_inc_ptr,  s->d_inc,      s->d_ifac,      s->d_bfac,     s->d_ebf_ptr,   s->d_ebf,
                  s->d_Rc,       s->d_Rv,       s->d_qw,        s->d_qphi,     s->d_mvec,      s->d_fw,
                  s->d_fphi,     s->d_fdphi,    s->d_flam,      s->d_K,        s->d_facetK,    s->d_Fe,
                  s->d_lift_ptr, s->d_lift_pos, s->d_Rm_ff, s->d_geo_ff, s->d_tpos, s->d_cseg, s->d_csrc, s->d_u2, s->d_Kd,
                  s->d_sell_off, s->d_sell_col, s->d_sell_pos};
    for (void* p : ps) dfree(p);
}

int ocmp_space_create(ocmp_mesh_t mesh, int32_t kind, int32_t order, uint32_t dirichlet_mask, ocmp_space_t* out) {
    if (!mesh || !out) return fail(OCMP_ERR_ARG, "ocmp_space_create: null argument");
    const int D = mesh->dim, nvp = D + 1, p = order;
    if (kind != OCMP_H1 && kind != OCMP_L2) return fail(OCMP_ERR_ARG, "ocmp_space_create: kind must be H1 or L2");
    if (p < 1 || p > 3) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_space_create: order must be 1..3");
    if (kind == OCMP_L2 && D != 2) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_space_create: L2 is built for triangles only");
    auto* s = new ocmp_space_s();
    s->mesh = mesh;
    s->kind = kind;
    s->order = p;
    s->dim = D;
    s->dirichlet_mask = dirichlet_mask;
    const int L = s->nloc = nloc_of(kind, D, p);
    const int64_t ne = mesh->ne, nv = mesh->nv;
    const int32_t* conn = mesh->conn.data();
    build_tables(kind, D, p, s->T);
    build_terms(kind, D, p, s->T);

    // ---- dof map
    s->dofs.resize((size_t)ne * L);
    if (kind == OCMP_L2) {
        s->ndof = ne * L;
        for (int64_t i = 0; i < ne * L; i++) s->dofs[i] = (int32_t)i;
    } else {
        const int nel = D == 2 ? 3 : 6, nfl = D == 2 ? 1 : 4;
        std::vector<int64_t> ek, fk;
        if (p >= 2) {
            ek.resize((size_t)ne * nel);
            parallel_for(ne, [&](int64_t a, int64_t b) {
                for (int64_t e = a; e < b; e++) {
                    int c = 0;
                    for (int x = 0; x < nvp; x++)
                        for (int y = x + 1; y < nvp; y++) ek[e * nel + c++] = (int64_t)conn[e * nvp + x] * nv + conn[e * nvp + y];
                }
            });
            std::sort(ek.begin(), ek.end());
            ek.erase(std::unique(ek.begin(), ek.end()), ek.end());
        }
        if (p >= 3) {
            fk.resize((size_t)ne * nfl);
            for (int64_t e = 0; e < ne; e++) {
                int c = 0;
                for (int x = 0; x < nvp; x++)
                    for (int y = x + 1; y < nvp; y++)
                        for (int z = y + 1; z < nvp; z++)
                            fk[e * nfl + c++] = ((int64_t)conn[e * nvp + x] * nv + conn[e * nvp + y]) * nv + conn[e * nvp + z];
            }
            std::sort(fk.begin(), fk.end());
            fk.erase(std::unique(fk.begin(), fk.end()), fk.end());
        }
        const int64_t ned = (int64_t)ek.size(), nfc = (int64_t)fk.size();
        const int epd = p - 1;
        s->ndof = nv + ned * epd + nfc * (p >= 3 ? 1 : 0);
        if (s->ndof >= (int64_t)1 << 31) {
            delete s;
            return fail(OCMP_ERR_ARG, "ocmp_space_create: too many dofs for 32-bit indices");
        }
        parallel_for(ne, [&](int64_t a, int64_t b) {
            for (int64_t e = a; e < b; e++) {
                const int32_t* v = conn + e * nvp;
                int c = 0;
                int32_t* d = &s->dofs[e * L];
                for (int x = 0; x < nvp; x++) d[c++] = v[x];
                if (p >= 2)
                    for (int x = 0; x < nvp; x++)
                        for (int y = x + 1; y < nvp; y++) {
                            int64_t id = std::lower_bound(ek.begin(), ek.end(), (int64_t)v[x] * nv + v[y]) - ek.begin();
                            for (int k = 0; k < epd; k++) d[c++] = (int32_t)(nv + id * epd + k);
                        }
                if (p >= 3)
                    for (int x = 0; x < nvp; x++)
                        for (int y = x + 1; y < nvp; y++)
                            for (int z = y + 1; z < nvp; z++) {
                                int64_t key = ((int64_t)v[x] * nv + v[y]) * nv + v[z];
                                int64_t id = std::lower_bound(fk.begin(), fk.end(), key) - fk.begin();
                                d[c++] = (int32_t)(nv + ned * epd + id);
                            }
            }
        });
    }
    const int64_t nd = s->ndof;

    // ---- facets
    {
        std::vector<std::pair<int64_t, int64_t>> fkeys((size_t)ne * nvp);
        parallel_for(ne, [&](int64_t a, int64_t b) {
            for (int64_t e = a; e < b; e++)
                for (int f = 0; f < nvp; f++) {
                    int64_t k = 0;
                    for (int v = 0; v < nvp; v++)
                        if (v != f) k = k * nv + conn[e * nvp + v];
                    fkeys[e * nvp + f] = {k, e * nvp + f};
                }
        });
        std::sort(fkeys.begin(), fkeys.end());
        for (size_t i = 0; i + 1 < fkeys.size(); i++)
            if (fkeys[i].first == fkeys[i + 1].first) {
                int64_t a = fkeys[i].second, b = fkeys[i + 1].second;
                s->ifac.push_back((int32_t)(a / nvp));
                s->ifac.push_back((int32_t)(a % nvp));
                s->ifac.push_back((int32_t)(b / nvp));
                s->ifac.push_back((int32_t)(b % nvp));
                i++;
            }
        s->nif = (int64_t)s->ifac.size() / 4;
        for (int64_t b = 0; b < mesh->nbf; b++) {
            int32_t vv[3];
            for (int k = 0; k < D; k++) vv[k] = mesh->bfac[b * D + k];
            std::sort(vv, vv + D);
            int64_t key = 0;
            for (int k = 0; k < D; k++) key = key * nv + vv[k];
            auto it = std::lower_bound(fkeys.begin(), fkeys.end(), std::make_pair(key, (int64_t)-1));
            if (it == fkeys.end() || it->first != key) continue;  // facet not on any element: ignored
            s->bfac.push_back((int32_t)(it->second / nvp));
            s->bfac.push_back((int32_t)(it->second % nvp));
            s->bfac.push_back(mesh->blab[b]);
        }
        s->nbf = (int64_t)s->bfac.size() / 3;
    }

    // ---- free dofs (H1): every function living on a Dirichlet-labelled facet is constrained
    s->freed.assign(nd, 1);
    if (kind == OCMP_H1)
        for (int64_t b = 0; b < s->nbf; b++) {
            int lab = s->bfac[3 * b + 2];
            if (lab < 0 || lab >= 32 || !((dirichlet_mask >> lab) & 1u)) continue;
            int64_t e = s->bfac[3 * b];
            int f = s->bfac[3 * b + 1];
            int c = 0;
            const int32_t* d = &s->dofs[e * L];
            for (int a = 0; a < nvp; a++, c++)
                if (a != f) s->freed[d[c]] = 0;
            if (p >= 2)
                for (int a = 0; a < nvp; a++)
                    for (int bb = a + 1; bb < nvp; bb++)
                        for (int k = 0; k < p - 1; k++, c++)
                            if (a != f && bb != f) s->freed[d[c]] = 0;
            if (p >= 3)
                for (int a = 0; a < nvp; a++)
                    for (int bb = a + 1; bb < nvp; bb++)
                        for (int cc = bb + 1; cc < nvp; cc++, c++)
                            if (a != f && bb != f && cc != f) s->freed[d[c]] = 0;
        }

    // ---- dof -> (element, local) incidence
    std::vector<int32_t> inc_ptr(nd + 1, 0), inc((size_t)ne * L);
    for (int64_t i = 0; i < ne * L; i++) inc_ptr[s->dofs[i] + 1]++;
    for (int64_t i = 0; i < nd; i++) inc_ptr[i + 1] += inc_ptr[i];
    {
        std::vector<int32_t> fill(inc_ptr.begin(), inc_ptr.end() - 1);
        for (int64_t i = 0; i < ne * L; i++) inc[fill[s->dofs[i]]++] = (int32_t)i;
    }
    // element -> interior facets (L2) and element -> boundary facets
    std::vector<int32_t> enb((size_t)ne * nvp, -1);  // facet index of local facet f (interior), or -1
    for (int64_t fi = 0; fi < s->nif; fi++) {
        enb[(int64_t)s->ifac[4 * fi] * nvp + s->ifac[4 * fi + 1]] = (int32_t)fi;
        enb[(int64_t)s->ifac[4 * fi + 2] * nvp + s->ifac[4 * fi + 3]] = (int32_t)fi;
    }
    std::vector<int32_t> ebf_ptr(ne + 1, 0), ebf((size_t)s->nbf);
    for (int64_t b = 0; b < s->nbf; b++) ebf_ptr[s->bfac[3 * b] + 1]++;
    for (int64_t e = 0; e < ne; e++) ebf_ptr[e + 1] += ebf_ptr[e];
    {
        std::vector<int32_t> fill(ebf_ptr.begin(), ebf_ptr.end() - 1);
        for (int64_t b = 0; b < s->nbf; b++) ebf[fill[s->bfac[3 * b]]++] = (int32_t)b;
    }
    const bool dgj = kind == OCMP_L2;

    // ---- CSR pattern (row-parallel sort/unique of the incident elements' dofs)
    std::vector<std::vector<int32_t>> rows(nd);
    std::vector<int64_t> rl(nd + 1, 0);
    parallel_for(nd, [&](int64_t a, int64_t b) {
        std::vector<int32_t> buf;
        for (int64_t r = a; r < b; r++) {
            buf.clear();
            for (int32_t k = inc_ptr[r]; k < inc_ptr[r + 1]; k++) {
                int64_t e = inc[k] / L;
                buf.insert(buf.end(), &s->dofs[e * L], &s->dofs[e * L] + L);
                if (dgj)
                    for (int f = 0; f < nvp; f++) {
                        int32_t fi = enb[e * nvp + f];
                        if (fi < 0) continue;
                        int64_t o = s->ifac[4 * fi] == e ? s->ifac[4 * fi + 2] : s->ifac[4 * fi];
                        buf.insert(buf.end(), &s->dofs[o * L], &s->dofs[o * L] + L);
                    }
            }
            std::sort(buf.begin(), buf.end());
            buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
            rows[r] = buf;
            rl[r + 1] = (int64_t)buf.size();
        }
    });
    for (int64_t r = 0; r < nd; r++) rl[r + 1] += rl[r];
    s->nnz = rl[nd];
    if (s->nnz >= (int64_t)1 << 31) {
        delete s;
        return fail(OCMP_ERR_ARG, "ocmp_space_create: nnz too large for 32-bit row pointers");
    }
    s->rowptr = rl;
    s->col.resize(s->nnz);
    parallel_for(nd, [&](int64_t a, int64_t b) {
        for (int64_t r = a; r < b; r++) {
            std::copy(rows[r].begin(), rows[r].end(), s->col.begin() + rl[r]);
            std::vector<int32_t>().swap(rows[r]);
        }
    });
    std::vector<std::vector<int32_t>>().swap(rows);

    // ---- slot tables: for element e and local row i, the position within CSR row dof(e,i) of
    // each column dof(e,j); the same for the 2L columns of every interior-facet matrix row (L2).
    for (int64_t r = 0; r < nd; r++) s->maxrow = std::max<int>(s->maxrow, (int)(rl[r + 1] - rl[r]));
    s->row_ranges = {0};
    if (kind == OCMP_H1 && p >= 2 && nv < nd) s->row_ranges.push_back(nv);
    s->row_ranges.push_back(nd);
    for (size_t q = 0; q + 1 < s->row_ranges.size(); q++) {
        int mx = 0;
        for (int64_t r = s->row_ranges[q]; r < s->row_ranges[q + 1]; r++) mx = std::max<int>(mx, (int)(rl[r + 1] - rl[r]));
        s->range_maxrow.push_back(mx);
    }
    if (s->maxrow > 255) {
        delete s;
        return fail(OCMP_ERR_UNSUPPORTED, "ocmp_space_create: a CSR row exceeds 255 entries");
    }
    const int64_t LL = (int64_t)L * L;
    const int SS = s->slot_stride = (L + 15) / 16 * 16;   // one 16-byte load per slice for L <= 16
    std::vector<uint8_t> slot((size_t)(ne * L * SS), 0);
    parallel_for(ne, [&](int64_t a0, int64_t b0) {
        for (int64_t e = a0; e < b0; e++)
            for (int i = 0; i < L; i++) {
                const int32_t r = s->dofs[e * L + i];
                const int32_t* c0 = s->col.data() + rl[r];
                const int64_t rn = rl[r + 1] - rl[r];
                for (int j = 0; j < L; j++)
                    slot[(e * L + i) * SS + j] = (uint8_t)(std::lower_bound(c0, c0 + rn, s->dofs[e * L + j]) - c0);
            }
    });
    std::vector<uint8_t> fslot;
    std::vector<int32_t> efac_ptr(ne + 1, 0), efac;
    if (dgj) {
        fslot.resize((size_t)s->nif * 4 * LL);
        parallel_for(s->nif, [&](int64_t a0, int64_t b0) {
            for (int64_t fi = a0; fi < b0; fi++) {
                const int64_t eL = s->ifac[4 * fi], eR = s->ifac[4 * fi + 2];
                for (int side = 0; side < 2; side++) {
                    const int64_t e = side ? eR : eL;
                    for (int i = 0; i < L; i++) {
                        const int32_t r = s->dofs[e * L + i];
                        const int32_t* c0 = s->col.data() + rl[r];
                        const int64_t rn = rl[r + 1] - rl[r];
                        for (int jj = 0; jj < 2 * L; jj++) {
                            const int32_t cd = jj < L ? s->dofs[eL * L + jj] : s->dofs[eR * L + jj - L];
                            fslot[((fi * 2 + side) * L + i) * 2 * L + jj] =
                                (uint8_t)(std::lower_bound(c0, c0 + rn, cd) - c0);
                        }
                    }
                }
            }
        });
        for (int64_t fi = 0; fi < s->nif; fi++) {
            efac_ptr[s->ifac[4 * fi] + 1]++;
            efac_ptr[s->ifac[4 * fi + 2] + 1]++;
        }
        for (int64_t e = 0; e < ne; e++) efac_ptr[e + 1] += efac_ptr[e];
        efac.resize(efac_ptr[ne]);
        std::vector<int32_t> fill(efac_ptr.begin(), efac_ptr.end() - 1);
        for (int64_t fi = 0; fi < s->nif; fi++) {
            efac[fill[s->ifac[4 * fi]]++] = (int32_t)(fi * 2);
            efac[fill[s->ifac[4 * fi + 2]]++] = (int32_t)(fi * 2 + 1);
        }
    }
    s->ncontrib = ne * LL + s->nif * 4 * LL + s->nbf * LL;
    std::vector<int32_t> diag(nd);
    for (int64_t r = 0; r < nd; r++) {
        const int32_t* c0 = s->col.data() + rl[r];
        diag[r] = (int32_t)(rl[r] + (std::lower_bound(c0, c0 + (rl[r + 1] - rl[r]), (int32_t)r) - c0));
    }
    // lift list: entries of free rows in constrained columns (the Dirichlet lift A_fD x_D)
    std::vector<int32_t> lift_ptr(nd + 1, 0), lift_pos;
    for (int64_t r = 0; r < nd; r++) {
        if (s->freed[r])
            for (int64_t k = rl[r]; k < rl[r + 1]; k++)
                if (!s->freed[s->col[k]]) lift_pos.push_back((int32_t)k);
        lift_ptr[r + 1] = (int32_t)lift_pos.size();
    }

    // ---- upload
    std::vector<int32_t> rp32(nd + 1);
    for (int64_t i = 0; i <= nd; i++) rp32[i] = (int32_t)rl[i];
    int st = OCMP_OK;
    auto U = [&](auto** dst, const auto& v) {
        if (!st) st = upload(dst, v.data(), v.size());
    };
    U(&s->d_dofs, s->dofs);
    U(&s->d_rowptr, rp32);
    U(&s->d_col, s->col);
    U(&s->d_free, s->freed);
    U(&s->d_diag, diag);
    U(&s->d_slot, slot);
    U(&s->d_fslot, fslot);
    U(&s->d_efac_ptr, efac_ptr);
    U(&s->d_efac, efac);
    for (int var = 0; var < 2; var++) {
        U(&s->d_slot_off[var], s->T.slot_off[var]);
        U(&s->d_term_g[var], s->T.term_g[var]);
        U(&s->d_term_coef[var], s->T.term_coef[var]);
        std::vector<float2> ff(s->T.term_coef[var].size());
        for (size_t t = 0; t < ff.size(); t++) {
            const double c = s->T.term_coef[var][t];
            const float hi = (float)c;
            ff[t] = make_float2(hi, (float)(c - (double)hi));
        }
        U(&s->d_term_coef_ff[var], ff);
    }
    U(&s->d_inc_ptr, inc_ptr);
    U(&s->d_inc, inc);
    U(&s->d_ifac, s->ifac);
    U(&s->d_bfac, s->bfac);
    U(&s->d_ebf_ptr, ebf_ptr);
    U(&s->d_ebf, ebf);
    U(&s->d_lift_ptr, lift_ptr);
    U(&s->d_lift_pos, lift_pos);
    U(&s->d_Rc, s->T.R_const);
    {
        // reference mass matrix as (hi, lo) float pairs for the double-float RHS
        const size_t LLm = (size_t)s->nloc * s->nloc;
        std::vector<float2> rm(LLm);
        for (size_t t = 0; t < LLm; t++) {
            const double c = s->T.R_const[t];
            const float hi = (float)c;
            rm[t] = make_float2(hi, (float)(c - (double)hi));
        }
        U(&s->d_Rm_ff, rm);
    }
    U(&s->d_Rv, s->T.R_vtx);
    U(&s->d_qw, s->T.qw);
    U(&s->d_qphi, s->T.qphi);
    U(&s->d_mvec, s->T.mvec);
    U(&s->d_fw, s->T.fw);
    U(&s->d_fphi, s->T.fphi);
    U(&s->d_fdphi, s->T.fdphi);
    U(&s->d_flam, s->T.flam);
    if (!st) st = dalloc(&s->d_K, (size_t)(ne * LL));
    if (!st) st = dalloc(&s->d_facetK, (size_t)(s->nif * 4 * LL + s->nbf * LL));
    if (!st) st = dalloc(&s->d_Fe, (size_t)ne * L);
    if (st) {
        free_space_device(s);
        delete s;
        return st;
    }
    *out = s;
    return OCMP_OK;
}

int ocmp_space_destroy(ocmp_space_t s) {
    if (!s) return OCMP_OK;
    free_space_device(s);
    delete s;
    return OCMP_OK;
}

int ocmp_space_info(ocmp_space_t s, ocmp_space_info_t* info) {
    if (!s || !info) return fail(OCMP_ERR_ARG, "ocmp_space_info: null argument");
    info->ndof = s->ndof;
    info->nnz = s->nnz;
    info->ne = s->mesh->ne;
    info->nv = s->mesh->nv;
    info->nloc = s->nloc;
    info->nq = s->T.nq;
    info->dim = s->dim;
    info->order = s->order;
    info->kind = s->kind;
    info->n_interior_facets = s->nif;
    info->n_boundary_facets = s->nbf;
    info->n_contrib = s->ncontrib;
    info->nfq = s->T.nfq;
    return OCMP_OK;
}

int ocmp_space_get_dofs(ocmp_space_t s, int32_t* d) {
    if (!s || !d) return fail(OCMP_ERR_ARG, "ocmp_space_get_dofs: null argument");
    if (s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_space_get_dofs: compound space");
    std::memcpy(d, s->dofs.data(), s->dofs.size() * sizeof(int32_t));
    return OCMP_OK;
}

int ocmp_space_get_pattern(ocmp_space_t s, int64_t* rp, int32_t* col) {
    if (!s || !rp || !col) return fail(OCMP_ERR_ARG, "ocmp_space_get_pattern: null argument");
    std::memcpy(rp, s->rowptr.data(), s->rowptr.size() * sizeof(int64_t));
    std::memcpy(col, s->col.data(), s->col.size() * sizeof(int32_t));
    return OCMP_OK;
}

int ocmp_space_get_free(ocmp_space_t s, uint8_t* f) {
    if (!s || !f) return fail(OCMP_ERR_ARG, "ocmp_space_get_free: null argument");
    std::memcpy(f, s->freed.data(), s->freed.size());
    return OCMP_OK;
}

int ocmp_space_quad_points(ocmp_space_t s, double* xyz) {
    if (s && s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_space_quad_points: compound space");
    if (!s || !xyz) return fail(OCMP_ERR_ARG, "ocmp_space_quad_points: null argument");
    const int D = s->dim, nvp = D + 1, nq = s->T.nq;
    const ocmp_mesh_s* m = s->mesh;
    parallel_for(m->ne, [&](int64_t a, int64_t b) {
        for (int64_t e = a; e < b; e++) {
            const int32_t* v = &m->conn[e * nvp];
            for (int q = 0; q < nq; q++)
                for (int r = 0; r < D; r++) {
                    double x0 = m->X[(int64_t)v[0] * D + r], acc = x0;
                    for (int c = 0; c < D; c++) acc += (m->X[(int64_t)v[c + 1] * D + r] - x0) * s->T.qxi[q * D + c];
                    xyz[(e * nq + q) * D + r] = acc;
                }
        }
    });
    return OCMP_OK;
}

int ocmp_set_boundary(ocmp_space_t s, uint32_t mask, const double* gval, double* u, void* stream) {
    if (s && s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_set_boundary: compound space");
    if (!s || !gval || !u) return fail(OCMP_ERR_ARG, "ocmp_set_boundary: null argument");
    return launch_set_boundary(s, mask, gval, u, (cudaStream_t)stream);
}

int ocmp_space_facet_quad_points(ocmp_space_t s, double* xyz) {
    if (s && s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_space_facet_quad_points: compound space");
    if (!s || !xyz) return fail(OCMP_ERR_ARG, "ocmp_space_facet_quad_points: null argument");
    const int D = s->dim, nvp = D + 1, nfq = s->T.nfq;
    const ocmp_mesh_s* m = s->mesh;
    for (int64_t b = 0; b < s->nbf; b++) {
        const int64_t e = s->bfac[3 * b];
        const int lf = s->bfac[3 * b + 1];
        const int32_t* v = &m->conn[e * nvp];
        for (int q = 0; q < nfq; q++) {
            const double* lam = &s->T.flam[((size_t)lf * nfq + q) * nvp];
            for (int r = 0; r < D; r++) {
                double acc = 0;
                for (int a = 0; a < nvp; a++) acc += lam[a] * m->X[(int64_t)v[a] * D + r];
                xyz[(b * nfq + q) * D + r] = acc;
            }
        }
    }
    return OCMP_OK;
}

int ocmp_space_boundary_facets(ocmp_space_t s, int32_t* out) {
    if (s && s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_space_boundary_facets: compound space");
    if (!s || !out) return fail(OCMP_ERR_ARG, "ocmp_space_boundary_facets: null argument");
    std::memcpy(out, s->bfac.data(), s->bfac.size() * sizeof(int32_t));
    return OCMP_OK;
}

namespace {
// Walks the facets whose label is in `mask` in the space's boundary-facet order. Per facet the
// sample points are: its D vertices; for order >= 2 the (p+2)-point Gauss rule on each of its edges
// (local vertex pairs in ascending order); for a tetrahedral face at order 3 the collapsed
// (p+2)^2-point rule on the face. With `xyz` the points are written; with `g` (samples at those
// points) the constrained dofs and their values are appended to idx/val: vertex dofs take g, edge
// bubbles the 1D L2 projection of what the vertex part leaves, face bubbles the 2D projection of what
// vertices and edges leave. A dof met again on a later facet takes the later facet's value.
int64_t walk_boundary(const ocmp_space_s* s, uint32_t mask, const double* g, double* xyz, std::vector<int32_t>* idx,
                      std::vector<double>* val) {
    const int D = s->dim, nvp = D + 1, p = s->order, L = s->nloc;
    const int nedge = nvp * (nvp - 1) / 2;
    std::vector<double> x1, w1, x2, w2;
    const int n1 = simplex_rule(1, p + 2, x1, w1), n2 = simplex_rule(2, p + 2, x2, w2);
    const ocmp_mesh_s* m = s->mesh;
    std::vector<double> dval;
    std::vector<uint8_t> own;
    if (g) {
        dval.assign(s->ndof, 0.0);
        own.assign(s->ndof, 0);
    }
    auto edge_id = [nvp](int a, int b) {
        int k = 0;
        for (int i = 0; i < nvp; i++)
            for (int j = i + 1; j < nvp; j++, k++)
                if (i == a && j == b) return k;
        return -1;
    };
    int64_t np = 0;
    Dn bb[kMaxLoc];
    for (int64_t b = 0; b < s->nbf; b++) {
        const int lab = s->bfac[3 * b + 2];
        if (lab < 0 || lab >= 32 || !((mask >> lab) & 1u)) continue;
        const int64_t e = s->bfac[3 * b];
        const int lf = s->bfac[3 * b + 1];
        const int32_t* cv = &m->conn[e * nvp];
        int av[3], c = 0;
        for (int v = 0; v < nvp; v++)
            if (v != lf) av[c++] = v;
        double coef[kMaxLoc] = {0};
        std::vector<int> touched;
        auto point = [&](const double* lam) {
            if (xyz)
                for (int r = 0; r < D; r++) {
                    double acc = 0;
                    for (int a = 0; a < nvp; a++) acc += lam[a] * m->X[(int64_t)cv[a] * D + r];
                    xyz[np * D + r] = acc;
                }
            return np++;
        };
        auto eval = [&](const double* lam) {
            double xi[3];
            for (int k = 0; k < D; k++) xi[k] = lam[k + 1];
            basis(s->kind, D, p, xi, bb);
        };
        for (int k = 0; k < D; k++) {
            double lam[4] = {0, 0, 0, 0};
            lam[av[k]] = 1;
            const int64_t q = point(lam);
            if (g) coef[av[k]] = g[q];
            touched.push_back(av[k]);
        }
        if (p >= 2)
            for (int i = 0; i < D; i++)
                for (int j = i + 1; j < D; j++) {
                    const int a = av[i], bv = av[j], e0 = nvp + edge_id(a, bv) * (p - 1);
                    double M[2][2] = {{0, 0}, {0, 0}}, r[2] = {0, 0};
                    for (int q = 0; q < n1; q++) {
                        double lam[4] = {0, 0, 0, 0};
                        lam[a] = 1 - x1[q];
                        lam[bv] = x1[q];
                        const int64_t pi = point(lam);
                        if (!g) continue;
                        eval(lam);
                        const double res = g[pi] - coef[a] * bb[a].v - coef[bv] * bb[bv].v;
                        for (int k = 0; k < p - 1; k++) {
                            r[k] += w1[q] * bb[e0 + k].v * res;
                            for (int l = 0; l < p - 1; l++) M[k][l] += w1[q] * bb[e0 + k].v * bb[e0 + l].v;
                        }
                    }
                    if (g) {
                        if (p == 2) {
                            coef[e0] = r[0] / M[0][0];
                        } else {
                            const double det = M[0][0] * M[1][1] - M[0][1] * M[1][0];
                            coef[e0] = (M[1][1] * r[0] - M[0][1] * r[1]) / det;
                            coef[e0 + 1] = (M[0][0] * r[1] - M[1][0] * r[0]) / det;
                        }
                    }
                    for (int k = 0; k < p - 1; k++) touched.push_back(e0 + k);
                }
        if (D == 3 && p == 3) {
            int fid = 0;
            for (int a = 0; a < nvp; a++)
                for (int b2 = a + 1; b2 < nvp; b2++)
                    for (int c2 = b2 + 1; c2 < nvp; c2++, fid++)
                        if (a == av[0] && b2 == av[1] && c2 == av[2]) goto found;
        found:
            const int f0 = nvp + nedge * (p - 1) + fid;
            double num = 0, den = 0;
            for (int q = 0; q < n2; q++) {
                double lam[4] = {0, 0, 0, 0};
                lam[av[0]] = 1 - x2[2 * q] - x2[2 * q + 1];
                lam[av[1]] = x2[2 * q];
                lam[av[2]] = x2[2 * q + 1];
                const int64_t pi = point(lam);
                if (!g) continue;
                eval(lam);
                double res = g[pi];
                for (int t : touched) res -= coef[t] * bb[t].v;
                num += w2[q] * bb[f0].v * res;
                den += w2[q] * bb[f0].v * bb[f0].v;
            }
            if (g) coef[f0] = num / den;
            touched.push_back(f0);
        }
        if (g)
            for (int t : touched) {
                const int32_t d = s->dofs[e * L + t];
                dval[d] = coef[t];
                own[d] = 1;
            }
    }
    if (g)
        for (int64_t i = 0; i < s->ndof; i++)
            if (own[i]) {
                idx->push_back((int32_t)i);
                val->push_back(dval[i]);
            }
    return np;
}
}  // namespace

int ocmp_boundary_points(ocmp_space_t s, uint32_t mask, int64_t* npts, double* xyz) {
    if (s && s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_boundary_points: compound space");
    if (!s || !npts) return fail(OCMP_ERR_ARG, "ocmp_boundary_points: null argument");
    if (s->kind != OCMP_H1) {
        *npts = 0;
        return OCMP_OK;
    }
    *npts = walk_boundary(s, mask, nullptr, xyz, nullptr, nullptr);
    return OCMP_OK;
}

int ocmp_set_boundary_values(ocmp_space_t s, uint32_t mask, const double* g, double* u, void* stream) {
    if (s && s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_set_boundary_values: compound space");
    if (!s || !g || !u) return fail(OCMP_ERR_ARG, "ocmp_set_boundary_values: null argument");
    if (s->kind != OCMP_H1) return OCMP_OK;
    std::vector<int32_t> idx;
    std::vector<double> val;
    walk_boundary(s, mask, g, nullptr, &idx, &val);
    return launch_scatter_values(idx, val, u, (cudaStream_t)stream);
}

int ocmp_l2_error(ocmp_space_t s, const double* u, const double* fq, double fconst, double* result, void* stream) {
    if (s && s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_l2_error: compound space");
    if (!s || !u || !result) return fail(OCMP_ERR_ARG, "ocmp_l2_error: null argument");
    return launch_l2_error(s, u, fq, fconst, result, (cudaStream_t)stream);
}

int ocmp_matrix_create_batch(ocmp_space_t s, int32_t nbatch, int32_t flags, ocmp_matrix_t* out) {
    if (!s || !out || nbatch < 1) return fail(OCMP_ERR_ARG, "ocmp_matrix_create: bad argument");
    auto* m = new ocmp_matrix_s();
    m->space = s;
    m->flags = flags;
    m->B = nbatch;
    const size_t nz = (size_t)s->nnz * nbatch, nd = (size_t)s->ndof * nbatch;
    if ((flags & OCMP_MAT_SELL32) && (!(flags & OCMP_MAT_JACOBI32) || nbatch != 1 || s->kind == OCMP_COMPOUND)) {
        delete m;
        return fail(OCMP_ERR_ARG, "ocmp_matrix_create: OCMP_MAT_SELL32 needs OCMP_MAT_JACOBI32 on a single matrix");
    }
    int st = (flags & OCMP_MAT_SELL32) ? space_build_sell(s) : OCMP_OK;
    if (!st) st = dalloc(&m->vals, nz);
    if (!st && (flags & OCMP_MAT_FP32)) st = dalloc(&m->vals32, nz);
    if (!st && (flags & OCMP_MAT_JACOBI64)) st = dalloc(&m->svals64, nz);
    if (!st && (flags & OCMP_MAT_JACOBI32)) {
        const size_t n32 = (flags & OCMP_MAT_SELL32) ? (size_t)s->sell_nent : nz;
        st = dalloc(&m->svals32, n32);
        if (!st && (flags & OCMP_MAT_SELL32) && cudaMemset(m->svals32, 0, sizeof(float) * n32) != cudaSuccess)
            st = OCMP_ERR_CUDA;
    }
    if (!st && (flags & (OCMP_MAT_JACOBI64 | OCMP_MAT_JACOBI32))) st = dalloc(&m->dinv, nd);
    if (!st && (flags & OCMP_MAT_JACOBI32)) st = dalloc(&m->dinv32, nd);
    if (!st) st = cudaMemset(m->vals, 0, sizeof(double) * nz) == cudaSuccess ? 0 : OCMP_ERR_CUDA;
    if (st) {
        dfree(m->vals);
        dfree(m->vals32);
        dfree(m->svals64);
        dfree(m->svals32);
        dfree(m->dinv);
        dfree(m->dinv32);
        delete m;
        return st;
    }
    *out = m;
    return OCMP_OK;
}

int ocmp_matrix_create(ocmp_space_t s, int32_t flags, ocmp_matrix_t* out) {
    return ocmp_matrix_create_batch(s, 1, flags, out);
}

int ocmp_matrix_destroy(ocmp_matrix_t m) {
    if (!m) return OCMP_OK;
    dfree(m->vals);
    dfree(m->vals32);
    dfree(m->svals64);
    dfree(m->svals32);
    dfree(m->dinv);
    dfree(m->dinv32);
    delete m;
    return OCMP_OK;
}

int ocmp_matrix_values(ocmp_matrix_t m, double** v64, float** v32) {
    if (!m) return fail(OCMP_ERR_ARG, "ocmp_matrix_values: null argument");
    if (v64) *v64 = m->vals;
    if (v32) *v32 = m->vals32;
    return OCMP_OK;
}

int ocmp_matrix_scaled_values(ocmp_matrix_t m, double** s64, float** s32, double** dinv) {
    if (!m) return fail(OCMP_ERR_ARG, "ocmp_matrix_scaled_values: null argument");
    if (s64) *s64 = m->svals64;
    if (s32) *s32 = m->svals32;
    if (dinv) *dinv = m->dinv;
    return OCMP_OK;
}

int ocmp_assemble_matrix(ocmp_matrix_t m, const ocmp_form_t* f, void* stream) {
    if (m && m->space->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_assemble_matrix: compound space (ocmp_th_assemble)");
    if (!m || !f) return fail(OCMP_ERR_ARG, "ocmp_assemble_matrix: null argument");
    if (m->B != 1) return fail(OCMP_ERR_ARG, "ocmp_assemble_matrix: batched matrix, use ocmp_assemble_matrix_batch");
    if (f->wind_kind == OCMP_WIND_VERTEX && !f->wind_vtx)
        return fail(OCMP_ERR_ARG, "ocmp_assemble_matrix: per-vertex wind needs wind_vtx");
    return launch_assemble_matrix(m, f, (cudaStream_t)stream);
}

int ocmp_assemble_matrix_batch(ocmp_matrix_t m, const ocmp_form_t* forms, void* stream) {
    if (m && m->space->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_assemble_matrix_batch: compound space (ocmp_th_assemble)");
    if (!m || !forms) return fail(OCMP_ERR_ARG, "ocmp_assemble_matrix_batch: null argument");
    const ocmp_space_s* s = m->space;
    for (int q = 0; q < m->B; q++) {
        if (forms[q].wind_kind == OCMP_WIND_VERTEX && !forms[q].wind_vtx)
            return fail(OCMP_ERR_ARG, "ocmp_assemble_matrix_batch: per-vertex wind needs wind_vtx");
        // a single-instance view of instance q
        ocmp_matrix_s v;
        v.space = m->space;
        v.flags = m->flags;
        v.vals = m->vals + q * s->nnz;
        v.vals32 = m->vals32 ? m->vals32 + q * s->nnz : nullptr;
        v.svals64 = m->svals64 ? m->svals64 + q * s->nnz : nullptr;
        v.svals32 = m->svals32 ? m->svals32 + q * s->nnz : nullptr;
        v.dinv = m->dinv ? m->dinv + q * s->ndof : nullptr;
        v.dinv32 = m->dinv32 ? m->dinv32 + q * s->ndof : nullptr;
        const int st = launch_assemble_matrix(&v, &forms[q], (cudaStream_t)stream);
        if (st) return st;
    }
    return OCMP_OK;
}

int ocmp_assemble_rhs(ocmp_space_t s, const ocmp_form_t* f, const ocmp_rhs_t* r, double* b, void* stream) {
    if (s && s->kind == OCMP_COMPOUND) return fail(OCMP_ERR_UNSUPPORTED, "ocmp_assemble_rhs: compound space");
    if (!s || !f || !r || !b) return fail(OCMP_ERR_ARG, "ocmp_assemble_rhs: null argument");
    if (r->src_kind == OCMP_SRC_QP && !r->src_qp) return fail(OCMP_ERR_ARG, "ocmp_assemble_rhs: src_qp is null");
    return launch_assemble_rhs(s, f, r, b, (cudaStream_t)stream);
}

int ocmp_matrix_autotune(ocmp_matrix_t m, const double* x, double* y, void* stream, int32_t* tpr, int32_t* unroll,
                         float* ms) {
    if (!m || !x || !y) return fail(OCMP_ERR_ARG, "ocmp_matrix_autotune: null argument");
    return autotune_spmv(m->space, m->vals, x, y, (cudaStream_t)stream, 10, tpr, unroll, ms);
}

int ocmp_spmv(ocmp_matrix_t m, const double* x, double* y, void* stream) {
    if (!m || !x || !y) return fail(OCMP_ERR_ARG, "ocmp_spmv: null argument");
    return launch_spmv64(m->space, m->vals, x, y, (cudaStream_t)stream);
}

int ocmp_spmv_axpby(ocmp_matrix_t m, double alpha, const double* x, double beta, double* y, void* stream) {
    if (!m || !x || !y) return fail(OCMP_ERR_ARG, "ocmp_spmv_axpby: null argument");
    return launch_spmv_axpby(m->space, m->vals, alpha, x, beta, y, (cudaStream_t)stream);
}

}  // extern "C"

#ifdef OCMP_TERM_GENERATOR
// Build-time generator (opencmp_gb300/build.py): writes, for the H1 element types of the
// double-float path, the element-matrix term tables of build_terms as straight-line device code:
// per (dimension, local size, wind variant) four functions, each writing the entries of a quarter
// of the symmetric slots (quarters balanced by term count) through a store functor st(index, value),
// index = i * nloc + j, so one generated body serves any element-matrix layout. With every factor index and coefficient
// a compile-time constant, the factors live in registers and the products need no table loads.
#include <cstdio>

int main(int argc, char** argv) {
    if (argc < 2) return 1;
    FILE* o = std::fopen(argv[1], "w");
    if (!o) return 2;
    std::fprintf(o, "// Generated by ocmp_host.cpp (OCMP_TERM_GENERATOR) at build time; do not edit.\n#pragma once\n\n");
    const int cases[][2] = {{2, 1}, {2, 2}, {2, 3}, {3, 1}, {3, 2}};
    for (const auto& cs : cases) {
        const int D = cs[0], p = cs[1];
        ocmp_tables T;
        ocmp::build_tables(OCMP_H1, D, p, T);
        ocmp::build_terms(OCMP_H1, D, p, T);
        const int L = T.nloc, NP = D + 1, NS = NP * (NP + 1) / 2;
        for (int var = 0; var < 2; var++) {
            const int NG = 1 + NS + (var ? NP * NP : NP);
            const auto& off = T.slot_off[var];
            const auto& tg = T.term_g[var];
            const auto& tc = T.term_coef[var];
            auto emit = [&](const char* acc, int a, int b) {
                for (int t = a; t < b; t++) {
                    const double c = tc[t];
                    const float hi = (float)c, lo = (float)(c - (double)hi);
                    uint32_t hb, lb;
                    std::memcpy(&hb, &hi, 4);
                    std::memcpy(&lb, &lo, 4);
                    std::fprintf(o, "        gterm(%sh, %sl, F[%d], __uint_as_float(0x%08xu), __uint_as_float(0x%08xu));\n", acc,
                                 acc, (int)tg[t], hb, lb);
                }
            };
            // the slots in (i <= j) order, split where the terms reach each quarter of the total:
            // run0 .. run3 write the entries of one quarter each (four threads per element)
            std::vector<int> si, sj;
            for (int i = 0; i < L; i++)
                for (int j = i; j < L; j++) {
                    si.push_back(i);
                    sj.push_back(j);
                }
            const int nsl = (int)si.size();
            const int total = off[4 * nsl];
            // slot boundaries at each quarter of the terms
            int cut[5] = {0, 0, 0, 0, nsl};
            for (int q = 1; q < 4; q++) {
                int c = cut[q - 1];
                while (c < nsl && off[4 * c] < (int64_t)total * q / 4) c++;
                cut[q] = c;
            }
            auto emit_slots = [&](const char* name, int s0, int s1) {
                std::fprintf(o, "    template <class ST>\n    static __device__ __forceinline__ void %s(const float2 (&F)[%d], ST& st) {\n",
                             name, NG);
                for (int slot = s0; slot < s1; slot++) {
                    const int i = si[slot], j = sj[slot];
                    const int o0 = off[4 * slot], o2 = off[4 * slot + 2], o3 = off[4 * slot + 3], o4 = off[4 * slot + 4];
                    std::fprintf(o, "        {\n        float sh = 0.f, sl = 0.f;\n");
                    emit("s", o0, o2);
                    std::fprintf(o, "        float ah = sh, al = sl;\n");
                    emit("a", o2, o3);
                    std::fprintf(o, "        st(%d, make_float2(ah, al));\n", i * L + j);
                    if (j != i) {
                        std::fprintf(o, "        float bh = sh, bl = sl;\n");
                        emit("b", o3, o4);
                        std::fprintf(o, "        st(%d, make_float2(bh, bl));\n", j * L + i);
                    }
                    std::fprintf(o, "        }\n");
                }
                std::fprintf(o, "    }\n");
            };
            std::fprintf(o, "template <> struct GenTerms<%d, %d, %d> {\n    static constexpr bool value = true;\n"
                            "    static constexpr int NG = %d;\n",
                         D, L, var, NG);
            emit_slots("run0", cut[0], cut[1]);
            emit_slots("run1", cut[1], cut[2]);
            emit_slots("run2", cut[2], cut[3]);
            emit_slots("run3", cut[3], cut[4]);
            std::fprintf(o, "};\n\n");
        }
    }
    std::fclose(o);
    return 0;
}
#endif
