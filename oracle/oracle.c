/*
 * CPU oracle for the OpenCMP finite-element hot path. TEST INFRASTRUCTURE ONLY: see oracle.h.
 *
 * Everything here is computed the direct way, so that it checks the GPU library rather than
 * mirrors it: element matrices by quadrature at each point with the basis evaluated through
 * forward-mode dual numbers (the GPU path contracts precomputed reference tensors instead), a
 * row-wise CSR build by per-row sort/unique, and textbook CG / restarted GMRES with modified
 * Gram-Schmidt (the GPU path uses classical Gram-Schmidt with re-orthogonalisation).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXLOC 24
#define MAXQ 512

/* ---------------------------------------------------------------- dual numbers (value + grad) */
typedef struct { double v, d[3]; } dn;
static dn dc(double c) { dn r = {c, {0, 0, 0}}; return r; }
static dn dadd(dn a, dn b) { dn r = {a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}}; return r; }
static dn dsub(dn a, dn b) { dn r = {a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}}; return r; }
static dn dscale(dn a, double s) { dn r = {a.v * s, {a.d[0] * s, a.d[1] * s, a.d[2] * s}}; return r; }
static dn dmul(dn a, dn b) {
    dn r = {a.v * b.v, {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1], a.d[2] * b.v + a.v * b.d[2]}};
    return r;
}

/* scaled Legendre L_k(x, t) = t^k P_k(x / t), k = 0..n (Bonnet recurrence in homogeneous form) */
static void scaled_legendre(int n, dn x, dn t, dn* out) {
    out[0] = dc(1.0);
    if (n >= 1) out[1] = x;
    dn t2 = dmul(t, t);
    for (int k = 1; k < n; k++)
        out[k + 1] = dscale(dsub(dscale(dmul(x, out[k]), 2.0 * k + 1.0), dscale(dmul(t2, out[k - 1]), (double)k)),
                            1.0 / (k + 1.0));
}

/* Jacobi P_j^{(alpha,0)}(s), j = 0..n */
static void jacobi_a0(int n, double alpha, dn s, dn* out) {
    out[0] = dc(1.0);
    if (n >= 1) out[1] = dscale(dadd(dscale(s, alpha + 2.0), dc(alpha)), 0.5);
    for (int k = 2; k <= n; k++) {
        double a = 2.0 * k * (k + alpha) * (2.0 * k + alpha - 2.0);
        double b = (2.0 * k + alpha - 1.0);
        double c1 = (2.0 * k + alpha) * (2.0 * k + alpha - 2.0);
        double c0 = alpha * alpha;
        double d = 2.0 * (k + alpha - 1.0) * (k - 1.0) * (2.0 * k + alpha);
        dn t1 = dscale(dmul(dadd(dscale(s, c1), dc(c0)), out[k - 1]), b);
        out[k] = dscale(dsub(t1, dscale(out[k - 2], d)), 1.0 / a);
    }
}

static int h1_nloc(int D, int p) { return D == 2 ? (p + 1) * (p + 2) / 2 : (p + 1) * (p + 2) * (p + 3) / 6; }

/* barycentric coordinates with reference gradients: lam0 = 1 - sum xi, lam_{k+1} = xi_k */
static void barycentric(int D, const double* xi, dn* lam) {
    lam[0] = dc(1.0);
    for (int k = 0; k < D; k++) {
        lam[0].v -= xi[k];
        lam[0].d[k] = -1.0;
        lam[k + 1] = dc(xi[k]);
        lam[k + 1].d[k] = 1.0;
    }
}

/* Hierarchical H1 basis of order p <= 3: vertex functions lam_v; edge functions
   lam_a lam_b L_k(lam_b - lam_a, lam_a + lam_b), k = 0..p-2, edges (a<b) lexicographic;
   face bubbles lam_a lam_b lam_c (p = 3), faces (a<b<c) lexicographic. */
static int h1_eval(int D, int p, const double* xi, dn* out) {
    dn lam[4];
    barycentric(D, xi, lam);
    int c = 0;
    for (int v = 0; v <= D; v++) out[c++] = lam[v];
    if (p >= 2)
        for (int a = 0; a <= D; a++)
            for (int b = a + 1; b <= D; b++) {
                dn L[4];
                scaled_legendre(p - 2, dsub(lam[b], lam[a]), dadd(lam[a], lam[b]), L);
                dn base = dmul(lam[a], lam[b]);
                for (int k = 0; k <= p - 2; k++) out[c++] = dmul(base, L[k]);
            }
    if (p >= 3)
        for (int a = 0; a <= D; a++)
            for (int b = a + 1; b <= D; b++)
                for (int cc = b + 1; cc <= D; cc++) out[c++] = dmul(dmul(lam[a], lam[b]), lam[cc]);
    return c;
}

/* Dubiner basis on the triangle: psi_ij = L_i(lam1 - lam0, lam0 + lam1) P_j^{(2i+1,0)}(2 lam2 - 1) */
static int l2_eval(int D, int p, const double* xi, dn* out) {
    (void)D;
    dn lam[4];
    barycentric(2, xi, lam);
    dn L[8];
    scaled_legendre(p, dsub(lam[1], lam[0]), dadd(lam[0], lam[1]), L);
    int c = 0;
    for (int i = 0; i <= p; i++) {
        dn P[8];
        jacobi_a0(p - i, 2.0 * i + 1.0, dsub(dscale(lam[2], 2.0), dc(1.0)), P);
        for (int j = 0; j <= p - i; j++) out[c++] = dmul(L[i], P[j]);
    }
    return c;
}

/* ---------------------------------------------------------------- quadrature */
static void gauss01(int n, double* x, double* w) {
    for (int i = 0; i < n; i++) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = 0.0;
            for (int k = 1; k <= n; k++) {
                double p2 = p1;
                p1 = p0;
                p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
            }
            pp = n * (z * p0 - p1) / (z * z - 1.0);
            double dz = p0 / pp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        x[i] = 0.5 * (1.0 - z);
        w[i] = 1.0 / ((1.0 - z * z) * pp * pp);
    }
}

/* collapsed (conical product) Gauss rule on the reference simplex of dimension D, n points per
   direction; exact for total degree 2n - 1 - (D - 1) */
static int simplex_rule(int D, int n, double* pts, double* wts) {
    double x[32], w[32];
    gauss01(n, x, w);
    int q = 0;
    if (D == 1) {
        for (int i = 0; i < n; i++) { pts[q] = x[i]; wts[q++] = w[i]; }
    } else if (D == 2) {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                pts[2 * q] = x[i];
                pts[2 * q + 1] = x[j] * (1.0 - x[i]);
                wts[q++] = w[i] * w[j] * (1.0 - x[i]);
            }
    } else {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++) {
                    pts[3 * q] = x[i];
                    pts[3 * q + 1] = x[j] * (1.0 - x[i]);
                    pts[3 * q + 2] = x[k] * (1.0 - x[i]) * (1.0 - x[j]);
                    wts[q++] = w[i] * w[j] * w[k] * (1.0 - x[i]) * (1.0 - x[i]) * (1.0 - x[j]);
                }
    }
    return q;
}

/* ---------------------------------------------------------------- space */
typedef struct {
    int D, kind, p, nloc, nvp;
    int64_t nv, ne, ndof, nnz, ned, nfc, nif, nbf;
    double* X;
    int32_t* conn;
    int32_t* dofs;
    int64_t* rowptr;
    int32_t* col;
    uint8_t* freed;
    int32_t* ifac; /* nif x 4: eL, fL, eR, fR   (local facet f = facet opposite local vertex f) */
    int32_t* bfac; /* nbf x 3: e, f, label */
    int nq;
    double qp[MAXQ * 3], qw[MAXQ];
    int nfq;
    double fqp[MAXQ * 2], fqw[MAXQ];
} or_sp;

static int cmp_i64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return x < y ? -1 : x > y;
}
static int cmp_i32(const void* a, const void* b) {
    int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return x < y ? -1 : x > y;
}
static int64_t find_i64(const int64_t* a, int64_t n, int64_t key) {
    int64_t lo = 0, hi = n - 1;
    while (lo <= hi) {
        int64_t m = (lo + hi) / 2;
        if (a[m] == key) return m;
        if (a[m] < key) lo = m + 1; else hi = m - 1;
    }
    return -1;
}
static int64_t find_col(const int32_t* c, int64_t lo, int64_t hi, int32_t key) {
    hi -= 1;
    while (lo <= hi) {
        int64_t m = (lo + hi) / 2;
        if (c[m] == key) return m;
        if (c[m] < key) lo = m + 1; else hi = m - 1;
    }
    return -1;
}

/* facet key of local facet f (vertices other than f) of element e, sorted ascending */
static int64_t facet_key(const or_sp* s, int64_t e, int f) {
    int64_t k = 0;
    for (int v = 0; v < s->nvp; v++)
        if (v != f) k = k * s->nv + s->conn[e * s->nvp + v];
    return k;
}

void* or_space_create(int D, int kind, int p, int64_t nv, const double* coords, int64_t ne, const int32_t* conn,
                      int64_t nbf, const int32_t* bfacets, const int32_t* blabels, uint32_t dirichlet_mask) {
    if ((D != 2 && D != 3) || p < 1 || p > 3 || (kind == OR_L2 && D != 2)) return NULL;
    or_sp* s = (or_sp*)calloc(1, sizeof(or_sp));
    s->D = D; s->kind = kind; s->p = p; s->nv = nv; s->ne = ne; s->nvp = D + 1;
    s->nloc = h1_nloc(D, p);
    s->X = (double*)malloc(sizeof(double) * nv * D);
    memcpy(s->X, coords, sizeof(double) * nv * D);
    s->conn = (int32_t*)malloc(sizeof(int32_t) * ne * (D + 1));
    memcpy(s->conn, conn, sizeof(int32_t) * ne * (D + 1));
    for (int64_t e = 0; e < ne; e++) qsort(s->conn + e * (D + 1), D + 1, sizeof(int32_t), cmp_i32);
    s->nq = simplex_rule(D, p + 2, s->qp, s->qw);
    s->nfq = simplex_rule(D - 1, p + 2, s->fqp, s->fqw);
    const int nvp = D + 1, nloc = s->nloc;

    /* edges and faces (global, sorted by vertex tuple) */
    int ne_loc = D == 2 ? 3 : 6, nf_loc = D == 2 ? 1 : 4;
    int64_t* ekeys = NULL; int64_t* fkeys = NULL;
    if (kind == OR_H1 && p >= 2) {
        ekeys = (int64_t*)malloc(sizeof(int64_t) * ne * ne_loc);
        for (int64_t e = 0; e < ne; e++) {
            int c = 0;
            for (int a = 0; a < nvp; a++)
                for (int b = a + 1; b < nvp; b++)
                    ekeys[e * ne_loc + c++] = (int64_t)s->conn[e * nvp + a] * nv + s->conn[e * nvp + b];
        }
        qsort(ekeys, ne * ne_loc, sizeof(int64_t), cmp_i64);
        int64_t m = 0;
        for (int64_t i = 0; i < ne * ne_loc; i++)
            if (i == 0 || ekeys[i] != ekeys[i - 1]) ekeys[m++] = ekeys[i];
        s->ned = m;
    }
    if (kind == OR_H1 && p >= 3) {
        fkeys = (int64_t*)malloc(sizeof(int64_t) * ne * nf_loc);
        for (int64_t e = 0; e < ne; e++) {
            int c = 0;
            for (int a = 0; a < nvp; a++)
                for (int b = a + 1; b < nvp; b++)
                    for (int cc = b + 1; cc < nvp; cc++)
                        fkeys[e * nf_loc + c++] = ((int64_t)s->conn[e * nvp + a] * nv + s->conn[e * nvp + b]) * nv +
                                                  s->conn[e * nvp + cc];
        }
        qsort(fkeys, ne * nf_loc, sizeof(int64_t), cmp_i64);
        int64_t m = 0;
        for (int64_t i = 0; i < ne * nf_loc; i++)
            if (i == 0 || fkeys[i] != fkeys[i - 1]) fkeys[m++] = fkeys[i];
        s->nfc = m;
    }
    /* element dof map */
    s->dofs = (int32_t*)malloc(sizeof(int32_t) * ne * nloc);
    if (kind == OR_L2) {
        s->ndof = ne * nloc;
        for (int64_t e = 0; e < ne; e++)
            for (int i = 0; i < nloc; i++) s->dofs[e * nloc + i] = (int32_t)(e * nloc + i);
    } else {
        int epd = p - 1;
        s->ndof = nv + s->ned * epd + s->nfc * (p >= 3 ? 1 : 0);
        for (int64_t e = 0; e < ne; e++) {
            int c = 0;
            const int32_t* v = s->conn + e * nvp;
            for (int a = 0; a < nvp; a++) s->dofs[e * nloc + c++] = v[a];
            if (p >= 2)
                for (int a = 0; a < nvp; a++)
                    for (int b = a + 1; b < nvp; b++) {
                        int64_t id = find_i64(ekeys, s->ned, (int64_t)v[a] * nv + v[b]);
                        for (int k = 0; k < epd; k++) s->dofs[e * nloc + c++] = (int32_t)(nv + id * epd + k);
                    }
            if (p >= 3)
                for (int a = 0; a < nvp; a++)
                    for (int b = a + 1; b < nvp; b++)
                        for (int cc = b + 1; cc < nvp; cc++) {
                            int64_t id = find_i64(fkeys, s->nfc, ((int64_t)v[a] * nv + v[b]) * nv + v[cc]);
                            s->dofs[e * nloc + c++] = (int32_t)(nv + s->ned * epd + id);
                        }
        }
    }
    free(ekeys);
    free(fkeys);

    /* facets: interior pairs from sorting all element facets; boundary facets matched by key */
    int64_t nfl = ne * nvp;
    int64_t* fk = (int64_t*)malloc(sizeof(int64_t) * nfl * 2);
    for (int64_t e = 0; e < ne; e++)
        for (int f = 0; f < nvp; f++) {
            fk[2 * (e * nvp + f)] = facet_key(s, e, f);
            fk[2 * (e * nvp + f) + 1] = e * nvp + f;
        }
    /* sort pairs (key, id) by key then id */
    {
        /* simple merge-free approach: sort indices by key via qsort on 128-bit records */
        typedef struct { int64_t k, id; } rec;
        qsort(fk, nfl, sizeof(rec), cmp_i64); /* compares first int64 = key */
        /* stabilise equal keys by id */
        for (int64_t i = 0; i + 1 < nfl; i++)
            if (fk[2 * i] == fk[2 * i + 2] && fk[2 * i + 1] > fk[2 * i + 3]) {
                int64_t t = fk[2 * i + 1]; fk[2 * i + 1] = fk[2 * i + 3]; fk[2 * i + 3] = t;
            }
    }
    s->ifac = (int32_t*)malloc(sizeof(int32_t) * 4 * (nfl / 2 + 1));
    s->nif = 0;
    for (int64_t i = 0; i + 1 < nfl; i++)
        if (fk[2 * i] == fk[2 * i + 2]) {
            int64_t a = fk[2 * i + 1], b = fk[2 * i + 3];
            s->ifac[4 * s->nif + 0] = (int32_t)(a / nvp);
            s->ifac[4 * s->nif + 1] = (int32_t)(a % nvp);
            s->ifac[4 * s->nif + 2] = (int32_t)(b / nvp);
            s->ifac[4 * s->nif + 3] = (int32_t)(b % nvp);
            s->nif++;
            i++;
        }
    /* sort interior facets by (eL, fL) so the order is the element-major order */
    s->nbf = nbf;
    s->bfac = (int32_t*)malloc(sizeof(int32_t) * 3 * (nbf + 1));
    int64_t* keys_only = (int64_t*)malloc(sizeof(int64_t) * nfl);
    for (int64_t i = 0; i < nfl; i++) keys_only[i] = fk[2 * i];
    for (int64_t b = 0; b < nbf; b++) {
        int32_t vv[3];
        for (int k = 0; k < D; k++) vv[k] = bfacets[b * D + k];
        qsort(vv, D, sizeof(int32_t), cmp_i32);
        int64_t key = 0;
        for (int k = 0; k < D; k++) key = key * nv + vv[k];
        int64_t pos = find_i64(keys_only, nfl, key);
        while (pos > 0 && keys_only[pos - 1] == key) pos--;
        int64_t id = pos >= 0 ? fk[2 * pos + 1] : -1;
        s->bfac[3 * b + 0] = (int32_t)(id >= 0 ? id / nvp : -1);
        s->bfac[3 * b + 1] = (int32_t)(id >= 0 ? id % nvp : -1);
        s->bfac[3 * b + 2] = blabels[b];
    }
    free(keys_only);
    free(fk);

    /* free dofs: every dof of a Dirichlet-labelled boundary facet is constrained (H1 only) */
    s->freed = (uint8_t*)malloc(s->ndof);
    memset(s->freed, 1, s->ndof);
    if (kind == OR_H1) {
        for (int64_t b = 0; b < nbf; b++) {
            int lab = s->bfac[3 * b + 2];
            if (lab < 0 || lab >= 32 || !((dirichlet_mask >> lab) & 1u) || s->bfac[3 * b] < 0) continue;
            int64_t e = s->bfac[3 * b];
            int f = s->bfac[3 * b + 1];
            /* a local function lives on the facet iff it does not involve vertex f */
            int c = 0;
            for (int a = 0; a < nvp; a++, c++)
                if (a != f) s->freed[s->dofs[e * nloc + c]] = 0;
            if (p >= 2)
                for (int a = 0; a < nvp; a++)
                    for (int bb = a + 1; bb < nvp; bb++)
                        for (int k = 0; k < p - 1; k++, c++)
                            if (a != f && bb != f) s->freed[s->dofs[e * nloc + c]] = 0;
            if (p >= 3)
                for (int a = 0; a < nvp; a++)
                    for (int bb = a + 1; bb < nvp; bb++)
                        for (int cc = bb + 1; cc < nvp; cc++, c++)
                            if (a != f && bb != f && cc != f) s->freed[s->dofs[e * nloc + c]] = 0;
        }
    }

    /* pattern: per row, union of the dofs of all incident elements (+ facet neighbours for L2) */
    int64_t nd = s->ndof;
    int64_t* cnt = (int64_t*)calloc(nd + 1, sizeof(int64_t));
    for (int64_t i = 0; i < ne * nloc; i++) cnt[s->dofs[i] + 1]++;
    for (int64_t i = 0; i < nd; i++) cnt[i + 1] += cnt[i];
    int64_t* inc = (int64_t*)malloc(sizeof(int64_t) * ne * nloc);
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * nd);
    memcpy(fill, cnt, sizeof(int64_t) * nd);
    for (int64_t i = 0; i < ne * nloc; i++) inc[fill[s->dofs[i]]++] = i / nloc;
    free(fill);
    /* element neighbours for L2 */
    int32_t* nbr = NULL;
    if (kind == OR_L2) {
        nbr = (int32_t*)malloc(sizeof(int32_t) * ne * nvp);
        for (int64_t i = 0; i < ne * nvp; i++) nbr[i] = -1;
        for (int64_t f = 0; f < s->nif; f++) {
            nbr[(int64_t)s->ifac[4 * f] * nvp + s->ifac[4 * f + 1]] = s->ifac[4 * f + 2];
            nbr[(int64_t)s->ifac[4 * f + 2] * nvp + s->ifac[4 * f + 3]] = s->ifac[4 * f];
        }
    }
    int64_t* rl = (int64_t*)calloc(nd + 1, sizeof(int64_t));
    int maxcand = 0;
    for (int64_t r = 0; r < nd; r++) {
        int c = (int)(cnt[r + 1] - cnt[r]) * nloc * (kind == OR_L2 ? (nvp + 1) : 1);
        if (c > maxcand) maxcand = c;
    }
    int32_t** rows = (int32_t**)malloc(sizeof(int32_t*) * nd);
#pragma omp parallel
    {
        int32_t* buf = (int32_t*)malloc(sizeof(int32_t) * (maxcand + 1));
#pragma omp for schedule(dynamic, 1024)
        for (int64_t r = 0; r < nd; r++) {
            int m = 0;
            for (int64_t k = cnt[r]; k < cnt[r + 1]; k++) {
                int64_t e = inc[k];
                for (int j = 0; j < nloc; j++) buf[m++] = s->dofs[e * nloc + j];
                if (kind == OR_L2)
                    for (int f = 0; f < nvp; f++) {
                        int32_t o = nbr[e * nvp + f];
                        if (o >= 0)
                            for (int j = 0; j < nloc; j++) buf[m++] = s->dofs[(int64_t)o * nloc + j];
                    }
            }
            qsort(buf, m, sizeof(int32_t), cmp_i32);
            int u = 0;
            for (int i = 0; i < m; i++)
                if (i == 0 || buf[i] != buf[i - 1]) buf[u++] = buf[i];
            rows[r] = (int32_t*)malloc(sizeof(int32_t) * (u + 1));
            memcpy(rows[r], buf, sizeof(int32_t) * u);
            rl[r + 1] = u;
        }
        free(buf);
    }
    for (int64_t r = 0; r < nd; r++) rl[r + 1] += rl[r];
    s->nnz = rl[nd];
    s->rowptr = rl;
    s->col = (int32_t*)malloc(sizeof(int32_t) * (s->nnz + 1));
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < nd; r++) {
        memcpy(s->col + rl[r], rows[r], sizeof(int32_t) * (rl[r + 1] - rl[r]));
        free(rows[r]);
    }
    free(rows);
    free(cnt);
    free(inc);
    free(nbr);
    return s;
}

void or_space_destroy(void* sp) {
    or_sp* s = (or_sp*)sp;
    if (!s) return;
    free(s->X); free(s->conn); free(s->dofs); free(s->rowptr); free(s->col); free(s->freed);
    free(s->ifac); free(s->bfac);
    free(s);
}
int64_t or_space_ndof(void* sp) { return ((or_sp*)sp)->ndof; }
int64_t or_space_nnz(void* sp) { return ((or_sp*)sp)->nnz; }
int or_space_nloc(void* sp) { return ((or_sp*)sp)->nloc; }
int64_t or_space_ninterior_facets(void* sp) { return ((or_sp*)sp)->nif; }
void or_space_get_dofs(void* sp, int32_t* d) { or_sp* s = (or_sp*)sp; memcpy(d, s->dofs, sizeof(int32_t) * s->ne * s->nloc); }
void or_space_get_sorted_conn(void* sp, int32_t* c) { or_sp* s = (or_sp*)sp; memcpy(c, s->conn, sizeof(int32_t) * s->ne * s->nvp); }
void or_space_get_pattern(void* sp, int64_t* rp, int32_t* col) {
    or_sp* s = (or_sp*)sp;
    memcpy(rp, s->rowptr, sizeof(int64_t) * (s->ndof + 1));
    memcpy(col, s->col, sizeof(int32_t) * s->nnz);
}
void or_space_get_free(void* sp, uint8_t* f) { or_sp* s = (or_sp*)sp; memcpy(f, s->freed, s->ndof); }
void or_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---------------------------------------------------------------- geometry and evaluation */
typedef struct { double J[3][3], Ji[3][3], det, adet; double x0[3]; } geo;

static void elem_geo(const or_sp* s, int64_t e, geo* g) {
    int D = s->D;
    const int32_t* v = s->conn + e * s->nvp;
    for (int r = 0; r < D; r++) {
        g->x0[r] = s->X[(int64_t)v[0] * D + r];
        for (int c = 0; c < D; c++) g->J[r][c] = s->X[(int64_t)v[c + 1] * D + r] - g->x0[r];
    }
    if (D == 2) {
        g->det = g->J[0][0] * g->J[1][1] - g->J[0][1] * g->J[1][0];
        g->Ji[0][0] = g->J[1][1] / g->det; g->Ji[0][1] = -g->J[0][1] / g->det;
        g->Ji[1][0] = -g->J[1][0] / g->det; g->Ji[1][1] = g->J[0][0] / g->det;
    } else {
        double (*a)[3] = g->J;
        double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
        double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
        double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
        g->det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
        double id = 1.0 / g->det;
        g->Ji[0][0] = c00 * id;
        g->Ji[1][0] = c01 * id;
        g->Ji[2][0] = c02 * id;
        g->Ji[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
        g->Ji[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * id;
        g->Ji[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
        g->Ji[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * id;
        g->Ji[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
        g->Ji[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * id;
    }
    g->adet = fabs(g->det);
}

/* basis values and physical gradients at reference point xi */
static int eval_phys(const or_sp* s, const geo* g, const double* xi, double* val, double (*grad)[3]) {
    dn b[MAXLOC];
    int n = s->kind == OR_H1 ? h1_eval(s->D, s->p, xi, b) : l2_eval(s->D, s->p, xi, b);
    for (int i = 0; i < n; i++) {
        val[i] = b[i].v;
        for (int r = 0; r < s->D; r++) {
            double acc = 0;
            for (int c = 0; c < s->D; c++) acc += g->Ji[c][r] * b[i].d[c];
            grad[i][r] = acc;
        }
    }
    return n;
}

static void ref_to_phys(const or_sp* s, const geo* g, const double* xi, double* x) {
    for (int r = 0; r < s->D; r++) {
        x[r] = g->x0[r];
        for (int c = 0; c < s->D; c++) x[r] += g->J[r][c] * xi[c];
    }
}
static void phys_to_ref(const or_sp* s, const geo* g, const double* x, double* xi) {
    for (int c = 0; c < s->D; c++) {
        xi[c] = 0;
        for (int r = 0; r < s->D; r++) xi[c] += g->Ji[c][r] * (x[r] - g->x0[r]);
    }
}

static void wind_at(const or_sp* s, const or_form* f, int64_t e, const double* xi, double* w) {
    int D = s->D;
    for (int k = 0; k < 3; k++) w[k] = 0;
    if (f->wind_kind == OR_WIND_CONST) {
        for (int k = 0; k < D; k++) w[k] = f->wind[k];
    } else if (f->wind_kind == OR_WIND_VERTEX) {
        double lam[4];
        lam[0] = 1.0;
        for (int k = 0; k < D; k++) { lam[k + 1] = xi[k]; lam[0] -= xi[k]; }
        for (int v = 0; v <= D; v++) {
            int32_t gv = s->conn[e * s->nvp + v];
            for (int k = 0; k < D; k++) w[k] += lam[v] * f->wind_vtx[(int64_t)gv * D + k];
        }
    }
}

static double source_at(int kind, const double* sp, int D, const double* x) {
    switch (kind) {
    case OR_SRC_CONST: return sp[0];
    case OR_SRC_SINPROD: {
        double v = sp[0];
        for (int k = 0; k < D; k++) v *= sin(M_PI * x[k]);
        return v;
    }
    case OR_SRC_GAUSS: {
        double r2 = 0;
        for (int k = 0; k < D; k++) r2 += (x[k] - sp[1 + k]) * (x[k] - sp[1 + k]);
        return sp[0] * exp(-r2 / (2.0 * sp[4] * sp[4]));
    }
    case OR_SRC_POLY_X1MX: return sp[0] * x[0] * (1.0 - x[0]);
    default: return 0.0;
    }
}

/* ---------------------------------------------------------------- element and facet matrices */
void or_element_matrix(void* sp, const or_form* f, int64_t e, double* K) {
    or_sp* s = (or_sp*)sp;
    int n = s->nloc, D = s->D;
    geo g;
    elem_geo(s, e, &g);
    memset(K, 0, sizeof(double) * n * n);
    double val[MAXLOC], grad[MAXLOC][3], w[3];
    for (int q = 0; q < s->nq; q++) {
        eval_phys(s, &g, s->qp + q * D, val, grad);
        wind_at(s, f, e, s->qp + q * D, w);
        double wq = s->qw[q] * g.adet;
        for (int i = 0; i < n; i++) {
            double wg = 0;
            for (int k = 0; k < D; k++) wg += w[k] * grad[i][k];
            for (int j = 0; j < n; j++) {
                double gg = 0;
                for (int k = 0; k < D; k++) gg += grad[i][k] * grad[j][k];
                K[i * n + j] += wq * (f->mass * val[i] * val[j] + f->dt * f->diff * gg - f->dt * val[j] * wg);
            }
        }
    }
}

/* physical point and facet data at facet quadrature point q of local facet lf of element e */
static void facet_point(const or_sp* s, const geo* g, int64_t e, int lf, int q, double* x, double* nrm, double* meas) {
    int D = s->D, nvp = s->nvp;
    int fv[3], c = 0;
    for (int v = 0; v < nvp; v++)
        if (v != lf) fv[c++] = s->conn[e * nvp + v];
    const double* P0 = s->X + (int64_t)fv[0] * D;
    const double* P1 = s->X + (int64_t)fv[1] * D;
    const double* Po = s->X + (int64_t)s->conn[e * nvp + lf] * D;
    if (D == 2) {
        double t = s->fqp[q];
        double tx = P1[0] - P0[0], ty = P1[1] - P0[1];
        double L = sqrt(tx * tx + ty * ty);
        x[0] = P0[0] + t * tx; x[1] = P0[1] + t * ty;
        nrm[0] = ty / L; nrm[1] = -tx / L;
        if ((Po[0] - P0[0]) * nrm[0] + (Po[1] - P0[1]) * nrm[1] > 0) { nrm[0] = -nrm[0]; nrm[1] = -nrm[1]; }
        *meas = L;
    } else {
        const double* P2 = s->X + (int64_t)fv[2] * D;
        double a[3], b[3], cr[3];
        for (int k = 0; k < 3; k++) { a[k] = P1[k] - P0[k]; b[k] = P2[k] - P0[k]; }
        cr[0] = a[1] * b[2] - a[2] * b[1]; cr[1] = a[2] * b[0] - a[0] * b[2]; cr[2] = a[0] * b[1] - a[1] * b[0];
        double L = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        double u = s->fqp[2 * q], v = s->fqp[2 * q + 1];
        for (int k = 0; k < 3; k++) { x[k] = P0[k] + u * a[k] + v * b[k]; nrm[k] = cr[k] / L; }
        double dd = 0;
        for (int k = 0; k < 3; k++) dd += (Po[k] - P0[k]) * nrm[k];
        if (dd > 0) for (int k = 0; k < 3; k++) nrm[k] = -nrm[k];
        *meas = L; /* |cross| = 2 * area; rule weights sum to 1/2 */
    }
    (void)g;
}

/* boundary facet matrix (nloc x nloc, rows = test) of element e, local facet lf, label lab */
static void bfacet_matrix(const or_sp* s, const or_form* f, int64_t e, int lf, int lab, double* K) {
    int n = s->nloc, D = s->D;
    memset(K, 0, sizeof(double) * n * n);
    uint32_t bit = 1u << lab;
    int has_out = (f->outflow_mask & bit) != 0, has_wn = (f->wn_mask & bit) != 0, has_nit = (f->nitsche_mask & bit) != 0;
    int has_rob = (f->robin_mask & bit) != 0;
    if (!has_out && !has_wn && !has_nit && !has_rob) return;
    geo g;
    elem_geo(s, e, &g);
    double h = pow(g.adet, 1.0 / D);
    double alpha = f->ipc * s->p * s->p / h;
    for (int q = 0; q < s->nfq; q++) {
        double x[3], nrm[3], meas, xi[3], val[MAXLOC], grad[MAXLOC][3], w[3];
        facet_point(s, &g, e, lf, q, x, nrm, &meas);
        phys_to_ref(s, &g, x, xi);
        eval_phys(s, &g, xi, val, grad);
        wind_at(s, f, e, xi, w);
        double wn = 0;
        for (int k = 0; k < D; k++) wn += w[k] * nrm[k];
        double wq = s->fqw[q] * meas * f->dt;
        for (int i = 0; i < n; i++) {
            double dni = 0;
            for (int k = 0; k < D; k++) dni += grad[i][k] * nrm[k];
            for (int j = 0; j < n; j++) {
                double dnj = 0;
                for (int k = 0; k < D; k++) dnj += grad[j][k] * nrm[k];
                double t = 0;
                if (has_out) t += val[i] * val[j] * (wn > 0 ? wn : 0.0);
                if (has_wn) t += val[i] * val[j] * wn;
                if (has_nit)
                    t += f->diff * (alpha * val[i] * val[j] - val[i] * dnj - val[j] * dni) + val[i] * val[j] * (wn > 0 ? wn : 0.0);
                /* Robin term of poisson.py:93-97, -dt dc r u v, with robin[lab] = -dc r */
                if (has_rob) t += f->robin[lab] * val[i] * val[j];
                K[i * n + j] += wq * t;
            }
        }
    }
}

/* interior facet matrix (2 nloc x 2 nloc; index < nloc: element L, else element R) */
static void ifacet_matrix(const or_sp* s, const or_form* f, int64_t fi, double* K) {
    int n = s->nloc, D = s->D, n2 = 2 * n;
    memset(K, 0, sizeof(double) * n2 * n2);
    int64_t eL = s->ifac[4 * fi], eR = s->ifac[4 * fi + 2];
    int lf = s->ifac[4 * fi + 1];
    geo gL, gR;
    elem_geo(s, eL, &gL);
    elem_geo(s, eR, &gR);
    double h = pow(gL.adet, 1.0 / D);
    double alpha = f->ipc * s->p * s->p / h;
    for (int q = 0; q < s->nfq; q++) {
        double x[3], nrm[3], meas, xL[3], xR[3], w[3];
        double v[2 * MAXLOC], gr[2 * MAXLOC][3];
        facet_point(s, &gL, eL, lf, q, x, nrm, &meas);
        phys_to_ref(s, &gL, x, xL);
        phys_to_ref(s, &gR, x, xR);
        eval_phys(s, &gL, xL, v, gr);
        eval_phys(s, &gR, xR, v + n, gr + n);
        wind_at(s, f, eL, xL, w);
        double wn = 0;
        for (int k = 0; k < D; k++) wn += w[k] * nrm[k];
        double wq = s->fqw[q] * meas * f->dt;
        for (int i = 0; i < n2; i++) {
            double si = i < n ? 1.0 : -1.0; /* jump sign */
            double jv = si * v[i];
            double avn = 0;
            for (int k = 0; k < D; k++) avn += 0.5 * gr[i][k] * nrm[k];
            for (int j = 0; j < n2; j++) {
                double sj = j < n ? 1.0 : -1.0;
                double ju = sj * v[j];
                double aun = 0;
                for (int k = 0; k < D; k++) aun += 0.5 * gr[j][k] * nrm[k];
                double t = f->diff * (alpha * ju * jv - aun * jv - avn * ju);
                double up = j < n ? v[j] * (wn > 0 ? wn : 0.0) : v[j] * (wn < 0 ? wn : 0.0);
                t += jv * up;
                K[i * n2 + j] += wq * t;
            }
        }
    }
}

static void add_block(or_sp* s, double* vals, const int32_t* rd, const int32_t* cd, int nr, int nc, const double* B) {
    for (int i = 0; i < nr; i++) {
        int32_t r = rd[i];
        for (int j = 0; j < nc; j++) {
            int64_t pos = find_col(s->col, s->rowptr[r], s->rowptr[r + 1], cd[j]);
            vals[pos] += B[i * nc + j];
        }
    }
}

int or_assemble_matrix(void* sp, const or_form* f, double* vals) {
    or_sp* s = (or_sp*)sp;
    int n = s->nloc;
    int64_t ne = s->ne, nd = s->ndof;
    double* Ke = (double*)malloc(sizeof(double) * ne * n * n);
    if (!Ke) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < ne; e++) or_element_matrix(sp, f, e, Ke + e * n * n);
    /* dof -> (element, local) incidence, then row-parallel accumulation */
    int64_t* cnt = (int64_t*)calloc(nd + 1, sizeof(int64_t));
    for (int64_t i = 0; i < ne * n; i++) cnt[s->dofs[i] + 1]++;
    for (int64_t i = 0; i < nd; i++) cnt[i + 1] += cnt[i];
    int64_t* inc = (int64_t*)malloc(sizeof(int64_t) * ne * n);
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * nd);
    memcpy(fill, cnt, sizeof(int64_t) * nd);
    for (int64_t i = 0; i < ne * n; i++) inc[fill[s->dofs[i]]++] = i;
    free(fill);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < nd; r++) {
        for (int64_t k = s->rowptr[r]; k < s->rowptr[r + 1]; k++) vals[k] = 0.0;
        for (int64_t k = cnt[r]; k < cnt[r + 1]; k++) {
            int64_t e = inc[k] / n;
            int i = (int)(inc[k] % n);
            for (int j = 0; j < n; j++) {
                int64_t pos = find_col(s->col, s->rowptr[r], s->rowptr[r + 1], s->dofs[e * n + j]);
                vals[pos] += Ke[(e * n + i) * n + j];
            }
        }
    }
    free(cnt);
    free(inc);
    free(Ke);
    /* facet terms */
    double* B = (double*)malloc(sizeof(double) * 4 * n * n);
    if (f->dg && s->kind == OR_L2) {
        int32_t dd[2 * MAXLOC];
        for (int64_t fi = 0; fi < s->nif; fi++) {
            ifacet_matrix(s, f, fi, B);
            for (int i = 0; i < n; i++) {
                dd[i] = s->dofs[(int64_t)s->ifac[4 * fi] * n + i];
                dd[n + i] = s->dofs[(int64_t)s->ifac[4 * fi + 2] * n + i];
            }
            add_block(s, vals, dd, dd, 2 * n, 2 * n, B);
        }
    }
    for (int64_t b = 0; b < s->nbf; b++) {
        if (s->bfac[3 * b] < 0) continue;
        int lab = s->bfac[3 * b + 2];
        if (lab < 0 || lab >= 32) continue;
        uint32_t bit = 1u << lab;
        if (!((f->outflow_mask | f->wn_mask | f->robin_mask | (s->kind == OR_L2 ? f->nitsche_mask : 0u)) & bit)) continue;
        or_form ff = *f;
        if (s->kind != OR_L2) ff.nitsche_mask = 0;
        bfacet_matrix(s, &ff, s->bfac[3 * b], s->bfac[3 * b + 1], lab, B);
        const int32_t* dd = s->dofs + (int64_t)s->bfac[3 * b] * n;
        add_block(s, vals, dd, dd, n, n, B);
    }
    free(B);
    return 0;
}

int or_assemble_rhs(void* sp, const or_form* f, const or_rhs* r, double* rhs) {
    or_sp* s = (or_sp*)sp;
    int n = s->nloc, D = s->D;
    memset(rhs, 0, sizeof(double) * s->ndof);
    double* Fe = (double*)calloc(s->ne * n, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < s->ne; e++) {
        geo g;
        elem_geo(s, e, &g);
        double val[MAXLOC], grad[MAXLOC][3], x[3];
        double up[MAXLOC];
        if (r->uprev)
            for (int j = 0; j < n; j++) up[j] = r->uprev[s->dofs[e * n + j]];
        for (int q = 0; q < s->nq; q++) {
            eval_phys(s, &g, s->qp + q * D, val, grad);
            ref_to_phys(s, &g, s->qp + q * D, x);
            double fq = r->src_kind != OR_SRC_NONE ? r->dt * source_at(r->src_kind, r->src, D, x) : 0.0;
            if (r->uprev) {
                double u = 0;
                for (int j = 0; j < n; j++) u += up[j] * val[j];
                fq += r->mass * u;
            }
            double wq = s->qw[q] * g.adet;
            for (int i = 0; i < n; i++) Fe[e * n + i] += wq * fq * val[i];
        }
    }
    for (int64_t e = 0; e < s->ne; e++)
        for (int i = 0; i < n; i++) rhs[s->dofs[e * n + i]] += Fe[e * n + i];
    free(Fe);
    /* boundary terms */
    for (int64_t b = 0; b < s->nbf; b++) {
        int64_t e = s->bfac[3 * b];
        if (e < 0) continue;
        int lf = s->bfac[3 * b + 1], lab = s->bfac[3 * b + 2];
        if (lab < 0 || lab >= 32) continue;
        uint32_t bit = 1u << lab;
        int has_b = (r->bval_mask & bit) != 0;
        int has_g = s->kind == OR_L2 && (f->nitsche_mask & bit) != 0;
        if (!has_b && !has_g) continue;
        geo g;
        elem_geo(s, e, &g);
        double h = pow(g.adet, 1.0 / D), alpha = f->ipc * s->p * s->p / h;
        for (int q = 0; q < s->nfq; q++) {
            double x[3], nrm[3], meas, xi[3], val[MAXLOC], grad[MAXLOC][3], w[3];
            facet_point(s, &g, e, lf, q, x, nrm, &meas);
            phys_to_ref(s, &g, x, xi);
            eval_phys(s, &g, xi, val, grad);
            wind_at(s, f, e, xi, w);
            double wn = 0;
            for (int k = 0; k < D; k++) wn += w[k] * nrm[k];
            double wq = s->fqw[q] * meas * r->dt;
            for (int i = 0; i < n; i++) {
                double t = 0;
                if (has_b) t += r->bval[lab] * val[i];
                if (has_g) {
                    double dni = 0;
                    for (int k = 0; k < D; k++) dni += grad[i][k] * nrm[k];
                    double gv = r->gval[lab];
                    t += f->diff * gv * (alpha * val[i] - dni) - val[i] * gv * (wn < 0 ? wn : 0.0);
                }
                rhs[s->dofs[e * n + i]] += wq * t;
            }
        }
    }
    return 0;
}

/* Dirichlet values: vertex dofs take g (constant per label); higher-order dofs on the facet 0 */
void or_set_boundary(void* sp, uint32_t mask, const double* gval, double* u) {
    or_sp* s = (or_sp*)sp;
    if (s->kind != OR_H1) return;
    int n = s->nloc, nvp = s->nvp;
    for (int64_t b = 0; b < s->nbf; b++) {
        int64_t e = s->bfac[3 * b];
        int lab = s->bfac[3 * b + 2];
        if (e < 0 || lab < 0 || lab >= 32 || !((mask >> lab) & 1u)) continue;
        int lf = s->bfac[3 * b + 1];
        int c = 0;
        for (int a = 0; a < nvp; a++, c++)
            if (a != lf) u[s->dofs[e * n + c]] = gval[lab];
        /* zero the edge / face dofs on the facet */
        c = nvp;
        if (s->p >= 2)
            for (int a = 0; a < nvp; a++)
                for (int bb = a + 1; bb < nvp; bb++)
                    for (int k = 0; k < s->p - 1; k++, c++)
                        if (a != lf && bb != lf) u[s->dofs[e * n + c]] = 0.0;
        if (s->p >= 3)
            for (int a = 0; a < nvp; a++)
                for (int bb = a + 1; bb < nvp; bb++)
                    for (int cc = bb + 1; cc < nvp; cc++, c++)
                        if (a != lf && bb != lf && cc != lf) u[s->dofs[e * n + c]] = 0.0;
    }
}

/* ---------------------------------------------------------------- linear algebra */
void or_spmv(int64_t n, const int64_t* rp, const int32_t* col, const double* val, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; r++) {
        double acc = 0;
        for (int64_t k = rp[r]; k < rp[r + 1]; k++) acc += val[k] * x[col[k]];
        y[r] = acc;
    }
}

static double dot_f(const or_sp* s, const double* a, const double* b) {
    double acc = 0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
    for (int64_t i = 0; i < s->ndof; i++)
        if (s->freed[i]) acc += a[i] * b[i];
    return acc;
}

/* residual on free dofs: r = (b - A x) restricted to free dofs, zero elsewhere */
static void resid(const or_sp* s, const double* vals, const double* b, const double* x, double* r) {
    or_spmv(s->ndof, s->rowptr, s->col, vals, x, r);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < s->ndof; i++) r[i] = s->freed[i] ? b[i] - r[i] : 0.0;
}

/* norm of the effective right-hand side (b - A x_D)_f, x_D = x with free entries zeroed */
static double rhs_norm(const or_sp* s, const double* vals, const double* b, const double* x) {
    double* xd = (double*)malloc(sizeof(double) * s->ndof);
    double* r = (double*)malloc(sizeof(double) * s->ndof);
    for (int64_t i = 0; i < s->ndof; i++) xd[i] = s->freed[i] ? 0.0 : x[i];
    resid(s, vals, b, xd, r);
    double nb = sqrt(dot_f(s, r, r));
    free(xd);
    free(r);
    return nb;
}

double or_relres(void* sp, const double* vals, const double* b, const double* x) {
    or_sp* s = (or_sp*)sp;
    double* r = (double*)malloc(sizeof(double) * s->ndof);
    resid(s, vals, b, x, r);
    double nr = sqrt(dot_f(s, r, r));
    double nb = rhs_norm(s, vals, b, x);
    free(r);
    return nb > 0 ? nr / nb : nr;
}

static void diag_inv(const or_sp* s, const double* vals, double* dinv) {
    for (int64_t r = 0; r < s->ndof; r++) {
        double d = 0;
        for (int64_t k = s->rowptr[r]; k < s->rowptr[r + 1]; k++)
            if (s->col[k] == r) d = vals[k];
        dinv[r] = (s->freed[r] && d != 0.0) ? 1.0 / d : 0.0;
    }
}

int or_cg(void* sp, const double* vals, const double* b, double* x, double tol, int maxit, int* iters, double* relres) {
    or_sp* s = (or_sp*)sp;
    int64_t n = s->ndof;
    double *r = malloc(8 * n), *z = malloc(8 * n), *p = malloc(8 * n), *q = malloc(8 * n), *dinv = malloc(8 * n);
    diag_inv(s, vals, dinv);
    double nb = rhs_norm(s, vals, b, x);
    if (nb == 0) nb = 1;
    resid(s, vals, b, x, r);
    for (int64_t i = 0; i < n; i++) { z[i] = dinv[i] * r[i]; p[i] = z[i]; }
    double rz = dot_f(s, r, z);
    double res = sqrt(dot_f(s, r, r)) / nb;
    int it = 0;
    while (res > tol && it < maxit) {
        or_spmv(n, s->rowptr, s->col, vals, p, q);
        for (int64_t i = 0; i < n; i++)
            if (!s->freed[i]) q[i] = 0;
        double alpha = rz / dot_f(s, p, q);
        for (int64_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
        for (int64_t i = 0; i < n; i++) z[i] = dinv[i] * r[i];
        double rz1 = dot_f(s, r, z);
        double beta = rz1 / rz;
        rz = rz1;
        for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        res = sqrt(dot_f(s, r, r)) / nb;
        it++;
    }
    /* report the true residual */
    *relres = or_relres(sp, vals, b, x);
    *iters = it;
    free(r); free(z); free(p); free(q); free(dinv);
    return *relres <= tol ? 0 : 1;
}

/* block-Jacobi blocks: element dof blocks (L2); for H1 falls back to point Jacobi */
static void block_inv(const or_sp* s, const double* vals, double* Binv) {
    int n = s->nloc;
    for (int64_t e = 0; e < s->ne; e++) {
        double A[MAXLOC][2 * MAXLOC];
        for (int i = 0; i < n; i++) {
            int32_t r = s->dofs[e * n + i];
            for (int j = 0; j < n; j++) {
                int64_t pos = find_col(s->col, s->rowptr[r], s->rowptr[r + 1], s->dofs[e * n + j]);
                A[i][j] = vals[pos];
                A[i][n + j] = (i == j);
            }
        }
        for (int c = 0; c < n; c++) {
            int pr = c;
            for (int i = c + 1; i < n; i++)
                if (fabs(A[i][c]) > fabs(A[pr][c])) pr = i;
            if (pr != c)
                for (int j = 0; j < 2 * n; j++) { double t = A[c][j]; A[c][j] = A[pr][j]; A[pr][j] = t; }
            double d = A[c][c];
            for (int j = 0; j < 2 * n; j++) A[c][j] /= d;
            for (int i = 0; i < n; i++)
                if (i != c) {
                    double m = A[i][c];
                    for (int j = 0; j < 2 * n; j++) A[i][j] -= m * A[c][j];
                }
        }
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) Binv[(e * n + i) * n + j] = A[i][n + j];
    }
}

static void apply_prec(const or_sp* s, int kind, const double* dinv, const double* Binv, const double* v, double* z) {
    int64_t nd = s->ndof;
    if (kind == 0) {
        for (int64_t i = 0; i < nd; i++) z[i] = s->freed[i] ? v[i] : 0.0;
    } else if (kind == 2 && Binv) {
        int n = s->nloc;
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < s->ne; e++)
            for (int i = 0; i < n; i++) {
                double acc = 0;
                for (int j = 0; j < n; j++) acc += Binv[(e * n + i) * n + j] * v[e * n + j];
                z[e * n + i] = acc;
            }
    } else {
        for (int64_t i = 0; i < nd; i++) z[i] = dinv[i] * v[i];
    }
}

int or_gmres(void* sp, const double* vals, const double* b, double* x, int m, int precond, double tol, int maxit,
             int* iters, double* relres) {
    or_sp* s = (or_sp*)sp;
    int64_t n = s->ndof;
    double* V = (double*)malloc(sizeof(double) * n * (m + 1));
    double* w = (double*)malloc(sizeof(double) * n);
    double* z = (double*)malloc(sizeof(double) * n);
    double* dinv = (double*)malloc(sizeof(double) * n);
    double* Binv = NULL;
    diag_inv(s, vals, dinv);
    if (precond == 2 && s->kind == OR_L2) {
        Binv = (double*)malloc(sizeof(double) * s->ne * s->nloc * s->nloc);
        block_inv(s, vals, Binv);
    }
    double* H = (double*)calloc((m + 1) * m, sizeof(double));
    double *cs = malloc(8 * m), *sn = malloc(8 * m), *g = malloc(8 * (m + 1)), *y = malloc(8 * m);
    double nb = rhs_norm(s, vals, b, x);
    if (nb == 0) nb = 1;
    int it = 0;
    double res = 0;
    for (;;) {
        resid(s, vals, b, x, V);
        double beta = sqrt(dot_f(s, V, V));
        res = beta / nb;
        if (res <= tol || it >= maxit) break;
        for (int64_t i = 0; i < n; i++) V[i] /= beta;
        for (int k = 0; k <= m; k++) g[k] = 0;
        g[0] = beta;
        int j;
        for (j = 0; j < m && it < maxit; j++, it++) {
            apply_prec(s, precond, dinv, Binv, V + j * n, z);
            or_spmv(n, s->rowptr, s->col, vals, z, w);
            for (int64_t i = 0; i < n; i++)
                if (!s->freed[i]) w[i] = 0;
            for (int k = 0; k <= j; k++) {
                double h = dot_f(s, w, V + k * n);
                H[k * m + j] = h;
                for (int64_t i = 0; i < n; i++) w[i] -= h * V[k * n + i];
            }
            double hn = sqrt(dot_f(s, w, w));
            H[(j + 1) * m + j] = hn;
            if (hn > 0)
                for (int64_t i = 0; i < n; i++) V[(j + 1) * n + i] = w[i] / hn;
            for (int k = 0; k < j; k++) {
                double a = H[k * m + j], bb = H[(k + 1) * m + j];
                H[k * m + j] = cs[k] * a + sn[k] * bb;
                H[(k + 1) * m + j] = -sn[k] * a + cs[k] * bb;
            }
            double a = H[j * m + j], bb = H[(j + 1) * m + j];
            double d = sqrt(a * a + bb * bb);
            cs[j] = a / d;
            sn[j] = bb / d;
            H[j * m + j] = d;
            H[(j + 1) * m + j] = 0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            if (fabs(g[j + 1]) / nb <= tol || hn == 0) { j++; it++; break; }
        }
        for (int k = j - 1; k >= 0; k--) {
            double acc = g[k];
            for (int l = k + 1; l < j; l++) acc -= H[k * m + l] * y[l];
            y[k] = acc / H[k * m + k];
        }
        for (int64_t i = 0; i < n; i++) w[i] = 0;
        for (int k = 0; k < j; k++)
            for (int64_t i = 0; i < n; i++) w[i] += y[k] * V[k * n + i];
        apply_prec(s, precond, dinv, Binv, w, z);
        for (int64_t i = 0; i < n; i++) x[i] += z[i];
    }
    *iters = it;
    *relres = or_relres(sp, vals, b, x);
    free(V); free(w); free(z); free(dinv); free(Binv); free(H); free(cs); free(sn); free(g); free(y);
    return *relres <= tol ? 0 : 1;
}

/* L2 projection of a built-in function onto the space (mass-matrix solve, all dofs) */
void or_project(void* sp, int src_kind, const double* src, double* u) {
    or_sp* s = (or_sp*)sp;
    or_form f;
    memset(&f, 0, sizeof(f));
    f.mass = 1.0;
    double* vals = (double*)malloc(sizeof(double) * s->nnz);
    or_assemble_matrix(sp, &f, vals);
    or_rhs r;
    memset(&r, 0, sizeof(r));
    r.dt = 1.0;
    r.src_kind = src_kind;
    memcpy(r.src, src, sizeof(double) * 8);
    double* b = (double*)malloc(sizeof(double) * s->ndof);
    or_assemble_rhs(sp, &f, &r, b);
    uint8_t* save = s->freed;
    s->freed = (uint8_t*)malloc(s->ndof);
    memset(s->freed, 1, s->ndof);
    for (int64_t i = 0; i < s->ndof; i++) u[i] = 0;
    int it;
    double rr;
    or_cg(sp, vals, b, u, 1e-14, 10000, &it, &rr);
    free(s->freed);
    s->freed = save;
    free(vals);
    free(b);
}

double or_l2_error(void* sp, const double* u, int src_kind, const double* src) {
    or_sp* s = (or_sp*)sp;
    int n = s->nloc, D = s->D;
    double acc = 0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
    for (int64_t e = 0; e < s->ne; e++) {
        geo g;
        elem_geo(s, e, &g);
        double val[MAXLOC], grad[MAXLOC][3], x[3];
        for (int q = 0; q < s->nq; q++) {
            eval_phys(s, &g, s->qp + q * D, val, grad);
            ref_to_phys(s, &g, s->qp + q * D, x);
            double uh = 0;
            for (int j = 0; j < n; j++) uh += u[s->dofs[e * n + j]] * val[j];
            double d = uh - source_at(src_kind, src, D, x);
            acc += s->qw[q] * g.adet * d * d;
        }
    }
    return sqrt(acc);
}

/* ---------------------------------------------------------------- reference tables (for the
 * numpy parts of the oracle: Taylor-Hood assembly in oracle/ins.py) */
int or_tabulate(int D, int kind, int p, int npts, const double* xi, double* vals, double* grads) {
    dn b[64];
    int L = 0;
    for (int q = 0; q < npts; q++) {
        L = kind == OR_H1 ? h1_eval(D, p, xi + (size_t)q * D, b) : l2_eval(D, p, xi + (size_t)q * D, b);
        for (int i = 0; i < L; i++) {
            vals[(size_t)q * L + i] = b[i].v;
            for (int k = 0; k < D; k++) grads[((size_t)q * L + i) * D + k] = b[i].d[k];
        }
    }
    return L;
}

int or_rule(int D, int n, double* pts, double* wts) { return simplex_rule(D, n, pts, wts); }
