/*
 * CPU oracle for the OpenCMP finite-element hot path (assembly into CSR + Krylov solve).
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker: the parity tests, the smoke check and the
 * CPU-baseline leg of bench.py call it. The product path (libopencmp_gpu.so) never links,
 * loads or calls anything declared here.
 *
 * It restates, in plain C with OpenMP, the weak forms OpenCMP builds and hands to NGSolve:
 *   - Poisson            opencmp/models/poisson.py:71-158
 *   - MultiComponentINS  opencmp/models/multi_component_ins.py:158-388 (velocity_fixed = True)
 *   - implicit Euler     opencmp/solvers/time_integration_schemes.py:79-132, 663-685 and
 *                        opencmp/models/base_model.py:418-497 (mass U*V, rhs u_n*V)
 *   - DG operators       opencmp/helpers/dg.py:22-83, alpha = ipc*p^2/h (base_model.py:150,
 *                        helpers/ngsolve_.py:48-70)
 *   - solve semantics    opencmp/models/base_model.py:886-947 (free dofs; direct solve on
 *                        L - A*gfu at 920-922; CG with initialize=False at 925-927; GMRes at 935-937)
 * The finite-element spaces (hierarchical H1 of order 1..3 on triangles and tetrahedra, Dubiner
 * L2 on triangles) and the DOF numbering are this project's documented conventions; NGSolve is a
 * third-party, unpinned dependency absent from the reference tree, so matrix-entry parity with it
 * is unpinned. The oracle is pinned at solution level against the reference's own fixtures
 * (pytests/full_system/poisson/transient_coarse, pytests/full_system/mcins/diffusion_convection)
 * and against manufactured solutions.
 */
#ifndef OPENCMP_ORACLE_H
#define OPENCMP_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { OR_H1 = 0, OR_L2 = 1 };
enum { OR_WIND_NONE = 0, OR_WIND_CONST = 1, OR_WIND_VERTEX = 2 };
enum { OR_SRC_NONE = 0, OR_SRC_CONST = 1, OR_SRC_SINPROD = 2, OR_SRC_GAUSS = 3, OR_SRC_POLY_X1MX = 4 };

typedef struct {
    double mass;            /* coefficient of  (u, v)                        (not scaled by dt) */
    double diff;            /* diffusion coefficient, term dt*diff*(grad u, grad v)               */
    double dt;              /* multiplies every term except the mass term                        */
    int wind_kind;          /* OR_WIND_*                                                          */
    double wind[3];         /* constant wind                                                      */
    const double* wind_vtx; /* per-vertex wind, nv*D, interpolated linearly (OR_WIND_VERTEX)      */
    double ipc;             /* interior penalty coefficient; nu = ipc * p^2, alpha = nu / h       */
    int dg;                 /* add interior-facet (skeleton) terms                                */
    uint32_t outflow_mask;  /* boundary labels carrying  dt * r c max(w.n, 0)                     */
    uint32_t wn_mask;       /* boundary labels carrying  dt * r c (w.n)   (MCINS Neumann half)    */
    uint32_t nitsche_mask;  /* DG Dirichlet labels: dt*diff*(alpha r c - r dc/dn - c dr/dn)
                               + dt*r c max(w.n,0)                                                */
    uint32_t robin_mask;    /* Robin labels: dt * robin[l] * r c  (poisson.py:93-97: -dt dc r u v) */
    double robin[32];
} or_form;

typedef struct {
    double dt;
    int src_kind;           /* OR_SRC_*                                                           */
    double src[8];          /* parameters of the source                                           */
    double mass;            /* coefficient of (u_prev, v)                                         */
    const double* uprev;    /* ndof or NULL                                                       */
    double bval[32];        /* per label: L += dt * bval * v on that boundary (Neumann-type)      */
    uint32_t bval_mask;
    double gval[32];        /* per label: DG Dirichlet datum g (constant)                         */
} or_rhs;

void* or_space_create(int D, int kind, int p, int64_t nv, const double* coords, int64_t ne,
                      const int32_t* conn, int64_t nbf, const int32_t* bfacets,
                      const int32_t* blabels, uint32_t dirichlet_mask);
void or_space_destroy(void* sp);
int64_t or_space_ndof(void* sp);
int64_t or_space_nnz(void* sp);
int or_space_nloc(void* sp);
int64_t or_space_ninterior_facets(void* sp);
void or_space_get_dofs(void* sp, int32_t* elem_dofs);
void or_space_get_sorted_conn(void* sp, int32_t* conn);
void or_space_get_pattern(void* sp, int64_t* rowptr, int32_t* col);
void or_space_get_free(void* sp, uint8_t* freedofs);

int or_assemble_matrix(void* sp, const or_form* f, double* vals);
int or_assemble_rhs(void* sp, const or_form* f, const or_rhs* r, double* rhs);
void or_element_matrix(void* sp, const or_form* f, int64_t e, double* Ke);
void or_set_boundary(void* sp, uint32_t mask, const double* gval_per_label, double* u);
void or_project(void* sp, int src_kind, const double* src, double* u);
double or_l2_error(void* sp, const double* u, int src_kind, const double* src);

void or_spmv(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val,
             const double* x, double* y);
int or_cg(void* sp, const double* vals, const double* b, double* x, double tol, int maxit,
          int* iters, double* relres);
int or_gmres(void* sp, const double* vals, const double* b, double* x, int restart, int precond,
             double tol, int maxit, int* iters, double* relres);
double or_relres(void* sp, const double* vals, const double* b, const double* x);
void or_set_threads(int n);

/* reference basis values (npts*L) and reference gradients (npts*L*D) at npts points; returns L */
int or_tabulate(int D, int kind, int p, int npts, const double* xi, double* vals, double* grads);
/* the collapsed simplex rule with n points per direction (n^D points, weights summing to 1/D!) */
int or_rule(int D, int n, double* pts, double* wts);

#ifdef __cplusplus
}
#endif
#endif
