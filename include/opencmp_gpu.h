/*
 * opencmp_gpu.h - C ABI of libopencmp_gpu.so, the GB300 (sm_103a) finite-element hot path behind
 * OpenCMP's Model/Solver plugin interface: form assembly into CSR followed by the Krylov solve.
 *
 * Plain C types only: host arrays are `const T*`, device arrays are raw device pointers (for
 * example `torch.Tensor.data_ptr()`), streams are `cudaStream_t` passed as `void*` (NULL = the
 * legacy default stream). Every function returns an ocmp_status; no exception crosses the ABI.
 * ocmp_last_error() returns the message of the last failure on the calling thread.
 *
 * Each entry point replaces one call OpenCMP makes into NGSolve (paths are relative to the
 * OpenCMP source tree):
 *   ocmp_mesh_create      <- opencmp/helpers/io.py:69-110        (load_mesh -> ngsolve.Mesh)
 *   ocmp_space_create     <- opencmp/models/poisson.py:60-65, multi_component_ins.py:95-117
 *                            (ngsolve.H1 / L2 (..., order, dirichlet, dgjumps); FESpace.FreeDofs)
 *   ocmp_assemble_matrix  <- opencmp/solvers/base_solver.py:368-377 (BilinearForm.Assemble) for the
 *                            forms of poisson.py:71-131 and multi_component_ins.py:158-300
 *   ocmp_assemble_rhs     <- base_solver.py:374-375 (LinearForm.Assemble) for poisson.py:133-158,
 *                            multi_component_ins.py:302-388 and the implicit-Euler mass term of
 *                            time_integration_schemes.py:663-685 / base_model.py:418-497
 *   ocmp_set_boundary     <- opencmp/models/base_model.py:321-341 (GridFunction.Set on Dirichlet
 *                            boundaries)
 *   ocmp_solver_create    <- opencmp/models/base_model.py:365-383 (ngsolve.Preconditioner(a, 'local'))
 *   ocmp_solve            <- opencmp/models/base_model.py:886-947 (linear_solve: solvers.CG with
 *                            initialize=False, solvers.GMRes with freedofs, direct solve on L - A*gfu)
 *   ocmp_spmv             <- the `a.mat * gfu.vec` products inside base_model.py:920-944
 *   ocmp_batch_*          <- a loop of the above over independent problem instances
 *   ocmp_guess_*          <- no counterpart: learned Krylov initial guess (its fallback is the
 *                            previous-step guess OpenCMP uses, base_model.py:925-937)
 */
#ifndef OPENCMP_GPU_H
#define OPENCMP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OCMP_ABI_VERSION 1

typedef enum {
    OCMP_OK = 0,
    OCMP_ERR_ARG = 1,          /* bad argument (null handle, unsupported size or order)          */
    OCMP_ERR_CUDA = 2,         /* a CUDA runtime call failed                                      */
    OCMP_ERR_NONFINITE = 3,    /* NaN / Inf met in the right-hand side or during the iteration    */
    OCMP_NOT_CONVERGED = 4,    /* iteration cap reached before the tolerance                      */
    OCMP_BREAKDOWN = 5,        /* Krylov breakdown (zero pivot / zero inner product)               */
    OCMP_TIMEOUT = 6,          /* a bounded device-side wait gave up                              */
    OCMP_ERR_UNSUPPORTED = 7,  /* combination not built (e.g. L2 on tetrahedra)                    */
    OCMP_ERR_NOMEM = 8         /* device allocation failed                                        */
} ocmp_status;

enum { OCMP_H1 = 0, OCMP_L2 = 1, OCMP_COMPOUND = 2 };  /* compound: the Taylor-Hood system (ocmp_th_*) */
enum { OCMP_WIND_NONE = 0, OCMP_WIND_CONST = 1, OCMP_WIND_VERTEX = 2 };
enum { OCMP_SRC_NONE = 0, OCMP_SRC_CONST = 1, OCMP_SRC_QP = 2 };
enum { OCMP_CG = 0, OCMP_GMRES = 1 };
enum { OCMP_PRE_NONE = 0, OCMP_PRE_JACOBI = 1, OCMP_PRE_BLOCK_JACOBI = 2, OCMP_PRE_USER = 3, OCMP_PRE_STRIP = 4,
       OCMP_PRE_CAHOUET_CHABARD = 5 };
enum { OCMP_FP64 = 0, OCMP_MIXED = 1 };

typedef struct ocmp_mesh_s* ocmp_mesh_t;
typedef struct ocmp_space_s* ocmp_space_t;
typedef struct ocmp_matrix_s* ocmp_matrix_t;
typedef struct ocmp_solver_s* ocmp_solver_t;
typedef struct ocmp_guess_s* ocmp_guess_t;

/* Bilinear form  a(u,v) = mass (u,v) + dt [ diff (grad u, grad v) - (u, w . grad v) ]
 *                        + dt * facet terms selected by the masks (bit l = boundary label l).
 * Terms follow multi_component_ins.py:158-300 (velocity_fixed) and poisson.py:71-131. */
typedef struct {
    double mass;             /* coefficient of the mass term (u, v); not scaled by dt            */
    double diff;             /* diffusion coefficient                                            */
    double dt;               /* time-step factor on every other term (1 for a stationary solve)  */
    int32_t wind_kind;       /* OCMP_WIND_*                                                       */
    double wind[3];          /* constant wind                                                     */
    const double* wind_vtx;  /* device, nv*dim: wind at the mesh vertices, linear in between      */
    double ipc;              /* interior penalty coefficient; alpha = ipc * order^2 / h            */
    int32_t dg;              /* add interior-facet (skeleton) SIPG + upwind terms (L2 spaces)      */
    uint32_t outflow_mask;   /* labels with  dt r c max(w.n, 0)      (total-flux / unlabelled)     */
    uint32_t wn_mask;        /* labels with  dt r c (w.n)            (Neumann half)                */
    uint32_t nitsche_mask;   /* DG Dirichlet labels (penalty, consistency, inflow upwind)          */
    int32_t skeleton_own_dt; /* nonzero: interior-facet terms take skeleton_dt instead of dt (OpenCMP
                                keeps them in the time-coefficient form, always implicit, while the
                                other operator terms are theta-weighted: time_integration_schemes.py) */
    double skeleton_dt;
    uint32_t robin_mask;     /* labels with a Robin term  dt robin[l] (u, v)_l: OpenCMP's
                                -dt dc r (u, v) on the marker, robin[l] = -dc r (poisson.py:93-97)   */
    double robin[32];        /* per label: the coefficient of the Robin facet mass term             */
} ocmp_form_t;

/* Linear form  L(v) = dt (f, v) + mass (u_prev, v) + dt * sum_l bval[l] <v>_l + DG Dirichlet data */
typedef struct {
    double dt;
    int32_t src_kind;        /* OCMP_SRC_*                                                        */
    double src_const;        /* f for OCMP_SRC_CONST                                              */
    const double* src_qp;    /* device, ne*nq: f at the quadrature points (ocmp_space_quad_points) */
    double mass;             /* coefficient of (u_prev, v)                                        */
    const double* uprev;     /* device, ndof, or NULL                                             */
    double bval[32];         /* per label, constant Neumann-type data                              */
    uint32_t bval_mask;
    double gval[32];         /* per label, constant DG Dirichlet datum                              */
    const double* bval_fq;   /* device, nbf*nfq or NULL: Neumann data at the boundary-facet quadrature
                                points (ocmp_space_facet_quad_points); used instead of bval[] on the
                                labels of bval_mask                                                  */
    const double* gval_fq;   /* device, nbf*nfq or NULL: DG Dirichlet data there, instead of gval[] */
    int32_t accumulate;      /* nonzero: b += L(v) instead of b = L(v)                            */
    int32_t dfloat;          /* nonzero: the mass term in double-float arithmetic on the FP32 pipes
                                (about 1e-14 relative to the FP64 product)                          */
} ocmp_rhs_t;

typedef struct {
    int64_t ndof, nnz, ne, nv;
    int32_t nloc, nq, dim, order, kind;
    int64_t n_interior_facets, n_boundary_facets, n_contrib;
    int32_t nfq;             /* quadrature points per facet                                        */
} ocmp_space_info_t;

typedef struct {
    int32_t method;          /* OCMP_CG / OCMP_GMRES                                               */
    int32_t restart;         /* GMRES restart length m (<= 128)                                    */
    int32_t precond;         /* OCMP_PRE_*                                                         */
    int32_t precision;       /* OCMP_FP64, or OCMP_MIXED: FP32 inner GMRES + FP64 refinement        */
    double tol;              /* on || (b - A x)_free ||_2 / || (b - A x_D)_free ||_2 (FP64)       */
    int32_t maxit;           /* total Krylov iterations                                             */
    double inner_tol;        /* mixed: relative reduction asked of each inner solve               */
    int32_t check_every;     /* host reads the convergence flag every k iterations (>= 1; 0: 8); -1:
                                GMRES checks first one iteration before the previous solve's count,
                                then after every iteration                                          */
} ocmp_solve_params_t;

typedef struct {
    int32_t status;          /* ocmp_status of the solve                                           */
    int32_t iterations;      /* Krylov iterations (inner iterations for OCMP_MIXED)                 */
    int32_t outer_iterations;/* refinement steps (OCMP_MIXED), restarts (GMRES)                    */
    double relres0;          /* FP64 relative residual of the initial guess                        */
    double relres;           /* FP64 relative residual at return, recomputed from b - A x           */
} ocmp_solve_info_t;

/* ---------------------------------------------------------------- general */
int ocmp_abi_version(void);
/* Kernels launched by this library so far (graph replays included); no counterpart in the reference */
uint64_t ocmp_launch_count(void);
int ocmp_last_error(char* buf, int len);
int ocmp_device_sync(void* stream);

/* ---------------------------------------------------------------- mesh and space */
int ocmp_mesh_create(const double* coords, int64_t nv, int32_t dim, const int32_t* elements, int64_t ne,
                     const int32_t* bfacets, const int32_t* blabels, int64_t nbf, ocmp_mesh_t* out);
int ocmp_mesh_destroy(ocmp_mesh_t mesh);

int ocmp_space_create(ocmp_mesh_t mesh, int32_t kind, int32_t order, uint32_t dirichlet_mask,
                      ocmp_space_t* out);
int ocmp_space_destroy(ocmp_space_t space);
int ocmp_space_info(ocmp_space_t space, ocmp_space_info_t* info);
int ocmp_space_get_dofs(ocmp_space_t space, int32_t* elem_dofs_host);            /* ne*nloc  */
int ocmp_space_get_pattern(ocmp_space_t space, int64_t* rowptr_host, int32_t* col_host);
int ocmp_space_get_free(ocmp_space_t space, uint8_t* free_host);                 /* ndof     */
int ocmp_space_quad_points(ocmp_space_t space, double* xyz_host);                /* ne*nq*dim */
int ocmp_set_boundary(ocmp_space_t space, uint32_t mask, const double* gval_host32, double* u_dev,
                      void* stream);
/* Boundary-facet quadrature points, nbf*nfq*dim (nbf = n_boundary_facets, nfq = info.nfq), in the
 * space's boundary-facet order; the points at which bval_fq / gval_fq are sampled. */
int ocmp_space_facet_quad_points(ocmp_space_t space, double* xyz_host);
/* The space's boundary facets: (element, local facet, label) per facet, nbf*3 */
int ocmp_space_boundary_facets(ocmp_space_t space, int32_t* elem_facet_label_host);
/* Space-dependent Dirichlet data (GridFunction.Set(g, definedon=...), base_model.py:321-341), as a
 * projection-based interpolation: vertex dofs take g at the vertex; the bubble dofs of each edge
 * (and, for 3D order 3, each face) of a facet whose label is in `mask` take the L2 projection, along
 * that edge (face), of g minus the part already fixed. ocmp_boundary_points lists the points at
 * which the caller samples g (count first with xyz_host = NULL); ocmp_set_boundary_values takes
 * the samples in that order and writes the constrained dofs of u_dev. */
int ocmp_boundary_points(ocmp_space_t space, uint32_t mask, int64_t* npts, double* xyz_host);
int ocmp_set_boundary_values(ocmp_space_t space, uint32_t mask, const double* g_host, double* u_dev, void* stream);
/* || u_h - f ||_{L2} by the space's element rule, f at the quadrature points (fq_dev, ne*nq) or the
 * constant fconst when fq_dev is NULL  <- opencmp/helpers/error.py:75-128 (norm('l2_norm', ...)) */
int ocmp_l2_error(ocmp_space_t space, const double* u_dev, const double* fq_dev, double fconst, double* result_host,
                  void* stream);

/* ---------------------------------------------------------------- assembly */
/* Matrix outputs written by each assembly (flags, OR-able). The FP64 values are always written.
 * The Jacobi-scaled values A D^-1 (D = diag A on free rows) are the Krylov matrices the GMRES path
 * uses with the point-Jacobi preconditioner; assembling them in the same pass saves a sweep.
 * OCMP_MAT_DFLOAT assembles the element matrices and their sums in double-float arithmetic (pairs of
 * FP32 values, about 48 significant bits) on the FP32 pipes, finishing each CSR entry with one FP64
 * addition; the FP64 values agree with the native FP64 assembly to about 1e-14 relative. */
enum {
    OCMP_MAT_FP32 = 1,
    OCMP_MAT_JACOBI64 = 2,
    OCMP_MAT_JACOBI32 = 4,
    OCMP_MAT_DFLOAT = 8,
    OCMP_MAT_SELL32 = 16
};
/* OCMP_MAT_SELL32 (with OCMP_MAT_JACOBI32, single matrices): the FP32 Jacobi-scaled values are
 * written in the space's SELL-32 order instead of CSR order (slices of 32 rows, each row padded to
 * its slice's width in 4-entry chunks, chunk-major within a slice, zero padding), the layout the
 * FP32 GMRES SpMV reads with 16-byte loads, a warp per slice; ocmp_matrix_scaled_values then
 * returns them in that order. */
int ocmp_matrix_create(ocmp_space_t space, int32_t flags, ocmp_matrix_t* out);
/* nbatch independent matrices on the space's pattern (instances of a batch of problems that differ
 * only in their coefficients); values are stored instance after instance. */
int ocmp_matrix_create_batch(ocmp_space_t space, int32_t nbatch, int32_t flags, ocmp_matrix_t* out);
int ocmp_matrix_destroy(ocmp_matrix_t mat);
int ocmp_matrix_values(ocmp_matrix_t mat, double** vals64_dev, float** vals32_dev);
/* Device pointers of the Jacobi-scaled values A D^-1 (FP64, FP32) and of D^-1 (NULL if not built). */
int ocmp_matrix_scaled_values(ocmp_matrix_t mat, double** svals64_dev, float** svals32_dev, double** dinv_dev);
int ocmp_assemble_matrix(ocmp_matrix_t mat, const ocmp_form_t* form, void* stream);
int ocmp_assemble_rhs(ocmp_space_t space, const ocmp_form_t* form, const ocmp_rhs_t* rhs, double* b_dev,
                      void* stream);
/* forms: host array of the matrix's nbatch forms (one per instance) */
int ocmp_assemble_matrix_batch(ocmp_matrix_t mat, const ocmp_form_t* forms, void* stream);
int ocmp_spmv(ocmp_matrix_t mat, const double* x_dev, double* y_dev, void* stream);
/* y = alpha * A x + beta * y (beta == 0: y is not read) - the explicit operator terms of the
 * explicit-Euler and Crank-Nicolson right-hand sides (time_integration_schemes.py:25-76, 134-191) */
int ocmp_spmv_axpby(ocmp_matrix_t mat, double alpha, const double* x_dev, double beta, double* y_dev, void* stream);
/* Autotuner: times the CSR SpMV of `mat` (x, y: ndof scratch vectors) for each built pair of threads
 * per row and loads in flight per thread, keeps the fastest for every kernel of the space that runs
 * rows (SpMV, residuals, GMRES), and reports it. */
int ocmp_matrix_autotune(ocmp_matrix_t mat, const double* x_dev, double* y_dev, void* stream, int32_t* tpr,
                         int32_t* unroll, float* ms);

/* ---------------------------------------------------------------- Krylov solve */
int ocmp_solver_create(ocmp_matrix_t mat, const ocmp_solve_params_t* params, ocmp_solver_t* out);
int ocmp_solver_destroy(ocmp_solver_t solver);
/* Refresh preconditioner data after the matrix values changed (Preconditioner.Update). */
int ocmp_solver_update(ocmp_solver_t solver, void* stream);
/* Solve A_ff x_f = (b - A x_D)_f in place; x_dev holds the Dirichlet values and the initial guess. */
int ocmp_solve(ocmp_solver_t solver, const double* b_dev, double* x_dev, void* stream, ocmp_solve_info_t* info);
/* GMRES on all nbatch systems of a batched matrix at once (b, x: nbatch vectors of ndof, instance
 * after instance; infos: nbatch entries). Each system has its own Krylov space, Hessenberg matrix,
 * tolerance test and restart count; the kernels cover every instance in one launch (instance =
 * blockIdx.y) and instances that have converged return immediately. */
int ocmp_solve_batch(ocmp_solver_t solver, const double* b_dev, double* x_dev, void* stream,
                     ocmp_solve_info_t* infos);
/* Solver groups: uneven instances in one kernel sequence. The instances of several GMRES solvers
 * (each a single or batched matrix of its own space: different sizes, orders and patterns) are
 * solved together: every kernel of the GMRES iteration is launched once over all of them, a fixed
 * grid striding over a device list of (instance, block) pairs of the instances still iterating
 * (each instance's share proportional to its rows, the rows per thread of its SpMV from its
 * space's autotuned choice; the list shrinks after every restart cycle), one restart cycle
 * replayed from a CUDA graph. Each instance keeps its own Krylov space, tolerance and
 * convergence test; converged instances return at the top of every kernel. No kernel waits on
 * another block: reductions end in the last block to finish. Members must be GMRES with point
 * Jacobi (or no) preconditioning, CSR Krylov matrices, and share restart, precision and maxit.
 * ocmp_group_solve takes one right-hand side and solution array per member (its instances one
 * after another) and fills infos for every instance in member order. The group borrows the
 * members' buffers: do not solve a member on its own while its group is in use. Replaces the
 * per-instance loop over opencmp/solvers solve calls (one Solver.solve per run directory) with one
 * call; no counterpart in the reference beyond that loop. */
typedef struct ocmp_group_s* ocmp_group_t;
int ocmp_group_create(const ocmp_solver_t* solvers, int32_t count, ocmp_group_t* out);
int ocmp_group_solve(ocmp_group_t group, const double* const* b_dev, double* const* x_dev, void* stream,
                     ocmp_solve_info_t* infos);
int ocmp_group_destroy(ocmp_group_t group);
/* Replay each GMRES restart cycle (m iterations, the x update and the next FP64 residual) from a
 * CUDA graph captured on first use (re-captured when b, x or the stream change). */
int ocmp_solver_set_graph(ocmp_solver_t solver, int32_t on);
/* OCMP_PRE_USER: the inverse diagonal (ndof, device) applied as the preconditioner; copied, and
 * taken over by the next ocmp_solver_update. */
int ocmp_solver_set_diag(ocmp_solver_t solver, const double* dinv_dev, void* stream);
/* Time every GMRES SpMV launch with CUDA events on its stream (single solves, outside graphs; up to
 * 4096 launches per solve); ocmp_solver_spmv_stats returns the launches that did the product (not
 * those queued past convergence, which return at once) and their total milliseconds since the
 * timing was switched on. No counterpart in the reference (measurement). */
int ocmp_solver_spmv_timing(ocmp_solver_t solver, int32_t on);
int ocmp_solver_spmv_stats(ocmp_solver_t solver, int64_t* launches, double* total_ms);

/* ---------------------------------------------------------------- strip direct preconditioner
 * OCMP_PRE_STRIP replaces the sparse direct solve of opencmp/models/base_model.py:906-922
 * (a.mat.Inverse(freedofs, 'pardiso' | 'umfpack'), then gfu += inv (L - A gfu)) by an exact block
 * factorisation used as the preconditioner of GMRES, whose FP64 residual decides convergence. The
 * dofs are cut into consecutive strips over which the matrix is block tridiagonal (greedy over the
 * row bandwidth: number the dofs so that the matrix is banded, e.g. the element-major L2 dofs of a
 * structured mesh whose elements run row by row); each strip's Schur complement is inverted
 * explicitly in FP32 by block Gauss-Jordan with 128 x 128 pivot tiles, and a preconditioner
 * application is one forward and one backward sweep of dense matrix-vector products. Built by
 * ocmp_solver_create (OCMP_ERR_UNSUPPORTED when the pattern has no such strips or a strip exceeds
 * 16384 dofs) and factorised by every ocmp_solver_update (not by ocmp_solver_create: OpenCMP
 * builds its preconditioners before the first assembly); ocmp_solve refuses a strip solver that
 * has not been factorised since its last failure. GMRES only.
 * ocmp_solver_strip_stats reports the last factorisation. No counterpart in the reference beyond
 * the direct solve it replaces. */
typedef struct {
    int64_t nstrips;         /* strips                                                             */
    int64_t max_strip;       /* largest strip, padded to a multiple of 128                          */
    int64_t bytes;           /* device memory of the factorisation                                  */
    double factor_ms;        /* wall time of the last factorisation on its stream (CUDA events)     */
    double gemm_ms;          /* time inside the dense products (0 unless ocmp_solver_strip_timing)  */
    double gemm_flops;       /* flops of those products                                             */
    int32_t singular_tiles;  /* pivot tiles that met a zero or non-finite pivot                     */
    int32_t gemm_kind;       /* 0: FP32 SIMT products, 1: tensor-core (tcgen05, 3xTF32) products    */
    double tile_ms;          /* time in the pivot-tile inversions (with ocmp_solver_strip_timing)   */
    double panel_ms;         /* time in the panel kernels (with ocmp_solver_strip_timing)           */
    int32_t fast_strips;     /* strips whose non-interface block splits into groups of <= 32 dofs   */
    int32_t schulz_strips;   /* of those, interface inverses by Newton-Schulz from the previous one */
    int32_t schulz_iterations; /* Newton-Schulz steps in total                                      */
    int32_t schulz_fallbacks;  /* Newton-Schulz attempts that fell back to Gauss-Jordan             */
    double gemm_bytes;       /* algorithmic bytes of the dense products (operands once, C out/in)   */
} ocmp_strip_stats_t;
int ocmp_solver_strip_stats(ocmp_solver_t solver, ocmp_strip_stats_t* out);
/* time every dense product of the next factorisations with CUDA events (measurement) */
int ocmp_solver_strip_timing(ocmp_solver_t solver, int32_t on);
/* dense products of the next factorisations: 0 FP32 SIMT (the default), 1 tensor cores */
int ocmp_solver_strip_gemm(ocmp_solver_t solver, int32_t kind);
/* on (the default): a strip whose non-interface dofs N fall into independent groups of at most 32
 * (a row of DG elements: the elements that do not touch the previous row) inverts those groups one
 * warp each, forms the interface Schur complement with one dense product and inverts it by
 * Newton-Schulz iteration started from the previous strip's inverse (Gauss-Jordan when that start
 * does not converge); off: block Gauss-Jordan over every strip's 128 x 128 tiles */
int ocmp_solver_strip_schulz(ocmp_solver_t solver, int32_t on);
/* C = beta C + alpha A B^T in FP32, row-major, K contiguous in A (M x K) and B (N x K): the dense
 * product of the strip factorisation, exposed for tests and measurement. kind 0: FP32 SIMT (K a
 * multiple of 16); kind 1: tcgen05 tensor cores, TF32 products with the 3xTF32 split for FP32
 * accuracy, operands staged by TMA (K a multiple of 32, operands 16-byte aligned). M and N are
 * multiples of 128. Synchronises the stream for kind 1 (it reads the kernel's wait flag). No
 * counterpart in the reference. */
int ocmp_dense_gemm_nt(int32_t kind, int32_t M, int32_t N, int32_t K, const float* A, int64_t lda, const float* B,
                       int64_t ldb, float* C, int64_t ldc, float alpha, float beta, void* stream);

/* ---------------------------------------------------------------- incompressible Navier-Stokes
 * Taylor-Hood system of OpenCMP's INS model (opencmp/models/ins.py) on triangles: velocity H1
 * order k (2 or 3) per component, pressure H1 order k-1, compound vector [u_x | u_y | p].
 *   ocmp_th_create       <- ins.py:90-128 (_construct_fes: VectorH1 x H1, velocity Dirichlet labels)
 *   ocmp_th_assemble     <- BilinearForm.Assemble of ins.py:178-251 plus the time-derivative mass
 *                           term (base_model.py:418-497); the interior-facet DG terms are not built
 *   ocmp_th_assemble_rhs <- LinearForm.Assemble of ins.py:253-314 (source, u_prev mass term, IMEX
 *                           explicit convection of construct_imex_explicit)
 *   ocmp_th_errors       <- opencmp/helpers/error.py:75-128 (l2_norm of u) and 151-167 (divergence)
 * Matrices on the compound space come from ocmp_matrix_create(compound, 0, ...); they are solved by
 * GMRES with OCMP_PRE_USER and the inverse diagonal of ocmp_th_block_diag. */
typedef struct ocmp_th_s* ocmp_th_t;
typedef struct {
    double mass;           /* coefficient of (u, v)                                              */
    double nu;             /* kinematic viscosity                                                */
    double dt;             /* factor of the viscous, convection and pressure terms               */
    double eps_p;          /* pressure regularisation  -dt eps_p (p, q)  (OpenCMP: 1e-10)        */
    const double* wind;    /* device: Oseen wind as a compound vector (velocity part read), or NULL */
    double tcoef;          /* factor of the time-coefficient terms (div u q, div v p, eps_p p q) in
                              place of dt: OpenCMP's CNLF doubles them (time_integration_schemes.py) */
} ocmp_th_form_t;
typedef struct {
    double dt;
    double src[2];         /* constant body force                                                */
    const double* src_qp;  /* device, ne*nq*2: body force at ocmp_th_quad_points, or NULL        */
    double mass;           /* coefficient of (u_prev, v)                                         */
    const double* uprev;   /* device compound vector, or NULL                                    */
    const double* imex;    /* device compound vector w: adds -imex_coef dt ((grad w) w, v), or NULL */
    double imex_coef;      /* factor of the explicit convection term                              */
    int32_t accumulate;    /* nonzero: b += L(v) instead of b = L(v)                            */
} ocmp_th_rhs_t;
int ocmp_th_create(ocmp_mesh_t mesh, int32_t order_u, uint32_t dirichlet_mask_u, ocmp_th_t* out);
int ocmp_th_destroy(ocmp_th_t th);
/* the velocity component space (order k), the pressure space (k-1) and the compound space; owned
 * by the system (do not destroy them) */
int ocmp_th_spaces(ocmp_th_t th, ocmp_space_t* velocity, ocmp_space_t* pressure, ocmp_space_t* compound);
int ocmp_th_nq(ocmp_th_t th);
int ocmp_th_quad_points(ocmp_th_t th, double* xyz_host);                       /* ne*nq*2 */
int ocmp_th_assemble(ocmp_th_t th, ocmp_matrix_t mat, const ocmp_th_form_t* form, void* stream);
int ocmp_th_assemble_rhs(ocmp_th_t th, const ocmp_th_rhs_t* rhs, double* b_dev, void* stream);
/* GMRES with OCMP_PRE_CAHOUET_CHABARD on a compound Taylor-Hood matrix [u | p]: the solve of the
 * saddle-point system OpenCMP hands to a sparse direct solver (ins.py with linear_solver = default).
 * The preconditioner is velocity point Jacobi (vdinv: nu entries, 0 on constrained rows) and on the
 * pressure block the Cahouet-Chabard approximation of the inverse Schur complement,
 *   z_p = -(alpha S^-1 r_p + beta mpinv r_p) / tc^2,   S = L_p + delta M_p  (the matrix pop),
 * alpha the mass coefficient, beta = dt nu, tc the factor of the divergence terms, mpinv the inverse
 * pressure-mass diagonal. S^-1 is applied exactly by the strip direct factorisation of pop, built on
 * the first call and refactorised when `refactor` is nonzero (pop's values changed); the other
 * arguments are copied on every call. No counterpart in the reference beyond the solve it
 * replaces. */
int ocmp_solver_set_cahouet_chabard(ocmp_solver_t solver, ocmp_matrix_t pop, const double* vdinv_dev,
                                    const double* mpinv_dev, int64_t nu, double alpha, double beta, double tc,
                                    int32_t refactor, void* stream);
/* Inverse of the block-diagonal preconditioner: 1/a_ii on free velocity rows; on pressure rows
 * -1/(|a_ii| + sum_j a_ij^2 / |a_jj|) over free velocity columns j (the diagonal of the Schur
 * complement B diag(A)^-1 B^T); 0 on constrained rows. */
int ocmp_th_block_diag(ocmp_th_t th, ocmp_matrix_t mat, double* dinv_dev, void* stream);
/* || u_h - ref ||_L2 over both velocity components (ref_qp: ne*nq*2, or NULL for 0) and || div u_h ||_L2 */
int ocmp_th_errors(ocmp_th_t th, const double* u_dev, const double* ref_qp_dev, double* l2, double* div,
                   void* stream);

/* ---------------------------------------------------------------- learned initial guess
 * No counterpart in the reference (OpenCMP starts each Krylov solve from the previous step's
 * solution, base_model.py:925-937). From the last k solutions u^n, u^{n-1}, ... (k <= 6) each dof
 * has the backward differences D_j = nabla^j u^n, j = 1..k-1. The guess
 *     x = u^n + D_1 + ... + D_p + S_{k-1} y(X),   X = [D_1 / S_1, ..., D_{k-1} / S_{k-1}]
 * is the degree-p extrapolation in time plus the correction of a per-dof MLP
 *     y = w3 . tanh(W2 tanh(W1 x + b1) + b2) + b3 + c . x   (hidden width 16, FP32, F = k-1 inputs),
 * S_j being the root mean square of D_j over the free dofs. A new network has zero output. Training
 * (ocmp_guess_residual_loss, ocmp_guess_backward, ocmp_guess_adam_step) minimises the FP64
 * relative residual |A e| / |b| the guess leaves; the solve's own FP64 residual test is unchanged,
 * so the guess never decides the accuracy of the result. */
int ocmp_guess_create(int32_t n_features, uint64_t seed, ocmp_guess_t* out);
int ocmp_guess_destroy(ocmp_guess_t g);
int ocmp_guess_nparams(ocmp_guess_t g);
int ocmp_guess_params(ocmp_guess_t g, float* host, int32_t set);       /* copy out (set=0) or in (set=1) */
int ocmp_guess_forward(ocmp_guess_t g, const float* X_dev, int64_t rows, float* Y_dev, void* stream);
/* mean squared error over `rows` samples and its parameter gradient (deterministic) */
int ocmp_guess_loss_grad(ocmp_guess_t g, const float* X_dev, const float* T_dev, int64_t rows, double* loss_host,
                         float* grad_host, void* stream);
/* parameter gradient of sum_r dY_r y_r (back-propagation of an upstream gradient), deterministic;
 * kept on the device for ocmp_guess_adam_step, copied to grad_host when it is not NULL */
int ocmp_guess_backward(ocmp_guess_t g, const float* X_dev, const float* dY_dev, int64_t rows, float* grad_host,
                        void* stream);
int ocmp_guess_adam_step(ocmp_guess_t g, float lr, void* stream);
/* The history is a backward-difference table in double-float held by the caller: tab_dev = k rows
 * of n (hi, lo) float pairs (2 k n floats), row j = nabla^j u^n, row 0 = u^n. ocmp_guess_push adds
 * the newest solution u_dev, m being the number of rows already valid (0 after a reset; after the
 * push min(m + 1, k) rows are valid). All table arithmetic runs on the FP32 pipes. */
int ocmp_guess_push(int64_t n, int32_t k, int32_t m, float* tab_dev, const double* u_dev, void* stream);
/* S_1..S_{k-1} into scales_dev (a 32-double buffer; on the device, no host synchronisation) and,
 * when X_dev is not NULL, the features X (ndof rows of k-1 floats, zero rows at constrained dofs;
 * the network must take F = k-1). free_dev may be NULL (all dofs free). k = 2..6 valid rows. */
int ocmp_guess_features(ocmp_guess_t g, int64_t n, int32_t k, const float* tab_dev, const uint8_t* free_dev,
                        double* scales_dev, float* X_dev, void* stream);
/* x = u^n + D_1 + ... + D_p (+ S_{k-1} y(X) when g is not NULL) on free dofs, u^n on constrained
 * dofs; p = base_order < k valid rows. With g = NULL it is the plain extrapolation (k = 1 or
 * p = 0: the previous-step guess) and scales_dev may be NULL. */
int ocmp_guess_predict(ocmp_guess_t g, int64_t n, int32_t k, const float* tab_dev, const uint8_t* free_dev,
                       const double* scales_dev, int32_t base_order, double* x_dev, void* stream);
/* training target T_i = (u^{n+1}_i - u^n_i - D_1 - ... - D_p) / S_{k-1} (0 at constrained dofs) */
int ocmp_guess_target(int64_t n, int32_t k, const float* tab_dev, const uint8_t* free_dev, const double* scales_dev,
                      int32_t base_order, const double* unext_dev, float* T_dev, void* stream);
/* Residual loss of a prediction Y (ndof rows) against the target T of one stored step: with
 * e = S (Y - T) on free dofs (S = *scale_dev = S_{k-1} of that step), loss = weight |(A e)_free|^2 /
 * |b_free|^2, `weight` times the squared relative residual the guess would start the solve with;
 * dY = d loss / dY = 2 weight S A^T (A e)_free / |b_free|^2. Needs a structurally symmetric pattern
 * (A^T gathers through a transpose-position map the space builds on first use). */
int ocmp_guess_residual_loss(ocmp_guess_t g, ocmp_matrix_t mat, const float* Y_dev, const float* T_dev,
                             const double* scale_dev, const double* b_dev, double weight, double* loss_host,
                             float* dY_dev, void* stream);
/* y = A^T x with the FP64 values (structurally symmetric patterns) */
int ocmp_spmv_transpose(ocmp_matrix_t mat, const double* x_dev, double* y_dev, void* stream);

/* ---------------------------------------------------------------- allocation-free solve
 * No counterpart in the reference: an addition for callers that cannot call cudaMalloc when they
 * solve - a host whose device memory belongs to another allocator's fixed pool (a fresh cudaMalloc
 * would take memory that pool has already claimed, or fail), or a loop that cannot take the
 * implicit device-wide synchronisation of cudaFree. Same FP64 Jacobi-preconditioned CG as
 * ocmp_solve with OCMP_CG, on the free dofs of `mat`, to the same relative-residual definition; it
 * allocates nothing (no cudaMalloc, cudaFree or allocating library call). Its workspace is a static
 * device array of 41 MiB that every GPU which loads this library holds until the process exits;
 * systems with more than OCMP_NOALLOC_MAX_NDOF dofs are rejected with OCMP_ERR_ARG, batched
 * matrices (B > 1) with OCMP_ERR_UNSUPPORTED. The first call on each device looks up that array's
 * device address (cudaGetSymbolAddress) with the device current. All calls share the one workspace
 * and it keeps the last call's contents (each call resets what must start at zero): calls whose
 * work overlaps on the GPU (different streams or threads) race, so serialise them. The host reads
 * the convergence flags every 8 iterations through a blocking copy into its own stack memory (no
 * pinned buffer is allocated for it), and the call returns OCMP_ERR_UNSUPPORTED on a stream that is
 * being captured, since those reads would invalidate the capture. */
#define OCMP_NOALLOC_MAX_NDOF 1048576
int ocmp_solve_cg_noalloc(ocmp_matrix_t mat, const double* b_dev, double* x_dev, double tol, int32_t maxit,
                          void* stream, ocmp_solve_info_t* info);

#ifdef __cplusplus
}
#endif
#endif
