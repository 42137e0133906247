"""GPU parity tests: libopencmp_gpu.so (through its C ABI) against the CPU oracle on the same inputs.

Tolerances: matrix and right-hand-side entries 1e-12 relative to the largest entry (FP64
assembly); solutions 1e-8 relative in the l2 norm of the coefficient vector with both solves
driven to a 1e-12 (FP64) / 1e-11 (mixed) relative residual; integer data (dof maps, CSR
pattern, free-dof masks) bit-exact.
"""
import math

import numpy as np
import pytest

from opencmp_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _spaces(oracle, mesh, kind, order, dirichlet=()):
    from opencmp_gb300 import fem
    g = fem.Space(mesh, 'H1' if kind == 0 else 'L2', order, dirichlet)
    o = oracle.Space(mesh, kind, order, mesh.label_mask(dirichlet) if kind == 0 else 0)
    return g, o


def _t(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device='cuda')


CASES = [
    ('tri-p1', lambda: M.unit_square(7), 0, 1),
    ('tri-p2', lambda: M.unit_square(9), 0, 2),
    ('tri-p3', lambda: M.unit_square(6), 0, 3),
    ('tet-p1', lambda: M.unit_cube(3), 0, 1),
    ('tet-p2', lambda: M.unit_cube(3), 0, 2),
    ('tet-p3', lambda: M.unit_cube(2), 0, 3),
    ('dg-p1', lambda: M.unit_square(6), 1, 1),
    ('dg-p2', lambda: M.unit_square(8), 1, 2),
    ('dg-p3', lambda: M.unit_square(5), 1, 3),
]


@pytest.mark.parametrize('name,mk,kind,order', CASES, ids=[c[0] for c in CASES])
def test_dofs_pattern_free_bit_exact(gpu_lib, oracle, name, mk, kind, order):
    m = mk()
    names = m.bc_names[:2]
    g, o = _spaces(oracle, m, kind, order, names)
    assert (g.ndof, g.nnz) == (o.ndof, o.nnz)
    assert np.array_equal(g.dofs(), o.dofs())
    rg, cg = g.pattern()
    ro, co = o.pattern()
    assert np.array_equal(rg, ro) and np.array_equal(cg, co)
    assert np.array_equal(g.FreeDofs(), o.freedofs())


def _forms(oracle, m, kind, with_vertex_wind):
    from opencmp_gb300 import fem
    D = m.dim
    wv = np.stack([-(m.coords[:, 1] - 0.5), m.coords[:, 0] - 0.5] + ([0.3 + 0 * m.coords[:, 0]] if D == 3 else []), 1)
    wind = (1.0, 0.5, 0.25)[:D]
    lab = lambda names: m.label_mask(names)  # noqa: E731
    out = [
        ('mass+diffusion', dict(mass=1.0, diff=0.7, dt=0.3)),
        ('convection-const', dict(mass=0.5, diff=1e-2, dt=1e-2, wind=wind,
                                  outflow_mask=lab(m.bc_names[1:2]), wn_mask=lab(m.bc_names[2:3]))),
    ]
    if with_vertex_wind:
        out.append(('convection-vertex', dict(mass=0.0, diff=1e-3, dt=1.0, wind_vtx=wv, outflow_mask=lab(m.bc_names))))
    if kind == 1:
        out.append(('dg-sipg-upwind', dict(mass=1.0, diff=1e-2, dt=0.5, wind_vtx=wv, dg=True, ipc=10.0,
                                           nitsche_mask=lab(m.bc_names))))
    res = []
    for nm, kw in out:
        okw = dict(kw)
        gkw = dict(kw)
        if 'wind_vtx' in kw:
            gkw['wind_vtx'] = _t(kw['wind_vtx'])
        res.append((nm, oracle.make_form(**okw), fem.make_form(**gkw), gkw))
    return res


@pytest.mark.parametrize('dfloat', [False, True], ids=['fp64', 'dfloat'])
@pytest.mark.parametrize('name,mk,kind,order', CASES, ids=[c[0] for c in CASES])
def test_matrix_entries_match_oracle(gpu_lib, oracle, name, mk, kind, order, dfloat):
    from opencmp_gb300 import fem
    m = mk()
    g, o = _spaces(oracle, m, kind, order, m.bc_names[:1])
    A = fem.Matrix(g, fp32=True, jacobi64=True, jacobi32=True, dfloat=dfloat)
    rp, col = o.pattern()
    rows = np.repeat(np.arange(o.ndof), np.diff(rp))
    free = o.freedofs()
    for nm, of, gf, keep in _forms(oracle, m, kind, True):
        A.assemble(gf)
        ag = A.values()
        ao = o.assemble(of)
        scale = np.abs(ao).max()
        err = np.abs(ag - ao).max() / scale
        assert err <= 1e-12, (nm, err)
        a32 = A.values32()
        assert np.abs(a32 - ag).max() <= 1e-7 * scale, nm
        # Jacobi-scaled outputs: A D^-1 with D the diagonal on free rows (0 on constrained ones)
        s64, s32, dinv = A.scaled_values()
        diag = ao[rp[:-1] + np.array([np.searchsorted(col[rp[r]:rp[r + 1]], r) for r in range(o.ndof)])]
        dref = np.where(free & (diag != 0), 1.0 / np.where(diag != 0, diag, 1.0), 0.0)
        assert np.abs(dinv - dref).max() <= 1e-12 * np.abs(dref).max(), nm
        sref = ao * dref[col]
        assert np.abs(s64 - sref).max() <= 1e-12 * np.abs(sref).max(), nm
        assert np.abs(s32 - sref).max() <= 1e-6 * np.abs(sref).max(), nm


def test_assembly_is_bit_reproducible(gpu_lib, oracle):
    from opencmp_gb300 import fem
    m = M.unit_cube(4)
    g = fem.Space(m, 'H1', 2, m.bc_names)
    A = fem.Matrix(g)
    f = fem.make_form(mass=1.0, diff=1e-2, dt=1e-3, wind=(1.0, 0.5, 0.25))
    A.assemble(f)
    v1 = A.values()
    A.assemble(f)
    v2 = A.values()
    assert v1.tobytes() == v2.tobytes()


def _src_sinprod(X, D):
    v = 2 * math.pi ** 2 * np.ones(X.shape[:-1])
    for k in range(D):
        v = v * np.sin(math.pi * X[..., k])
    return v


@pytest.mark.parametrize('dfloat', [False, True])
@pytest.mark.parametrize('name,mk,kind,order', CASES, ids=[c[0] for c in CASES])
def test_rhs_matches_oracle(gpu_lib, oracle, name, mk, kind, order, dfloat):
    import torch
    from opencmp_gb300 import fem
    m = mk()
    D = m.dim
    g, o = _spaces(oracle, m, kind, order, m.bc_names[:1])
    rng = np.random.default_rng(1)
    up = rng.standard_normal(g.ndof)
    lab0 = 1
    nit = m.label_mask(m.bc_names[:2]) if kind == 1 else 0
    of = oracle.make_form(diff=0.3, dt=0.2, wind=(1.0, -0.5, 0.2)[:D], nitsche_mask=nit, dg=kind == 1)
    gf = fem.make_form(diff=0.3, dt=0.2, wind=(1.0, -0.5, 0.2)[:D], nitsche_mask=nit, dg=kind == 1)
    fq = _t(_src_sinprod(g.quad_points(), D))
    if dfloat:
        # a double-float assembly first, so the RHS also runs on the space's static geometry
        fem.Matrix(g, dfloat=True).assemble(gf)
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    gv = {0: 0.7, 1: -0.4}
    fem.assemble_rhs(g, gf, fem.make_rhs(dt=0.2, src_qp=fq, mass=0.9, uprev=_t(up), bval={lab0: 2.5}, gval=gv,
                                         dfloat=dfloat), b)
    bo = o.rhs(of, oracle.make_rhs(dt=0.2, src_kind=oracle.SRC_SINPROD, src=(2 * math.pi ** 2,), mass=0.9, uprev=up,
                                   bval={lab0: 2.5}, gval=gv))
    bg = b.cpu().numpy()
    err = np.abs(bg - bo).max() / np.abs(bo).max()
    assert err <= 1e-12, err


def _solve_pair(oracle, m, kind, order, dirichlet, fkw, method, precond, precision, tol):
    import torch
    from opencmp_gb300 import fem
    g, o = _spaces(oracle, m, kind, order, dirichlet)
    gkw = dict(fkw)
    if 'wind_vtx' in fkw:
        gkw['wind_vtx'] = _t(fkw['wind_vtx'])
    A = fem.Matrix(g, fp32=precision == 'mixed', jacobi64=precision == 'fp64', jacobi32=precision == 'mixed',
                   dfloat=precision == 'mixed')
    A.assemble(fem.make_form(**gkw))
    fq = _t(_src_sinprod(g.quad_points(), m.dim))
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    fem.assemble_rhs(g, fem.make_form(**gkw), fem.make_rhs(src_qp=fq), b)
    x = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    sv = fem.KrylovSolver(A, method=method, restart=40, precond=precond, precision=precision, tol=tol, maxit=5000,
                          inner_tol=1e-5)
    info = sv.solve(b, x)
    ao = o.assemble(oracle.make_form(**fkw))
    bo = o.rhs(oracle.make_form(**fkw), oracle.make_rhs(src_kind=oracle.SRC_SINPROD, src=(2 * math.pi ** 2,)))
    xo = np.zeros(o.ndof)
    if method == 'CG':
        o.cg(ao, bo, xo, tol=1e-13, maxit=20000)
    else:
        o.gmres(ao, bo, xo, restart=60, precond=2 if precond == 'block_jacobi' else 1, tol=1e-13, maxit=20000)
    xg = x.cpu().numpy()
    return info, xg, xo, o, ao, bo


SOLVES = [
    ('poisson-cg-fp64', lambda: M.unit_square(24), 0, 2, 'all', dict(diff=1.0), 'CG', 'jacobi', 'fp64'),
    ('poisson-cg-mixed', lambda: M.unit_square(24), 0, 2, 'all', dict(diff=1.0), 'CG', 'jacobi', 'mixed'),
    ('cd-gmres-fp64', lambda: M.unit_square(20), 0, 3, 'all', dict(diff=1e-2, wind=(1.0, 0.4)), 'GMRES', 'jacobi', 'fp64'),
    ('cd-gmres-mixed', lambda: M.unit_square(20), 0, 2, 'all', dict(diff=1e-2, wind=(1.0, 0.4)), 'GMRES', 'jacobi', 'mixed'),
    ('tet-transient-fp64', lambda: M.unit_cube(5), 0, 2, 'all', dict(mass=1.0, diff=1e-2, dt=1e-3, wind=(1.0, 0.5, 0.25)),
     'GMRES', 'jacobi', 'fp64'),
    ('tet-transient-mixed', lambda: M.unit_cube(5), 0, 2, 'all', dict(mass=1.0, diff=1e-2, dt=1e-3, wind=(1.0, 0.5, 0.25)),
     'GMRES', 'jacobi', 'mixed'),
    ('dg-blockjacobi-fp64', lambda: M.unit_square(12), 1, 2, (), dict(diff=1e-2, dg=True, ipc=10.0, nitsche_mask=15,
                                                                      wind=(1.0, 0.3)), 'GMRES', 'block_jacobi', 'fp64'),
    ('dg-blockjacobi-mixed', lambda: M.unit_square(12), 1, 2, (), dict(diff=1e-2, dg=True, ipc=10.0, nitsche_mask=15,
                                                                       wind=(1.0, 0.3)), 'GMRES', 'block_jacobi', 'mixed'),
]


@pytest.mark.parametrize('name,mk,kind,order,dirichlet,fkw,method,precond,precision', SOLVES,
                         ids=[s[0] for s in SOLVES])
def test_solution_matches_oracle(gpu_lib, oracle, name, mk, kind, order, dirichlet, fkw, method, precond, precision):
    m = mk()
    d = m.bc_names if dirichlet == 'all' else dirichlet
    tol = 1e-12 if precision == 'fp64' else 1e-11
    info, xg, xo, o, ao, bo = _solve_pair(oracle, m, kind, order, d, fkw, method, precond, precision, tol)
    assert info.status == 0
    assert info.relres <= tol
    # the oracle recomputes the FP64 relative residual of the GPU solution
    assert o.relres(ao, bo, xg) <= 1.05 * tol
    assert np.linalg.norm(xg - xo) <= 1e-8 * np.linalg.norm(xo)
    if precision == 'mixed':
        assert info.outer_iterations >= 1


def test_solve_is_bit_reproducible(gpu_lib, oracle):
    import torch
    from opencmp_gb300 import fem
    m = M.unit_cube(4)
    g = fem.Space(m, 'H1', 2, m.bc_names)
    A = fem.Matrix(g)
    f = fem.make_form(mass=1.0, diff=1e-2, dt=1e-2, wind=(1.0, 0.5, 0.25))
    A.assemble(f)
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    fem.assemble_rhs(g, f, fem.make_rhs(src_const=1.0), b)
    sv = fem.KrylovSolver(A, method='GMRES', restart=20, tol=1e-10)
    xs = []
    for _ in range(2):
        x = torch.zeros_like(b)
        sv.solve(b, x)
        xs.append(x.cpu().numpy().tobytes())
    assert xs[0] == xs[1]


def test_nonfinite_rhs_is_reported(gpu_lib, oracle):
    """Fault injected on the host: a NaN in the right-hand side gives OCMP_ERR_NONFINITE, no hang."""
    import torch
    from opencmp_gb300 import fem, _lib
    m = M.unit_square(8)
    g = fem.Space(m, 'H1', 2, m.bc_names)
    A = fem.Matrix(g)
    A.assemble(fem.make_form(diff=1.0))
    b = torch.ones(g.ndof, dtype=torch.float64, device='cuda')
    k = int(np.flatnonzero(g.FreeDofs())[3])   # a NaN on a constrained row never enters the solve
    b[k] = float('nan')
    x = torch.zeros_like(b)
    info = fem.KrylovSolver(A, method='GMRES', tol=1e-8).solve(b, x, raise_on_fail=False)
    assert info.status == _lib.ERR_NONFINITE
    # an unreachable tolerance in few iterations reports NOT_CONVERGED
    b[k] = 1.0
    info = fem.KrylovSolver(A, method='CG', tol=1e-30, maxit=3).solve(b, torch.zeros_like(b), raise_on_fail=False)
    assert info.status == _lib.NOT_CONVERGED


def test_reference_fixture_transient_poisson_gpu(gpu_lib, oracle, coarse_mesh, ref_bounds):
    """The reference's transient Poisson fixture (implicit Euler, H1 order 3) on the GPU path."""
    import torch
    from opencmp_gb300 import fem
    m = coarse_mesh
    d = ['left', 'right']
    g, o = _spaces(oracle, m, 0, 3, d)
    dt = 1e-3
    f = fem.make_form(mass=1.0, diff=1.0, dt=dt)
    A = fem.Matrix(g)
    A.assemble(f)
    sv = fem.KrylovSolver(A, method='CG', tol=1e-12, maxit=1000)
    u = _t(o.project(oracle.SRC_POLY_X1MX, (1.0,)))
    b = torch.zeros_like(u)
    for _ in range(1000):
        fem.assemble_rhs(g, f, fem.make_rhs(dt=dt, mass=1.0, uprev=u), b)
        x = u.clone()
        g.set_boundary({m.bc_names.index('left'): 0.0, m.bc_names.index('right'): 0.0}, x)
        sv.solve(b, x)
        u = x
    err = o.l2_error(u.cpu().numpy(), oracle.SRC_NONE, ())
    exp = ref_bounds['by_id']['test_poisson.py::TestTransient::test_implicit_euler_cg']['bounds'][0]
    assert math.isclose(err, exp, rel_tol=ref_bounds['rtol']['value'], abs_tol=1e-12)
    analytic = 8 / math.pi ** 3 / math.sqrt(2) * (1 / (1 + math.pi ** 2 * 1e-3)) ** 1000
    assert abs(err - analytic) < 0.01 * analytic


@pytest.mark.gpu
def test_sell32_krylov_matrix_matches_csr(gpu_lib):
    """The FP32 Jacobi-scaled Krylov matrix written by the assembly in SELL-32 order (16-byte loads,
    a warp per slice of 32 rows) gives the mixed-precision GMRES the same products as the CSR copy,
    up to the FP32 summation order: iteration counts within 15 % and the same solution to the
    solve's accuracy."""
    import torch
    from opencmp_gb300 import fem
    m = M.unit_cube(8)
    g = fem.Space(m, 'H1', 2, m.bc_names)
    form = fem.make_form(mass=1.0, diff=1e-2, dt=1e-2, wind=(1.0, 0.5, 0.25))
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    fem.assemble_rhs(g, form, fem.make_rhs(dt=1e-2, src_const=1.0), b)
    out = {}
    for sell in (False, True):
        A = fem.Matrix(g, jacobi32=True, dfloat=True, sell=sell)
        A.assemble(form)
        x = torch.zeros_like(b)
        info = fem.KrylovSolver(A, method='GMRES', restart=30, precision='mixed', tol=1e-11).solve(b, x)
        assert info.status == 0 and info.relres <= 1e-11
        out[sell] = (x.cpu().numpy(), info.iterations)
    # near the FP32 round-off floor the refinement's inner cycles differ with the summation order
    assert abs(out[True][1] - out[False][1]) <= max(2, 0.15 * out[False][1]), (out[True][1], out[False][1])
    assert np.linalg.norm(out[True][0] - out[False][0]) <= 1e-8 * np.linalg.norm(out[False][0])
