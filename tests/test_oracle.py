"""CPU tests of the oracle (the checker): pinned against the reference's own fixtures and test
bounds, against manufactured solutions, and against scipy's direct solver."""
import math

import numpy as np
import pytest

from opencmp_gb300 import mesh as M


def test_config1_counts(oracle):
    s = oracle.Space(M.unit_square(64), oracle.H1, 2, 0b1111)
    assert (s.ndof, s.nnz) == (16641, 189441)


def test_dg_and_tet_counts(oracle):
    m = M.unit_square(16)
    s = oracle.Space(m, oracle.L2, 2, 0)
    nif = oracle.lib().or_space_ninterior_facets(s.h)
    assert nif == 3 * 16 * 16 - 2 * 16
    assert s.ndof == m.ne * 6 and s.nnz == 36 * (m.ne + 2 * nif)
    # Kuhn-split cube: axis edges, one diagonal per grid face, one body diagonal per cube
    n = 4
    t = oracle.Space(M.unit_cube(n), oracle.H1, 2, 0)
    ned = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3
    assert t.ndof == (n + 1) ** 3 + ned
    n = 64
    assert (n + 1) ** 3 + 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3 == 2146689  # the 3D benchmark mesh


@pytest.mark.parametrize('p,rate', [(1, 4.0), (2, 8.0), (3, 16.0)])
def test_h1_poisson_convergence(oracle, p, rate):
    f = oracle.make_form(diff=1.0)
    r = oracle.make_rhs(src_kind=oracle.SRC_SINPROD, src=(2 * math.pi ** 2,))
    errs = []
    for n in (8, 16):
        s = oracle.Space(M.unit_square(n), oracle.H1, p, 0b1111)
        A = s.assemble(f)
        b = s.rhs(f, r)
        x = np.zeros(s.ndof)
        s.cg(A, b, x, tol=1e-13)
        errs.append(s.l2_error(x, oracle.SRC_SINPROD, (1.0,)))
    assert errs[0] / errs[1] > 0.85 * rate


@pytest.mark.parametrize('p,rate', [(1, 4.0), (2, 8.0)])
def test_dg_sipg_convergence_and_symmetry(oracle, p, rate):
    f = oracle.make_form(diff=1.0, dg=True, ipc=10.0, nitsche_mask=0b1111)
    r = oracle.make_rhs(src_kind=oracle.SRC_SINPROD, src=(2 * math.pi ** 2,))
    errs = []
    for n in (8, 16):
        s = oracle.Space(M.unit_square(n), oracle.L2, p, 0)
        A = s.assemble(f)
        b = s.rhs(f, r)
        x = np.zeros(s.ndof)
        s.gmres(A, b, x, restart=60, precond=2, tol=1e-12, maxit=20000)
        errs.append(s.l2_error(x, oracle.SRC_SINPROD, (1.0,)))
        Ac = s.csr(A)
        assert abs(Ac - Ac.T).max() < 1e-12 * abs(Ac).max()
    assert errs[0] / errs[1] > 0.85 * rate


def test_krylov_matches_direct(oracle):
    import scipy.sparse.linalg as spla
    m = M.unit_square(12)
    s = oracle.Space(m, oracle.H1, 2, m.label_mask(['left', 'bottom']))
    f = oracle.make_form(mass=1.0, diff=0.05, dt=0.1, wind=(1.0, 0.3), outflow_mask=m.label_mask(['right', 'top']))
    A = s.assemble(f)
    b = s.rhs(f, oracle.make_rhs(dt=0.1, src_kind=oracle.SRC_CONST, src=(1.0,)))
    fr = s.freedofs()
    Ac = s.csr(A)
    xd = np.zeros(s.ndof)
    xd[fr] = spla.spsolve(Ac[fr][:, fr].tocsc(), b[fr])
    x = np.zeros(s.ndof)
    it, rr = s.gmres(A, b, x, restart=40, precond=1, tol=1e-13)
    assert rr <= 1e-13
    assert np.linalg.norm(x - xd) <= 1e-10 * np.linalg.norm(xd)


def test_element_matrix_identities(oracle):
    m = M.unit_cube(2)
    s = oracle.Space(m, oracle.H1, 2, 0)
    K = s.element_matrix(oracle.make_form(diff=1.0), 3)
    # constants are in the kernel of the stiffness matrix (vertex functions sum to one)
    assert np.abs(K[:, :4].sum(axis=1)).max() < 1e-13
    Mm = s.element_matrix(oracle.make_form(mass=1.0), 3)
    assert abs(Mm[:4, :4].sum() - 1.0 / 8 / 6) < 1e-15


def _transient_poisson(oracle, m, dg):
    dmask = m.label_mask(['left', 'right'])
    s = oracle.Space(m, oracle.L2 if dg else oracle.H1, 3, dmask)
    dt = 1e-3
    f = oracle.make_form(mass=1.0, diff=1.0, dt=dt, dg=dg, ipc=10.0, nitsche_mask=dmask if dg else 0)
    A = s.assemble(f)
    u = s.project(oracle.SRC_POLY_X1MX, (1.0,))
    for _ in range(1000):
        b = s.rhs(f, oracle.make_rhs(dt=dt, mass=1.0, uprev=u))
        x = u.copy()
        s.set_boundary(dmask, {}, x)
        if dg:
            s.gmres(A, b, x, restart=50, precond=2, tol=1e-13)
        else:
            s.cg(A, b, x, tol=1e-13)
        u = x
    return s.l2_error(u, oracle.SRC_NONE, ())


@pytest.mark.parametrize('dg', [False, True])
def test_reference_fixture_transient_poisson(oracle, coarse_mesh, ref_bounds, dg):
    """pytests/full_system/poisson (implicit Euler, unit_square_coarse.vol, H1/L2 order 3)."""
    err = _transient_poisson(oracle, coarse_mesh, dg)
    exp = ref_bounds['by_id']['test_poisson.py::TestTransient::test_implicit_euler_cg']['bounds'][0]
    rtol = ref_bounds['rtol']['value']
    assert math.isclose(err, exp, rel_tol=rtol, abs_tol=1e-12)           # the reference's own check
    analytic = 8 / math.pi ** 3 / math.sqrt(2) * (1 / (1 + math.pi ** 2 * 1e-3)) ** 1000
    assert abs(err - analytic) < 0.01 * analytic                          # semi-discrete exact value


def test_reference_fixture_mcins_diffusion_convection(oracle, coarse_mesh, ref_bounds):
    """pytests/full_system/mcins/diffusion_convection (implicit Euler CG, order 3, components a, b)."""
    m = coarse_mesh
    dmask = m.label_mask(['left'])
    s = oracle.Space(m, oracle.H1, 3, dmask)
    dt = 0.01
    f = oracle.make_form(mass=1.0, diff=0.1, dt=dt, wind=(1.0, 0.0), wn_mask=m.label_mask(['top', 'bottom', 'right']))
    A = s.assemble(f)

    def ramp(t):
        return 0.5 * (0 - 1) * math.cos(t * math.pi) + 0.5 if t < 1.0 else 1.0
    bounds = ref_bounds['by_id']['test_mcins.py::TestDiffusionConvection::test_implicit_euler_cg']['bounds']
    for (g, ic, ref), exp in zip([(lambda t: 1.1 - ramp(t), 1.1, 0.1), (ramp, 0.0, 1.0)], bounds):
        u = s.project(oracle.SRC_CONST, (ic,))
        for k in range(1000):
            b = s.rhs(f, oracle.make_rhs(dt=dt, mass=1.0, uprev=u))
            x = u.copy()
            s.set_boundary(dmask, {m.bc_names.index('left'): g((k + 1) * dt)}, x)
            s.gmres(A, b, x, restart=50, precond=1, tol=1e-14)
            u = x
        err = s.l2_error(u, oracle.SRC_CONST, (ref,))
        assert math.isclose(err, exp, rel_tol=3, abs_tol=1e-12)
