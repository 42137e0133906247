"""Taylor-Hood (incompressible Navier-Stokes) system on the GPU (ocmp_th_*) against the oracle's
restatement (oracle/ins.py): CSR pattern bit-exact, matrix and right-hand side entries to 1e-12,
a steady Stokes solve through GMRES with the block-diagonal preconditioner, the error functionals,
and the oracle's own Stokes convergence rate (CPU)."""
import math

import numpy as np
import pytest

from opencmp_gb300 import mesh as M


def _stokes_case():
    """Manufactured steady Stokes: u = curl psi with psi = (x(1-x)y(1-y))^2, p = x - 1/2, nu = 1,
    f = -lap u + grad p (expanded symbolically)."""
    def exact(X):
        x, y = X[..., 0], X[..., 1]
        ux = 2 * x ** 2 * y * (x - 1) ** 2 * (y - 1) * (2 * y - 1)
        uy = -2 * x * y ** 2 * (x - 1) * (2 * x - 1) * (y - 1) ** 2
        return np.stack([ux, uy], -1)

    def force(X):
        x, y = X[..., 0], X[..., 1]
        fx = -4 * (2 * y - 1) * (3 * x ** 4 - 6 * x ** 3 + 6 * x ** 2 * y ** 2 - 6 * x ** 2 * y + 3 * x ** 2
                                 - 6 * x * y ** 2 + 6 * x * y + y ** 2 - y) + 1.0
        fy = 4 * (2 * x - 1) * (6 * x ** 2 * y ** 2 - 6 * x ** 2 * y + x ** 2 - 6 * x * y ** 2 + 6 * x * y - x
                                + 3 * y ** 4 - 6 * y ** 3 + 3 * y ** 2)
        return np.stack([fx, fy], -1)
    return exact, force


def test_oracle_taylor_hood_stokes_rate(oracle):
    from oracle.ins import TaylorHood
    exact, force = _stokes_case()
    errs = []
    for n in (4, 8, 16):
        m = M.unit_square(n)
        th = TaylorHood(m, 2, m.label_mask(m.bc_names))
        A = th.matrix(0.0, 1.0, 1.0)
        f = force(th.quad_points())
        Fe = np.einsum('eq,qi,eqc->eci', th.W, th.phi, f)
        b = np.zeros(th.ndof)
        np.add.at(b, th.dv, Fe[:, 0])
        np.add.at(b, th.nu + th.dv, Fe[:, 1])
        u = th.solve(A, b, np.zeros(th.ndof))
        errs.append(th.l2_error(u, exact))
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(rates) > 2.8, (errs, rates)


def _pair(oracle, n, k):
    from opencmp_gb300 import fem
    from oracle.ins import TaylorHood
    m = M.unit_square(n)
    mask = m.label_mask(m.bc_names)
    return m, fem.TaylorHood(m, k, m.bc_names), TaylorHood(m, k, mask)


@pytest.mark.gpu
@pytest.mark.parametrize('k,oseen,tcoef', [(2, False, None), (2, True, None), (3, False, None), (3, True, None),
                                           (2, False, 2e-3)])
def test_th_matrix_matches_oracle(gpu_lib, oracle, k, oseen, tcoef):
    import torch
    m, g, o = _pair(oracle, 6, k)
    rng = np.random.default_rng(k)
    w = rng.standard_normal(o.ndof) if oseen else None
    A = g.matrix()
    g.assemble(A, mass=1.0, nu=1e-3, dt=1e-3, eps_p=1e-10,
               wind=torch.as_tensor(w, device='cuda') if oseen else None, tcoef=tcoef)
    Ao = o.matrix(1.0, 1e-3, 1e-3, wind=w, tcoef=tcoef)
    rp, col = g.C.pattern()
    np.testing.assert_array_equal(rp, Ao.indptr)
    np.testing.assert_array_equal(col, Ao.indices)
    v = A.values()
    assert np.abs(v - Ao.data).max() <= 1e-12 * np.abs(Ao.data).max()
    free = np.concatenate([o.V.freedofs(), o.V.freedofs(), np.ones(o.np_, bool)])
    np.testing.assert_array_equal(g.C.FreeDofs(), free)


@pytest.mark.gpu
@pytest.mark.parametrize('k', [2, 3])
def test_th_rhs_matches_oracle(gpu_lib, oracle, k):
    import torch
    m, g, o = _pair(oracle, 5, k)
    rng = np.random.default_rng(3)
    u0 = rng.standard_normal(o.ndof)
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    ut = torch.as_tensor(u0, device='cuda')
    u1 = rng.standard_normal(o.ndof)
    g.assemble_rhs(b, dt=0.01, src=(0.5, -1.0), mass=1.0, uprev=ut, imex=ut)
    g.assemble_rhs(b, dt=0.01, imex=torch.as_tensor(u1, device='cuda'), imex_coef=-3.0, accumulate=True)
    bo = o.rhs(0.01, f=(0.5, -1.0), mass=1.0, uprev=u0, imex=u0) + o.rhs(0.01, imex=u1, imex_coef=-3.0)
    bg = b.cpu().numpy()
    assert np.abs(bg - bo).max() <= 1e-12 * np.abs(bo).max()


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_th_stokes_solve_matches_oracle(gpu_lib, oracle, precision):
    import torch
    from opencmp_gb300 import fem
    exact, force = _stokes_case()
    m, g, o = _pair(oracle, 12, 2)
    A = g.matrix()
    g.assemble(A, mass=0.0, nu=1.0, dt=1.0)
    fq = torch.as_tensor(force(g.quad_points()), device='cuda')
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    g.assemble_rhs(b, dt=1.0, src_qp=fq)
    dinv = torch.zeros_like(b)
    g.block_diag(A, dinv)
    sv = fem.KrylovSolver(A, method='GMRES', restart=100, precond='user', precision=precision, tol=1e-10, maxit=20000)
    sv.set_diag(dinv)
    sv.update()
    x = torch.zeros_like(b)
    info = sv.solve(b, x)
    assert info.status == 0 and info.relres <= 1e-10
    Ao = o.matrix(0.0, 1.0, 1.0)
    f = force(o.quad_points())
    Fe = np.einsum('eq,qi,eqc->eci', o.W, o.phi, f)
    bo = np.zeros(o.ndof)
    np.add.at(bo, o.dv, Fe[:, 0])
    np.add.at(bo, o.nu + o.dv, Fe[:, 1])
    assert np.abs(b.cpu().numpy() - bo).max() <= 1e-12 * np.abs(bo).max()
    xo = o.solve(Ao, bo, np.zeros(o.ndof))
    xg = x.cpu().numpy()
    nv = 2 * o.nu
    assert np.linalg.norm(xg[:nv] - xo[:nv]) <= 1e-7 * np.linalg.norm(xo[:nv])
    l2, dv = g.errors(x, torch.as_tensor(exact(g.quad_points()), device='cuda'))
    assert abs(l2 - o.l2_error(xo, exact)) <= 1e-6 * l2
    assert abs(dv - o.divergence(xo)) <= 1e-6 * dv
