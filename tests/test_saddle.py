"""Flexible GMRES with the Cahouet-Chabard pressure preconditioner (opencmp_gb300/saddle.py) on
the lid-driven cavity's Taylor-Hood systems.

CPU: the host FGMRES loop runs on CPU tensors with the oracle's matrices (scipy products, scipy
pressure solves) and must reproduce the oracle's direct solve, with iteration counts that do not
grow with the mesh; the lid's corner values decide whether the discrete lid leaks (and with it
whether the pressure carries a constant of order flux / (dt eps)).
GPU: the same solver through the library's SpMV and pressure CG against the oracle's direct solve.
"""
import numpy as np
import pytest

from opencmp_gb300 import mesh as M

DT, NU = 1e-3, 1e-3


def _cavity(n, k=2, leaky=False):
    """Oracle Taylor-Hood cavity system of one Euler IMEX step from rest, lid (1, 0).

    The lid is applied first and the walls last (corners at rest: the lid does not leak); with
    ``leaky`` all four labels are set in one call, where the label order gives one top corner the
    lid value and the other the wall value."""
    from oracle.ins import TaylorHood
    m = M.unit_square(n)
    th = TaylorHood(m, k, m.label_mask(m.bc_names))
    lab = {s: m.bc_names.index(s) for s in m.bc_names}
    u = np.zeros(th.ndof)
    walls = {lab['bottom']: (0.0, 0.0), lab['left']: (0.0, 0.0), lab['right']: (0.0, 0.0)}
    if leaky:
        th.set_boundary(m.label_mask(m.bc_names), {**walls, lab['top']: (1.0, 0.0)}, u)
    else:
        th.set_boundary(1 << lab['top'], {lab['top']: (1.0, 0.0)}, u)
        th.set_boundary(m.label_mask(['bottom', 'left', 'right']), walls, u)
    A = th.matrix(1.0, NU, DT)
    b = th.rhs(DT, mass=1.0, uprev=u, imex=u)
    return m, th, A, b, u


def _cc_cpu(th, A, inner_tol=None):
    """matvec / Cahouet-Chabard preconditioner on CPU tensors from the oracle's matrices; the pressure
    solve is exact (sparse LU) or, with inner_tol, a Jacobi-CG to that relative tolerance."""
    import scipy.sparse.linalg as spla
    import torch
    from oracle import oracle as O
    Q = th.Q
    Mp = Q.csr(Q.assemble(O.make_form(mass=1.0)))
    Lr = Q.csr(Q.assemble(O.make_form(mass=1e-10 / DT, diff=1.0)))
    lu = spla.splu(Lr.tocsc())
    n2 = 2 * th.nu
    dv = A.diagonal()[:n2]
    du = np.where(th.free[:n2], 1.0 / dv, 0.0)
    mpi = 1.0 / Mp.diagonal()
    dl = 1.0 / Lr.diagonal()
    counts = []

    def cg(r):
        x = np.zeros_like(r)
        res = r.copy()
        z = dl * res
        p = z.copy()
        rz = res @ z
        nr = np.linalg.norm(r)
        k = 0
        while np.linalg.norm(res) > inner_tol * nr and k < 2000:
            q = Lr @ p
            a = rz / (p @ q)
            x += a * p
            res -= a * q
            z = dl * res
            rz, rz0 = res @ z, rz
            p = z + rz / rz0 * p
            k += 1
        counts.append(k)
        return x

    def matvec(v, out):
        out.copy_(torch.from_numpy(A @ v.numpy()))

    def precond(r, z):
        rn = r.numpy()
        rp = rn[n2:]
        y = lu.solve(rp) if inner_tol is None else cg(rp)
        zn = np.concatenate([du * rn[:n2], -(y + DT * NU * mpi * rp) / DT ** 2])
        z.copy_(torch.from_numpy(zn))
    return matvec, precond, counts


def _solve_cpu(n, inner_tol=None, tol=1e-10):
    import torch
    from opencmp_gb300.saddle import fgmres
    m, th, A, b, u = _cavity(n)
    matvec, precond, counts = _cc_cpu(th, A, inner_tol)
    x = torch.from_numpy(u.copy())
    info = fgmres(matvec, precond, torch.from_numpy(b), x, torch.from_numpy(th.free), restart=50, tol=tol,
                  maxit=1000)
    return th, A, b, u, x.numpy(), info, counts


def test_lid_corners_decide_the_leak(oracle):
    """With one moving corner the discrete lid carries a net inflow of dt h / 2 through the pressure
    rows, and the eps-regularised pressure block turns it into a constant pressure of about
    flux / (dt eps |Omega|); with both top corners at rest the flux is zero to round-off."""
    for n in (8, 16):
        _, th, A, b, u = _cavity(n, leaky=True)
        fr = th.free
        bp = (b - A @ np.where(fr, 0.0, u))[2 * th.nu:]
        assert abs(bp.sum() - DT / (2 * n)) <= 1e-12 * DT
        x = th.solve(A, b, u)
        assert abs(x[2 * th.nu:].mean()) > 1e6
        _, th, A, b, u = _cavity(n)
        bp = (b - A @ np.where(th.free, 0.0, u))[2 * th.nu:]
        assert abs(bp.sum()) <= 1e-15
        x = th.solve(A, b, u)
        assert abs(x[2 * th.nu:].mean()) < 1.0


@pytest.mark.parametrize('inner_tol', [None, 0.1])
def test_fgmres_cahouet_chabard_matches_direct(oracle, inner_tol):
    its = []
    for n in (8, 16, 32):
        th, A, b, u, x, info, counts = _solve_cpu(n, inner_tol)
        assert info.status == 0 and info.relres <= 1e-10, (n, info.relres)
        xo = th.solve(A, b, u)
        n2 = 2 * th.nu
        assert np.linalg.norm(x[:n2] - xo[:n2]) <= 1e-7 * np.linalg.norm(xo[:n2])
        pd, po = x[n2:] - x[n2:].mean(), xo[n2:] - xo[n2:].mean()
        assert np.linalg.norm(pd - po) <= 1e-6 * np.linalg.norm(po)
        # the relative residual of the oracle's definition
        fr = th.free
        r = np.where(fr, b - A @ x, 0.0)
        r0 = np.where(fr, b - A @ np.where(fr, 0.0, u), 0.0)
        assert np.linalg.norm(r) <= 1.01 * info.relres * np.linalg.norm(r0)
        its.append(info.iterations)
    # mesh-independent: no growth from 16 x 16 to 32 x 32 beyond a quarter
    assert its[2] <= 1.25 * its[1] + 5, its
    assert its[2] <= 200, its


def test_fgmres_restarts_and_reports_like_the_library(oracle):
    """A short restart (10) forces several cycles; the iteration count, cycle count and initial relative
    residual follow the library's conventions (relres0 = 1 from a zero free part)."""
    import torch
    from opencmp_gb300.saddle import fgmres
    _, th, A, b, u = _cavity(8)
    matvec, precond, _ = _cc_cpu(th, A)
    x = torch.from_numpy(u.copy())
    info = fgmres(matvec, precond, torch.from_numpy(b), x, torch.from_numpy(th.free), restart=10, tol=1e-9,
                  maxit=2000)
    assert info.status == 0 and info.outer_iterations > 1
    assert abs(info.relres0 - 1.0) <= 1e-12
    # converged start: no iteration
    info2 = fgmres(matvec, precond, torch.from_numpy(b), x, torch.from_numpy(th.free), restart=5, tol=1e-6)
    assert info2.iterations == 0 and info2.status == 0
    # iteration cap: reports NOT_CONVERGED with the true residual
    x3 = torch.from_numpy(u.copy())
    info3 = fgmres(matvec, precond, torch.from_numpy(b), x3, torch.from_numpy(th.free), restart=5, tol=1e-14,
                   maxit=3)
    assert info3.status == 4 and info3.iterations == 3 and 0 < info3.relres < 1


# ------------------------------------------------------------------------------------------- GPU

def _gpu_cavity(n, precision='fp64', inner_tol=0.1, impl='library'):
    import torch
    from opencmp_gb300 import fem
    from opencmp_gb300.saddle import SaddleSolver
    m = M.unit_square(n)
    th = fem.TaylorHood(m, 2, m.bc_names)
    lab = {s: m.bc_names.index(s) for s in m.bc_names}
    u = torch.zeros(th.ndof, dtype=torch.float64, device='cuda')
    for c, val in ((0, 1.0), (1, 0.0)):
        th.V.set_boundary({lab['top']: val}, th.component(u, c))
        th.V.set_boundary({lab['bottom']: 0.0, lab['left']: 0.0, lab['right']: 0.0}, th.component(u, c))
    A = th.matrix()
    th.assemble(A, mass=1.0, nu=NU, dt=DT)
    b = torch.zeros_like(u)
    th.assemble_rhs(b, dt=DT, mass=1.0, uprev=u, imex=u)
    sv = SaddleSolver(th, A, restart=50, tol=1e-10, maxit=1000, inner_tol=inner_tol, precision=precision, impl=impl)
    sv.update(mass=1.0, dt=DT, nu=NU)
    return th, A, b, u, sv


@pytest.mark.gpu
@pytest.mark.parametrize('precision,impl', [('fp64', 'library'), ('mixed', 'library'), ('fp64', 'host'),
                                            ('mixed', 'host')])
def test_gpu_saddle_solver_matches_oracle(gpu_lib, oracle, precision, impl):
    """Both implementations of the Cahouet-Chabard solve against the oracle: the library's device
    GMRES with the exact (strip-factorised) pressure block, and host FGMRES with the inexact
    Jacobi-CG pressure block, whose inner iterations it reports."""
    its = []
    for n in (16, 32):
        th, A, b, u, sv = _gpu_cavity(n, precision, impl=impl)
        _, tho, Ao, bo, uo = _cavity(n)
        np.testing.assert_allclose(u.cpu().numpy(), uo, rtol=0, atol=1e-15)
        assert np.abs(b.cpu().numpy() - bo).max() <= 1e-12 * np.abs(bo).max()
        x = u.clone()
        info = sv.solve(b, x)
        assert info.status == 0 and info.relres <= 1e-10
        xo = tho.solve(Ao, bo, uo)
        xg = x.cpu().numpy()
        n2 = 2 * tho.nu
        assert np.linalg.norm(xg[:n2] - xo[:n2]) <= 1e-7 * np.linalg.norm(xo[:n2])
        pd, po = xg[n2:] - xg[n2:].mean(), xo[n2:] - xo[n2:].mean()
        assert np.linalg.norm(pd - po) <= 1e-6 * np.linalg.norm(po)
        fr = tho.free
        r = np.where(fr, bo - Ao @ xg, 0.0)
        r0 = np.where(fr, bo - Ao @ np.where(fr, 0.0, uo), 0.0)
        # the GPU solution satisfies the oracle's system (its matrix equal to the GPU's to 1e-12)
        assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(r0)
        assert (info.inner_iterations > 0) == (impl == 'host')
        its.append(info.iterations)
    assert its[1] <= 1.25 * its[0] + 5 and its[1] <= 200, its


def test_fgmres_edge_cases():
    """Host FGMRES on small dense systems (CPU tensors): an exact preconditioner converges in one
    iteration (lucky breakdown, |w| = 0); a zero operator reports BREAKDOWN and leaves x alone;
    constrained entries of x are kept; a zero right-hand side with a zero free part returns at once."""
    import torch
    from opencmp_gb300 import _lib as LB
    from opencmp_gb300.saddle import fgmres
    rng = np.random.default_rng(1)
    n = 12
    A = rng.standard_normal((n, n)) + n * np.eye(n)
    free = np.ones(n, bool)
    free[[0, 5]] = False
    b = torch.from_numpy(rng.standard_normal(n))
    x = torch.zeros(n, dtype=torch.float64)
    x[0], x[5] = 2.0, -1.0
    fr = torch.from_numpy(free)

    def mv(v, out):
        out.copy_(torch.from_numpy(A @ v.numpy()))

    # exact inverse of the free block as the preconditioner
    Aff = A[np.ix_(free, free)]
    Affi = np.linalg.inv(Aff)

    def exact(r, z):
        zn = np.zeros(n)
        zn[free] = Affi @ r.numpy()[free]
        z.copy_(torch.from_numpy(zn))
    info = fgmres(mv, exact, b, x, fr, restart=10, tol=1e-12)
    assert info.status == LB.OK and info.iterations == 1 and info.relres <= 1e-12
    assert x[0] == 2.0 and x[5] == -1.0
    xs = x.numpy()
    assert np.allclose(A[free] @ xs, b.numpy()[free], rtol=0, atol=1e-10)
    # zero operator: breakdown, x untouched
    x2 = torch.zeros(n, dtype=torch.float64)
    info2 = fgmres(lambda v, out: out.zero_(), lambda r, z: z.copy_(r * fr), b, x2, fr, restart=10, tol=1e-8)
    assert info2.status == LB.BREAKDOWN and info2.iterations == 1 and float(x2.abs().max()) == 0.0
    # zero right-hand side and zero free part: already converged (relres 0 over a unit norm)
    x3 = torch.zeros(n, dtype=torch.float64)
    info3 = fgmres(mv, exact, torch.zeros(n, dtype=torch.float64), x3, torch.ones(n, dtype=torch.bool), tol=1e-8)
    assert info3.status == LB.OK and info3.iterations == 0 and info3.relres == 0.0
