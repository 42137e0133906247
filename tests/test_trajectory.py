"""Trajectory of the optimised transient path against the oracle's FP64 implicit-Euler trajectory.

The optimised step is the one the benchmark times on config 3: double-float assembly (matrix,
Jacobi-scaled FP32 Krylov matrix and mass right-hand side), the learned initial guess under its
convergence judge (cubic extrapolation in time plus the trained network), FP32-inner GMRES(30) with
FP64 refinement. It runs here on the 16^3 x 6 mesh from the Gaussian start for 24 steps, after the
network was trained on the solver's own trajectories at two other diffusivities.

The oracle's trajectory solves every step to a 1e-13 relative residual. A solve stopped at a 1e-8
relative residual leaves a solution error of a few 1e-5 on this mass-dominated system (the oracle's
own FP64 GMRES from the previous-step guess, stopped at 1e-8, drifts 3.4e-5 from the tight
trajectory over these steps), so the check is twofold:
* at the benchmark tolerance (1e-8) every step meets it and stays within 1e-4 of the tight
  trajectory, the band the reference's own stopping rule allows;
* with the tolerance at 1e-12 the same path follows the tight trajectory to 1e-7 at every step, and
  its final state to 1e-8: nothing in the path (double-float assembly, FP32 inner iteration,
  extrapolated or learned start) drifts beyond what the stopping tolerance decides.
"""
import numpy as np
import pytest

from opencmp_gb300 import mesh as M

pytestmark = pytest.mark.gpu

EPS, WIND, DT = 1e-2, (1.0, 0.5, 0.25), 1e-3


def gaussian(X):
    c = np.array([0.25, 0.25, 0.25])
    return np.exp(-((X - c) ** 2).sum(-1) / (2 * 0.1 ** 2))


def _setup(n):
    import torch
    from opencmp_gb300 import fem
    from opencmp_gb300.guess import LearnedGuess
    m = M.unit_cube(n)
    space = fem.Space(m, 'H1', 2, m.bc_names)
    A = fem.Matrix(space, jacobi32=True, dfloat=True)
    u0 = torch.as_tensor(fem.interpolate_p2(space, gaussian), device='cuda')
    guess = LearnedGuess(space, k=5, base_order=3, seed=0)
    # training on the solver's own trajectories at two other diffusivities (the held-out one is EPS)
    b = torch.zeros(space.ndof, dtype=torch.float64, device='cuda')
    sv = fem.KrylovSolver(A, method='GMRES', restart=30, precond='jacobi', precision='mixed', tol=1e-8, maxit=2000,
                          inner_tol=1e-4, check_every=6)
    keep = []
    for eps in (3e-3, 3e-2):
        f = fem.make_form(mass=1.0, diff=eps, dt=DT, wind=WIND)
        A.assemble(f)
        sv.update()
        At = fem.Matrix(space)
        At.assemble(f)
        keep.append(At)
        u = u0.clone()
        guess.reset()
        guess.push(u)
        for _ in range(20):
            fem.assemble_rhs(space, f, fem.make_rhs(dt=DT, mass=1.0, uprev=u), b)
            x = torch.empty_like(u)
            guess.extrapolate(x)
            sv.solve(b, x)
            guess.collect(x, At, b)
            guess.push(x)
            u = x
    guess.train(steps=150, lr=3e-3)
    guess.drop_samples()
    return m, space, A, u0, guess


def _trajectory(space, A, u0, guess, tol, steps):
    import torch
    from opencmp_gb300 import fem
    sv = fem.KrylovSolver(A, method='GMRES', restart=30, precond='jacobi', precision='mixed', tol=tol, maxit=4000,
                          inner_tol=1e-4, check_every=6)
    form = fem.make_form(mass=1.0, diff=EPS, dt=DT, wind=WIND)
    b = torch.zeros(space.ndof, dtype=torch.float64, device='cuda')
    u = u0.clone()
    guess.reset()
    guess.reset_judge()
    guess.push(u)
    out, kinds, infos = [], [], []
    for _ in range(steps):
        A.assemble(form)
        sv.update()
        fem.assemble_rhs(space, form, fem.make_rhs(dt=DT, mass=1.0, uprev=u, dfloat=True), b)
        x = torch.empty_like(u)
        used = guess.predict(x)
        info = sv.solve(b, x)
        guess.push(x)
        guess.judge(info, used)
        out.append(x.cpu().numpy())
        kinds.append(used)
        infos.append(info)
        u = x
    return out, kinds, infos


def _oracle_trajectory(oracle, m, steps):
    from opencmp_gb300.fem import interpolate_p2_arrays
    o = oracle.Space(m, oracle.H1, 2, m.label_mask(m.bc_names))
    f = oracle.make_form(mass=1.0, diff=EPS, dt=DT, wind=WIND)
    A = o.assemble(f)
    u = interpolate_p2_arrays(m.coords, o.sorted_conn(), o.dofs(), o.ndof, gaussian)
    out = []
    for _ in range(steps):
        b = o.rhs(f, oracle.make_rhs(dt=DT, mass=1.0, uprev=u))
        x = u.copy()
        o.gmres(A, b, x, restart=60, precond=1, tol=1e-13, maxit=5000)
        out.append(x)
        u = x
    return o, A, out


def test_optimised_trajectory_follows_the_oracle(gpu_lib, oracle):
    steps = 24
    m, space, A, u0, guess = _setup(16)
    assert (space.dofs().ravel() == oracle.Space(m, oracle.H1, 2, m.label_mask(m.bc_names)).dofs().ravel()).all()
    o, Ao, ref = _oracle_trajectory(oracle, m, steps)
    # at the benchmark's tolerance
    traj, kinds, infos = _trajectory(space, A, u0, guess, 1e-8, steps)
    assert all(i.status == 0 and i.relres <= 1e-8 for i in infos)
    assert 'network' in kinds, kinds          # the trained network did start solves under its judge
    dev = [np.linalg.norm(x - r) / np.linalg.norm(r) for x, r in zip(traj, ref)]
    assert max(dev) <= 1e-4, dev
    # with a tight tolerance the same path follows the oracle's trajectory
    traj, kinds, infos = _trajectory(space, A, u0, guess, 1e-12, steps)
    assert all(i.status == 0 and i.relres <= 1e-12 for i in infos)
    dev = [np.linalg.norm(x - r) / np.linalg.norm(r) for x, r in zip(traj, ref)]
    assert max(dev) <= 1e-7, dev
    assert dev[-1] <= 1e-8, dev[-1]
