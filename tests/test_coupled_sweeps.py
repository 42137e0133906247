"""Segregated sweeps over coupled reaction variables (solvers.Solver._solve_all) on a small dense
stand-in for each variable's system: the sweeps reach the compound system's solution, start every
solve from the previous sweep's values, and converge in a few sweeps at any dt. No GPU."""
import types

import numpy as np
import pytest
import torch

from opencmp_gb300.solvers import Solver

# OpenCMP's coupled first-order reaction fixture: a' = -5a + 4.5b, b' = 5a - 5b, c' = 0.5b
K_OWN = {'a': -5.0, 'b': -5.0, 'c': 0.0}
K_CROSS = {'a': {'b': 4.5}, 'b': {'a': 5.0}, 'c': {'b': 0.5}}
N = 12


def _system():
    rng = np.random.default_rng(3)
    B = rng.standard_normal((N, N))
    Mm = B @ B.T / N + np.eye(N)           # a mass-like SPD matrix
    L = np.diag(np.full(N, 2.0)) - np.diag(np.ones(N - 1), 1) - np.diag(np.ones(N - 1), -1)
    return torch.tensor(Mm), torch.tensor(L)


class FakeSweeps(Solver):
    """The sweep driver of Solver with each variable's theta step replaced by a dense solve of
    (M - theta dt k_own M + theta dt L) u = M u^n + theta dt sum_j k_j M c_j (+ the explicit half)."""

    def __init__(self):
        self.M, self.L = _system()
        self.model = types.SimpleNamespace(vars={n: types.SimpleNamespace(name=n) for n in 'abc'},
                                           coupled=lambda: True)
        self.guess_mode = 'previous'
        self.warm_flags = []
        self.guesses = []
        self.solves = 0

    def _solve_var(self, v, theta, dt, t_new, t_old, transient, u_from=None, u_to=None, warm=False):
        olds, cur = self._coupling
        self.warm_flags.append(warm)
        self.guesses.append(u_to.clone())
        n = v.name
        A = self.M * (1 - theta * dt * K_OWN[n]) + theta * dt * self.L
        rhs = self.M @ u_from - (1 - theta) * dt * (self.L - K_OWN[n] * self.M) @ u_from
        for o, k in K_CROSS[n].items():
            rhs = rhs + theta * dt * k * (self.M @ cur[o]) + (1 - theta) * dt * k * (self.M @ olds[o])
        u_to.copy_(torch.linalg.solve(A, rhs))
        self.solves += 1


def _compound(sw, theta, dt, olds):
    """The compound system's solution, assembled as one block matrix."""
    M, L = sw.M.numpy(), sw.L.numpy()
    idx = {n: i for i, n in enumerate('abc')}
    A = np.zeros((3 * N, 3 * N))
    b = np.zeros(3 * N)
    for n, i in idx.items():
        A[i * N:(i + 1) * N, i * N:(i + 1) * N] = M * (1 - theta * dt * K_OWN[n]) + theta * dt * L
        u0 = olds[n].numpy()
        b[i * N:(i + 1) * N] = M @ u0 - (1 - theta) * dt * (L - K_OWN[n] * M) @ u0
        for o, k in K_CROSS[n].items():
            j = idx[o]
            A[i * N:(i + 1) * N, j * N:(j + 1) * N] -= theta * dt * k * M
            b[i * N:(i + 1) * N] += (1 - theta) * dt * k * M @ olds[o].numpy()
    x = np.linalg.solve(A, b)
    return {n: x[i * N:(i + 1) * N] for n, i in idx.items()}


@pytest.mark.parametrize('dt', [3.3e-4, 0.05, 0.5, 5.0, 50.0])
@pytest.mark.parametrize('theta', [1.0, 0.5])
def test_sweeps_reach_compound_solution(dt, theta):
    sw = FakeSweeps()
    rng = np.random.default_rng(7)
    src = {n: torch.tensor(rng.uniform(0.0, 1.0, N)) for n in 'abc'}
    olds = {n: src[n].clone() for n in 'abc'}
    dst = {n: torch.zeros(N, dtype=torch.float64) for n in 'abc'}
    sw._solve_all(theta, dt, dt, 0.0, True, src=src, dst=dst)
    ref = _compound(sw, theta, dt, olds)
    for n in 'abc':
        assert np.linalg.norm(dst[n].numpy() - ref[n]) <= 1e-9 * np.linalg.norm(ref[n])
        assert torch.equal(src[n], olds[n])        # the step's start values are untouched
    # plain Gauss-Seidel needs 186 sweeps here at dt = 50 (contraction near 0.9), the mixing 26
    assert sw.solves <= 3 * 30
    assert all(sw.warm_flags)
    assert sw._coupling is None


def test_each_sweep_starts_from_the_previous_sweeps_values():
    sw = FakeSweeps()
    src = {n: torch.full((N,), 0.5, dtype=torch.float64) for n in 'abc'}
    dst = {n: torch.zeros(N, dtype=torch.float64) for n in 'abc'}
    seen = []

    orig = FakeSweeps._solve_var

    def record(self, v, *a, **kw):
        orig(self, v, *a, **kw)
        seen.append((v.name, kw['u_to'].clone()))
    sw._solve_var = types.MethodType(record, sw)
    sw._solve_all(1.0, 0.5, 0.5, 0.0, True, src=src, dst=dst)
    # the first sweep starts from the step's start values, the second from the first sweep's results
    assert torch.equal(sw.guesses[0], src['a'])
    assert torch.equal(sw.guesses[3], seen[0][1])


def test_unconverged_sweeps_raise():
    sw = FakeSweeps()
    sw.max_sweeps = 2
    src = {n: torch.full((N,), 0.5, dtype=torch.float64) for n in 'abc'}
    dst = {n: torch.zeros(N, dtype=torch.float64) for n in 'abc'}
    with pytest.raises(RuntimeError, match='did not converge'):
        sw._solve_all(1.0, 50.0, 50.0, 0.0, True, src=src, dst=dst)
    assert sw._coupling is None
