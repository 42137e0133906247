"""Learned initial guess: GPU kernels against the NumPy oracle, and the gain of the trained network
over the previous-step guess OpenCMP uses (opencmp/models/base_model.py:925-937)."""
import numpy as np
import pytest

from opencmp_gb300 import mesh as M


def test_oracle_mlp_gradient_matches_finite_differences():
    from oracle import mlp
    rng = np.random.default_rng(0)
    F = 4
    P = rng.standard_normal(mlp.layout(F)['n']) * 0.3
    X = rng.standard_normal((50, F))
    T = rng.standard_normal(50)
    loss, g = mlp.loss_grad(P, X, T)
    eps = 1e-6
    for p in rng.choice(len(P), 40, replace=False):
        Pp, Pm = P.copy(), P.copy()
        Pp[p] += eps
        Pm[p] -= eps
        fd = (mlp.loss_grad(Pp, X, T)[0] - mlp.loss_grad(Pm, X, T)[0]) / (2 * eps)
        assert abs(fd - g[p]) <= 1e-6 * max(1.0, abs(g[p]))


@pytest.mark.gpu
def test_gpu_mlp_forward_and_gradients_match_oracle(gpu_lib):
    import torch
    from opencmp_gb300.guess import GuessNet
    from oracle import mlp
    rng = np.random.default_rng(3)
    F = 4
    net = GuessNet(F, seed=5)
    P = (rng.standard_normal(net.nparams) * 0.3).astype(np.float32)
    net.set_params(P)
    assert np.array_equal(net.params(), P)
    X = rng.standard_normal((3000, F)).astype(np.float32)
    T = rng.standard_normal(3000).astype(np.float32)
    Xd, Td = torch.as_tensor(X, device='cuda'), torch.as_tensor(T, device='cuda')
    Y = torch.empty(3000, dtype=torch.float32, device='cuda')
    net.forward(Xd, Y)
    yo, _ = mlp.forward(P.astype(np.float64), X.astype(np.float64))
    assert np.abs(Y.cpu().numpy() - yo).max() <= 1e-5 * max(1.0, np.abs(yo).max())
    loss, g = net.loss_grad(Xd, Td, want_grad=True)
    lo, go = mlp.loss_grad(P.astype(np.float64), X.astype(np.float64), T.astype(np.float64))
    assert abs(loss - lo) <= 1e-5 * lo
    assert np.abs(g - go).max() <= 1e-4 * np.abs(go).max()
    # deterministic reductions: the same gradient bits twice
    _, g2 = net.loss_grad(Xd, Td, want_grad=True)
    assert g.tobytes() == g2.tobytes()


def _transient(space, A, sv, guess, eps, steps, collect=False, use=False):
    import torch
    from opencmp_gb300 import fem
    form = fem.make_form(mass=1.0, diff=eps, dt=1e-3, wind=(1.0, 0.5, 0.25))
    A.assemble(form)
    sv.update()
    X = space.mesh.coords
    u = torch.as_tensor(fem.interpolate_p2(space, lambda P: np.exp(-((P - 0.3) ** 2).sum(-1) / 0.02)),
                        device='cuda')
    b = torch.zeros_like(u)
    guess.reset()
    guess.push(u)
    stats = []
    for _ in range(steps):
        fem.assemble_rhs(space, form, fem.make_rhs(dt=1e-3, mass=1.0, uprev=u), b)
        x = torch.empty_like(u)
        if use:
            guess.predict(x, A, b)
        else:
            x.copy_(u)
        info = sv.solve(b, x)
        stats.append((info.iterations, info.relres0, info.relres))
        if collect:
            guess.collect(x, A, b)
        guess.push(x)
        u = x
    return stats


@pytest.mark.gpu
def test_trained_guess_beats_previous_step_guess(gpu_lib):
    """Trains on eps in {2e-3, 2e-2, 7e-2}, evaluates on held-out eps = 1e-2."""
    from opencmp_gb300 import fem
    from opencmp_gb300.guess import LearnedGuess
    m = M.unit_cube(10)
    space = fem.Space(m, 'H1', 2, m.bc_names)
    A = fem.Matrix(space, jacobi32=True, dfloat=True)
    sv = fem.KrylovSolver(A, method='GMRES', restart=30, precision='mixed', tol=1e-8, maxit=500, inner_tol=1e-4)
    guess = LearnedGuess(space, k=4, use_residual=True, seed=0)
    for eps in (2e-3, 2e-2, 7e-2):
        _transient(space, A, sv, guess, eps, 20, collect=True)
    before = guess.eval_loss()
    guess.train(steps=300, batch=1 << 14, lr=3e-3)
    after = guess.eval_loss()
    # training starts from the linear-extrapolation network (linear skip = first difference)
    assert after < before
    base = _transient(space, A, sv, guess, 1e-2, 12)
    learned = _transient(space, A, sv, guess, 1e-2, 12, use=True)
    # every solve reaches the FP64 tolerance whatever the guess
    assert max(s[2] for s in base + learned) <= 1e-8
    it_base = np.mean([s[0] for s in base[4:]])
    it_learn = np.mean([s[0] for s in learned[4:]])
    r0_base = np.mean([s[1] for s in base[4:]])
    r0_learn = np.mean([s[1] for s in learned[4:]])
    print('iterations previous-step {:.1f} learned {:.1f}; relres0 {:.2e} -> {:.2e}'.format(
        it_base, it_learn, r0_base, r0_learn))
    # what the trained network gains: a smaller initial FP64 residual than the previous-step guess
    assert r0_learn < 0.5 * r0_base


class _Info:
    def __init__(self, it, r0):
        self.iterations, self.relres0 = it, r0


def test_guess_judge_falls_back_without_gain():
    """Host-side judge logic (no GPU): the network is switched off when it stops paying."""
    from opencmp_gb300.guess import LearnedGuess
    g = LearnedGuess.__new__(LearnedGuess)
    g.judge_window = 3
    g.reset_judge()
    for _ in range(3):
        g.judge(_Info(18, 8e-3), used=False)
    g.judge(_Info(12, 1e-3), used=True)
    g.judge(_Info(13, 1e-3), used=True)
    g.judge(_Info(12, 1e-3), used=True)
    assert g.enabled
    g.judge(_Info(25, 1e-3), used=True)
    g.judge(_Info(25, 1e-3), used=True)
    g.judge(_Info(25, 1e-3), used=True)
    assert not g.enabled and 'iterations' in g.fallback_reason
    g.reset_judge()
    g.judge(_Info(18, 8e-3), used=False)
    g.judge(_Info(10, 2e-2), used=True)
    assert not g.enabled and 'initial residual' in g.fallback_reason
