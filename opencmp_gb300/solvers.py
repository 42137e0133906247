"""OpenCMP solvers on the GPU path (``opencmp/solvers``).

:class:`StationarySolver` follows ``opencmp/solvers/stationary.py:37-77``: the forms with dt = 1 and
no time-derivative term, one assembly, one linear solve.

:class:`TransientMultiStepSolver` runs the one-step schemes of
``opencmp/solvers/time_integration_schemes.py`` as a theta method (explicit Euler theta = 0,
lines 25-76; Crank-Nicolson theta = 1/2, lines 134-191; implicit Euler theta = 1, lines 79-132):

    (M + theta dt K_ode + dt K_skel) u^{n+1} = M u^n - (1 - theta) dt K_ode u^n
                                              + theta L(t^{n+1}) + (1 - theta) L(t^n)

where K_skel are the interior-facet DG terms (the time-coefficient form, always implicit) and K_ode
the rest of the operator. Every step advances t, applies the Dirichlet data at the new time,
reassembles both forms (``base_solver.py:521-607``), refreshes the preconditioner and solves from
the previous step's solution. ``get_solver_class`` follows ``opencmp/solvers/misc.py:27-63``.

For MultiComponentINS with a fixed velocity OpenCMP's stationary driver takes the nonlinear
(Anderson) branch; here the stationary solve is the single linear solve that model reduces to.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib as LB
from . import fem
from . import saving
from .config import ConfigParser
from .fem import _ptr, _stream

THETA = {'explicit euler': 0.0, 'crank nicolson': 0.5, 'implicit euler': 1.0}
# schemes whose implicit part the model builds itself, with the explicit (IMEX) part; the value is
# the number of previous solutions the scheme reads (base_solver.py:44-55)
IMEX = {'euler IMEX': 1, 'CNLF': 2, 'SBDF': 3}


class Solver:
    def __init__(self, model_class, config: ConfigParser):
        self.config = config
        # restart (base_solver.py:150-213): the checkpoint's time starts time_range, its solution
        # replaces the initial condition
        transient = config.get_item(['TRANSIENT', 'transient'], bool)
        order = IMEX.get(config.get_item(['TRANSIENT', 'scheme'], str), 1) if transient else 1
        self.restart_file = saving.resolve_restart(config, model_class.name(), order)
        self.model = model_class(config)
        self.model.setup()
        if self.restart_file is not None:
            self.model.load_state(saving.read_sol(str(self.restart_file)))
        self.saver = saving.SolutionFileSaver(self.model, config) \
            if config.get_item(['VISUALIZATION', 'save_to_file'], bool) else None
        self.num_iters = 0
        self.transient = config.get_item(['TRANSIENT', 'transient'], bool)
        self.check_error = config.get_item(['ERROR ANALYSIS', 'check_error'], bool)
        self.t = 0.0
        self.infos = []
        # new [SOLVER] key: the Krylov start of each transient step, 'previous' (OpenCMP's: the last
        # solution), 'extrapolated' (cubic extrapolation in time of the last solutions, the
        # fallback of the learned guess) or 'learned' (that extrapolation plus the correction of a
        # network trained on the run's own first `learned_train_steps` steps once the history is
        # full, kept only while its convergence judge sees it save Krylov iterations); the last two
        # for fixed-step schemes, restarted when dt changes
        self.guess_mode = config.get_item(['SOLVER', 'initial_guess'], str).strip().lower()
        if self.guess_mode not in ('previous', 'extrapolated', 'learned'):
            raise NotImplementedError('initial_guess {!r} is not on the GPU path (previous, extrapolated or '
                                      'learned)'.format(self.guess_mode))
        self.learn_steps = config.get_item(['SOLVER', 'learned_train_steps'], int)
        self.learn_iters = config.get_item(['SOLVER', 'learned_train_iters'], int)

    def _solve_var(self, v, theta: float, dt: float, t_new: float, t_old: float, transient: bool,
                   u_from=None, u_to=None, warm: bool = False):
        """One theta step of variable v from u_from (default v.u) into u_to (default v.u); the
        solve starts from u_from, or with `warm` from what u_to holds (the previous sweep's value)."""
        m = self.model
        u_to = v.u if u_to is None else u_to
        uprev = (v.u if u_from is None else u_from).clone() if transient else None
        if uprev is not None and not warm and u_to.data_ptr() != uprev.data_ptr():
            u_to.copy_(uprev)
        g = self._guess(v, dt, uprev) if transient else None
        used = None
        if g is not None:
            if self.guess_mode == 'learned':
                used = g.predict(u_to)
            else:
                g.extrapolate(u_to)
        v.set_dirichlet(t_new, u_to)
        mass = 1.0 if transient else 0.0
        # _assemble (base_solver.py:368-377): the bilinear and linear forms of this step, then the
        # preconditioner update
        m.t_form = t_new                    # time of the step's time-dependent form data (Robin r)
        form = m.form(v, mass, theta * dt, dt)
        r, keep = m.rhs(v, t_new, theta * dt, mass=mass, uprev=uprev)
        v.a.form = form
        v.L._assemble = lambda vec: fem.assemble_rhs(v.space, form, r, vec)
        v.a.Assemble()
        v.L.Assemble()
        v.pre.Update()
        if transient and theta < 1.0:
            # (1 - theta) [L(t^n) - dt K_ode u^n]
            r0, keep0 = m.rhs(v, t_old, (1.0 - theta) * dt, accumulate=True)
            op_form = m.form(v, 0.0, 1.0, 0.0)
            fem.assemble_rhs(v.space, op_form, r0, v.b)
            if v.op is None:
                v.op = fem.Matrix(v.space)
            v.op.assemble(op_form)
            LB.call('ocmp_spmv_axpby', v.op.h, -(1.0 - theta) * dt, _ptr(uprev), 1.0, _ptr(v.b), _stream(None))
            del keep0
        if transient and getattr(m, 'linearize', None) == 'IMEX' and hasattr(m, 'imex_explicit'):
            m.imex_explicit(v, dt, t_new, uprev)
        if getattr(self, '_coupling', None) is not None:
            olds, cur = self._coupling
            m.coupling_rhs(v, theta if transient else 1.0, dt if transient else 1.0, olds, cur)
        info = v.solve(u_to)
        del keep
        if g is not None:
            if self.guess_mode == 'learned':
                self._learn(v, g, u_to, info, used)
            g.push(u_to)
        self.infos.append(info)
        return info

    def _learn(self, v, g, u_new, info, used):
        """Learned guess: collect the run's first steps as training samples (each keeps a copy of
        its step's matrix for the residual loss), train once they are in, then let the judge
        decide after every step whether the network's guess still saves iterations."""
        if not g.trained:
            if g.ready and len(g.samples) < self.learn_steps:
                A = fem.Matrix(v.space)
                A.device_values()[0].copy_(v.mat.device_values()[0])
                g.collect(u_new, A, v.b)
            if len(g.samples) >= self.learn_steps:
                g.train(steps=self.learn_iters, lr=3e-3)
                g.drop_samples()
                g.reset_judge()
            return
        g.judge(info, used)

    def _guess(self, v, dt, uprev):
        """The variable's extrapolation history (None for the previous-step guess); restarted from
        u^n when the step size changes, since the extrapolation assumes equal steps."""
        if self.guess_mode == 'previous' or not getattr(self, 'fixed_step', False):
            return None
        from .guess import LearnedGuess
        g = getattr(v, 'guess', None)
        if g is None:
            # the learned guess reads 4 backward differences (5 solutions); the plain extrapolation 3
            g = v.guess = LearnedGuess(v.space, k=5 if self.guess_mode == 'learned' else 4, base_order=3)
        if getattr(v, 'guess_dt', None) != dt or g.m == 0:
            g.reset()
            g.push(uprev)
            v.guess_dt = dt
        return g

    def _solve_all(self, theta: float, dt: float, t_new: float, t_old: float, transient: bool, src=None, dst=None):
        """One step of every variable from src into dst ({name: tensor}; None: in place). Where a
        source reads another variable (coupled reactions, which OpenCMP solves as one compound
        system), segregated sweeps over the variables repeat, each with the others' latest values
        and the step's start values, until no variable changes by more than 1e-10 relative: the
        compound system's solution. Each sweep's solves start from the previous sweep's values: a
        solve restarted from the step's start ends anywhere within its 1e-12 residual, about
        cond(A) 1e-12 in the solution, and the change between sweeps would not fall below that.

        The sweeps are a fixed-point map x -> G(x) that contracts by about
        k_ab k_ba dt^2 / ((1 - k_aa dt)(1 - k_bb dt)) per sweep for a pair of first-order reactions,
        which tends to a constant near 1 as dt grows; Anderson mixing over the last
        `anderson_depth` sweeps (x <- G(x) - dG gamma, gamma the least-squares fit of the sweep's
        change f = G(x) - x by the earlier changes' differences dF) takes the sweeps to the fixed
        point in a few steps at any dt."""
        m = self.model
        names = list(m.vars)
        src = src or {n: m.vars[n].u for n in names}
        dst = dst or {n: m.vars[n].u for n in names}
        if not m.coupled():
            for n in names:
                self._solve_var(m.vars[n], theta, dt, t_new, t_old, transient, u_from=src[n], u_to=dst[n])
            return
        if self.guess_mode != 'previous':
            raise NotImplementedError('coupled reactions run with the previous-step initial guess')
        olds = {n: src[n].clone() for n in names}
        for n in names:
            if dst[n].data_ptr() != src[n].data_ptr():
                dst[n].copy_(src[n])
        self._coupling = (olds, dst)
        sizes = [dst[n].numel() for n in names]
        dF, dG = [], []
        f_prev = g_prev = None
        try:
            for sweep in range(self.max_sweeps):
                before = {n: dst[n].clone() for n in names}
                for n in names:
                    self._solve_var(m.vars[n], theta, dt, t_new, t_old, transient, u_from=olds[n], u_to=dst[n],
                                    warm=True)
                change = max(float(torch.linalg.vector_norm(dst[n] - before[n]) /
                                   max(float(torch.linalg.vector_norm(dst[n])), 1e-300)) for n in names)
                if sweep > 0 and change <= 1e-10:
                    return
                g = torch.cat([dst[n] for n in names])
                f = g - torch.cat([before[n] for n in names])
                if f_prev is not None:
                    dF.append(f - f_prev)
                    dG.append(g - g_prev)
                    if len(dF) > self.anderson_depth:
                        dF.pop(0)
                        dG.pop(0)
                f_prev, g_prev = f, g
                if dF:
                    Fm = torch.stack(dF, 1)
                    scale = torch.linalg.vector_norm(Fm, dim=0)
                    scale = torch.where(scale > 0, scale, torch.ones_like(scale))
                    Fs = Fm / scale
                    gram = (Fs.T @ Fs).cpu().numpy()
                    rhs = (Fs.T @ f).cpu().numpy()
                    gamma = np.linalg.lstsq(gram, rhs, rcond=1e-12)[0] / scale.cpu().numpy()
                    x = g - torch.stack(dG, 1) @ torch.from_numpy(gamma).to(g)
                    for n, part in zip(names, torch.split(x, sizes)):
                        dst[n].copy_(part)
        finally:
            self._coupling = None
        raise RuntimeError('coupled reactions: the segregated sweeps did not converge in {} sweeps'.format(
            self.max_sweeps))

    max_sweeps = 100
    anderson_depth = 10

    def _step(self, theta: float, dt: float, t_new: float, t_old: float, transient: bool):
        if hasattr(self.model, 'step'):
            self.model.step(theta, dt, t_new, t_old, transient, self.infos)
            return
        self._solve_all(theta, dt, t_new, t_old, transient)

    def solve(self):
        raise NotImplementedError

    def report(self):
        if self.check_error:
            for ln in self.model.errors(self.t):
                print(ln)


class StationarySolver(Solver):
    def solve(self):
        self._step(1.0, 1.0, 0.0, 0.0, False)
        return self.model.vars


class TransientMultiStepSolver(Solver):
    fixed_step = True

    def __init__(self, model_class, config):
        super().__init__(model_class, config)
        self.scheme = config.get_item(['TRANSIENT', 'scheme'], str)
        if self.scheme in IMEX and getattr(self.model, 'linearize', None) != 'IMEX':
            raise NotImplementedError('{!r} needs a model with the IMEX linearisation on the GPU path'.format(
                self.scheme))
        if self.scheme not in THETA and self.scheme not in IMEX:
            raise NotImplementedError('time scheme {!r} is not on the GPU path (one of {})'.format(
                self.scheme, sorted(THETA) + sorted(IMEX)))
        self.theta = THETA.get(self.scheme, 1.0)
        self.t_range = config.get_list(['TRANSIENT', 'time_range'], float)
        self.dt = config.get_item(['TRANSIENT', 'dt'], float)
        self.t = self.t_range[0]
        self._next_dt = None
        order = IMEX.get(self.scheme, 1)
        if order > 1 and not hasattr(self.model, 'startup_step'):
            raise NotImplementedError('{!r} is on the GPU path for the INS model; other models take euler IMEX'.format(
                self.scheme))
        if order > 1:
            # start-up (transient_multistep.py:51-100): order - 1 implicit-Euler steps of dt = 1e-10;
            # the first step of the scheme itself also takes 1e-10 (its dt is reset after the step)
            for _ in range(order - 1):
                t_old = self.t
                self.t = t_old + 1e-10
                self.model.startup_step(1e-10, self.t, self.infos)
            self._next_dt = 1e-10

    def solve(self):
        """The time loop of base_solver.py:801-865: step until t reaches the end of the range
        (np.isclose), the step shortened to land on the end time (base_solver.py:379-420), printing
        the error metrics after every step when check_error is set, and writing the solution files
        the save frequency asks for (base_solver.py:562-586; the initial condition first)."""
        t1 = self.t_range[1]
        if self.saver is not None:
            self.saver.save(self.t)
        while self.t < t1 and not np.isclose(self.t, t1):
            t_old = self.t
            dt = min(self.dt if self._next_dt is None else self._next_dt, t1 - t_old)
            self._next_dt = None
            self.t = t_old + dt
            self._step(self.theta, dt, self.t, t_old, True)
            self.num_iters += 1
            if self.saver is not None:
                self.saver.after_step(self.num_iters, self.t, self.t_range[0], dt)
            if self.check_error:
                self.report()
        return self.model.vars


class AdaptiveSolver(TransientMultiStepSolver):
    """Adaptive time stepping of opencmp/solvers/adaptive_transient_solvers: each attempt solves the
    step twice, estimates the local error from the L2 difference of the two solutions and accepts
    or repeats the step (base_adaptive_transient_multistep.py:41-143):

      factor = clamp(sqrt((abs + rel |u|) / err), 0.3, 2), dt_new = min(0.9 dt factor, dt_max, t_end - t)

    over the components; the step is accepted when every err <= abs + rel |u|.
      two step   (adaptive_two_step.py): Crank-Nicolson predictor, implicit-Euler corrector (kept);
      three step (adaptive_three_step.py): one implicit-Euler step of dt against two of dt/2 (kept);
                 a rejected attempt repeats with dt/2 (base_adaptive_transient_RK.py)."""

    fixed_step = False  # attempts of different dt: the step history does not extrapolate

    def __init__(self, model_class, config):
        Solver.__init__(self, model_class, config)
        if hasattr(self.model, 'step') and not hasattr(self.model, 'adaptive_state'):
            raise NotImplementedError('adaptive time stepping is not on the GPU path for this model')
        self.scheme = config.get_item(['TRANSIENT', 'scheme'], str)
        self.t_range = config.get_list(['TRANSIENT', 'time_range'], float)
        self.dt = config.get_item(['TRANSIENT', 'dt'], float)
        self.t = self.t_range[0]
        tol = config.get_dict(['TRANSIENT', 'dt_tolerance'])
        self.abs_tol, self.rel_tol = float(tol.get('absolute', 0.0)), float(tol['relative'])
        self.dt_range = sorted(config.get_list(['TRANSIENT', 'dt_range'], float))
        self.max_rejects = config.get_item(['TRANSIENT', 'maximum_rejected_solves'], int)
        self._scratch = {}

    def _buf(self, v, k):
        key = (v.name, k)
        if key not in self._scratch:
            self._scratch[key] = torch.zeros_like(v.u)
        return self._scratch[key]

    def _attempt(self, dt, t_old):
        """Both solutions of every variable for one attempt; returns {name: (kept, other)}."""
        t_new = t_old + dt
        vs = self.model.vars
        cur = {n: v.u for n, v in vs.items()}
        buf = {k: {n: self._buf(v, k) for n, v in vs.items()} for k in 'abc'}
        if self.scheme == 'adaptive two step':
            self._solve_all(0.5, dt, t_new, t_old, True, src=cur, dst=buf['a'])
            self._solve_all(1.0, dt, t_new, t_old, True, src=cur, dst=buf['b'])
            return {n: (buf['b'][n], buf['a'][n]) for n in vs}
        self._solve_all(1.0, dt, t_new, t_old, True, src=cur, dst=buf['a'])
        self._solve_all(1.0, dt / 2, t_old + dt / 2, t_old, True, src=cur, dst=buf['b'])
        self._solve_all(1.0, dt / 2, t_new, t_old + dt / 2, True, src=buf['b'], dst=buf['c'])
        return {n: (buf['c'][n], buf['a'][n]) for n in vs}

    def _attempt_model(self, dt, t_old):
        """Both solutions of an attempt for a model that steps itself (INS): the kept one stays in the
        model; returns (state before the attempt, kept, other)."""
        m = self.model
        t_new = t_old + dt
        st0 = m.adaptive_state()
        if self.scheme == 'adaptive two step':
            m.step(0.5, dt, t_new, t_old, True, self.infos)
            other = m.u.clone()
            m.adaptive_restore(st0)
            m.step(1.0, dt, t_new, t_old, True, self.infos)
        else:
            m.step(1.0, dt, t_new, t_old, True, self.infos)
            other = m.u.clone()
            m.adaptive_restore(st0)
            m.step(1.0, dt / 2, t_old + dt / 2, t_old, True, self.infos)
            m.step(1.0, dt / 2, t_new, t_old + dt / 2, True, self.infos)
        return st0, m.u.clone(), other

    def solve(self):
        t1 = self.t_range[1]
        rejects = 0
        if self.saver is not None:
            self.saver.save(self.t)
        whole = hasattr(self.model, 'step')
        while self.t < t1 and not np.isclose(self.t, t1):
            dt = min(self.dt, t1 - self.t)
            errs, norms = [], []
            if whole:
                st0, kept, other = self._attempt_model(dt, self.t)
                for e, nrm in self.model.local_errors(kept, other):
                    errs.append(e)
                    norms.append(nrm)
                sols = {}
            else:
                sols = self._attempt(dt, self.t)
            for name, (kept, other) in sols.items():
                v = self.model.vars[name]
                errs.append(v.space.l2_error(kept - other) or 1e-10)
                norms.append(v.space.l2_error(kept) or 1e-10)
            dt_err = min(dt * 0.9 * min(2.0, max(0.3, math.sqrt((self.abs_tol + self.rel_tol * nrm) / e)))
                         for e, nrm in zip(errs, norms))
            if dt_err < self.dt_range[0]:
                raise RuntimeError('At t = {} further time steps must be smaller than the minimum time step ({}).'
                                   .format(self.t, dt_err))
            accept = all(e <= self.abs_tol + self.rel_tol * nrm for e, nrm in zip(errs, norms))
            if accept:
                for name, (kept, _) in sols.items():
                    self.model.vars[name].u.copy_(kept)
                self.t += dt
                self.num_iters += 1
                if self.saver is not None:
                    self.saver.after_step(self.num_iters, self.t, self.t_range[0], dt)
                rest = t1 - self.t
                self.dt = min(dt_err, self.dt_range[1], rest if rest > 0 else dt_err)
                rejects = 0
                if self.check_error:
                    self.report()
            else:
                if whole:
                    self.model.adaptive_restore(st0)
                rejects += 1
                if rejects > self.max_rejects:
                    raise RuntimeError('At t = {} the maximum number of rejected time steps has been exceeded.'
                                       .format(self.t))
                self.dt = dt / 2 if self.scheme == 'adaptive three step' else min(dt_err, self.dt_range[1])
        return self.model.vars


def get_solver_class(config: ConfigParser):
    """Solver class for the configured time scheme (opencmp/solvers/misc.py:27-63)."""
    transient = config.get_item(['TRANSIENT', 'transient'], bool)
    scheme = config.get_item(['TRANSIENT', 'scheme'], str)
    if not transient:
        return StationarySolver
    if scheme in THETA or scheme in IMEX:
        return TransientMultiStepSolver
    if scheme in ('adaptive two step', 'adaptive three step'):
        return AdaptiveSolver
    if 'adaptive' in scheme or scheme in ('RK 222', 'RK 232'):
        raise NotImplementedError('time scheme {!r} is not on the GPU path'.format(scheme))
    raise TypeError('Have not implemented {} time integration yet.'.format(scheme))
