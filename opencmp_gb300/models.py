"""OpenCMP models on the GPU path.

Mirrors ``opencmp/models`` for the models of the hot path: :class:`Poisson`
(``opencmp/models/poisson.py:71-158``) and :class:`MultiComponentINS` with ``velocity_fixed = True``
(``opencmp/models/multi_component_ins.py:158-388``: diffusion, conservative advection, upwind
facets, outflow on total-flux and unlabelled boundaries, the Neumann (w.n) half, DG Dirichlet
terms). The registry and lookup follow ``opencmp/models/__init__.py:30-36`` and
``opencmp/models/misc.py:27-50``.

Each model variable (Poisson's u; each MCINS component) is a scalar GPU space with its matrices and
Krylov solver. OpenCMP assembles the MCINS components in one compound space; with the velocity fixed
and no reactions the compound system is block diagonal, so solving the components one after another
gives the same solution.

OpenCMP splits each model's operator into a *time-coefficient* part (the interior-facet DG terms,
always implicit) and an *ODE* part (everything else), which the time schemes weight
(``time_integration_schemes.py``). The forms built here keep that split: ``dt`` scales the ODE terms
and ``skeleton_dt`` the interior-facet terms.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _lib as LB
from . import fem
from . import forms
from .config import ConfigParser, Expr, load_sub_config, parse, set_import_dir, value_map
from .mesh import load_mesh
from .saddle import SaddleSolver


class _RobinData:
    """-r q of a Robin marker's [r, q] (the linear form's data, poisson.py:153-157)."""

    def __init__(self, v):
        self.v = v
        self.depends_on_space = isinstance(v, Expr) and v.depends_on_space

    def __call__(self, X, t):
        if isinstance(self.v, Expr):
            pts = None if X is None else np.asarray(X).reshape(-1, np.asarray(X).shape[-1])
            rq = np.asarray(self.v(pts, t), float).reshape(-1, 2)
        else:
            rq = np.asarray(self.v, float).reshape(-1, 2)
        out = -rq[:, 0] * rq[:, 1]
        return float(out[0]) if X is None else out.reshape(np.asarray(X).shape[:-1])


def _scalar_at(v, t) -> Optional[float]:
    """The value as a float when it does not depend on x, y, z (None otherwise)."""
    if isinstance(v, _RobinData):
        return None if v.depends_on_space else v(None, t)
    if isinstance(v, Expr):
        if v.depends_on_space:
            return None
        return float(v(None, t))
    if v is None:
        return None
    return float(v)


def _at(v, X, t):
    """A parsed config value at the points X (..., dim) and time t."""
    if isinstance(v, (Expr, _RobinData)):
        return v(X, t)
    return np.full(X.shape[:-1], float(v))


def affine_parts(v, names: List[str], X, t: float):
    """A source that reads model variables, split as f = f0 + sum_j k_j c_j: f0 at the points X
    (c = 0) and the coefficients k_j, which must not vary in space; anything but an affine
    dependence on the variables is refused. OpenCMP puts the part that reads the unknowns into the
    bilinear form (multi_component_ins.py:243-257)."""
    used = [n for n in names if isinstance(v, Expr) and n in v.mvars]
    other = set(v.mvars) - set(names) if isinstance(v, Expr) else set()
    if other:
        raise NotImplementedError('expression {!r} reads {} (not model variables of the GPU path)'.format(
            v.text, sorted(other)))
    zero = {n: 0.0 for n in names}
    f0 = np.asarray(v(X, t, zero), float)
    ks = {}
    for n in used:
        one = dict(zero)
        one[n] = 1.0
        k = np.asarray(v(X, t, one), float) - f0
        two = dict(zero)
        two[n] = 2.0
        k2 = np.asarray(v(X, t, two), float) - f0
        if np.abs(k2 - 2 * k).max() > 1e-12 * max(1.0, np.abs(k).max()) or np.ptp(k) > 1e-12 * max(1.0, np.abs(k).max()):
            raise NotImplementedError('source {!r}: only constant-coefficient linear terms in the model variables '
                                      'are on the GPU path'.format(v.text))
        ks[n] = float(k.reshape(-1)[0])
    for i, a in enumerate(used):
        for b in used[i + 1:]:
            both = dict(zero)
            both[a] = both[b] = 1.0
            if np.abs(np.asarray(v(X, t, both), float) - f0 - ks[a] - ks[b]).max() > 1e-12 * max(1.0, abs(ks[a]) + abs(ks[b])):
                raise NotImplementedError('source {!r}: products of model variables are not on the GPU path'.format(v.text))
    return f0, ks


def _accepted(info, accept: float) -> bool:
    return info.status == LB.OK or (info.status == LB.NOT_CONVERGED and np.isfinite(info.relres) and (
        info.relres <= accept or (np.isfinite(info.relres0) and info.relres <= 1e-12 * info.relres0)))


def checked_solve(solver, b, x, accept: float):
    """Solve; a stop at the iteration cap is accepted when the FP64 relative residual reached
    `accept` (the round-off floor of an ill-conditioned system), or fell by 1e-12 from the initial
    residual (NGSolve's Krylov criterion; it decides where the right-hand side cancels to round-off,
    as when the solution reaches zero), otherwise it raises.

    A solve that fails from an initial guess whose residual is larger than the right-hand side
    (relres0 > 1: the right-hand side cancelled far below the guess's residual, as when the solution
    reaches zero in one step) is repeated once from zero on the free dofs: the round-off of cancelling
    the guess, eps |A| |x0|, is what kept the first attempt from the tolerance."""
    info = solver.solve(b, x, raise_on_fail=False)
    if _accepted(info, accept):
        return info
    space = getattr(getattr(solver, 'mat', None), 'space', None)
    if (info.status == LB.NOT_CONVERGED and np.isfinite(info.relres0) and info.relres0 > 1.0
            and hasattr(space, 'FreeDofs')):
        free = space.FreeDofs()
        if free.shape[0] == x.numel():
            x[torch.from_numpy(free).to(x.device)] = 0.0
            info = solver.solve(b, x, raise_on_fail=False)
            if _accepted(info, accept):
                return info
    LB.check(info.status)
    return info


class Variable:
    """One scalar unknown: its GPU space, system and operator matrices, solver and solution."""

    def __init__(self, model: 'Model', name: str, element: str):
        self.model = model
        self.name = name
        self.kind = 'L2' if (model.DG or element == 'L2') else 'H1'
        bc = model.bc
        self.dirichlet = bc.get('dirichlet', {}).get(name, {})
        self.neumann = bc.get('neumann', {}).get(name, {})
        self.total_flux = bc.get('total_flux', {}).get(name, {})
        self.robin = bc.get('robin', {}).get(name, {})
        if self.robin and not isinstance(model, Poisson):
            raise NotImplementedError('Robin boundary conditions are on the GPU path for the Poisson model')
        if bc.get('surface_rxn', {}).get(name):
            raise NotImplementedError('surface-reaction boundary conditions are not on the GPU path')
        names = set(model.mesh.bc_names)
        for d in (self.dirichlet, self.neumann, self.total_flux, self.robin):
            for marker in d:
                if marker not in names:
                    raise ValueError('boundary {!r} is not a label of the mesh ({})'.format(marker, sorted(names)))
        dnames = list(self.dirichlet) if self.kind == 'H1' else []
        self.space = fem.Space(model.mesh, self.kind, model.interp_ord, dnames, gmesh=model.gmesh)
        P = dict(model.solver_params)
        direct_dg = False
        if P['method'] == 'auto':
            # a direct solve in OpenCMP: CG where the operator is symmetric positive definite, else
            # GMRES; for DG spaces GMRES preconditioned by the strip direct factorisation (the
            # counterpart of the sparse LU OpenCMP refactorises each step) where the pattern allows
            P['method'] = 'CG' if model.symmetric(self) else 'GMRES'
            direct_dg = P['method'] == 'GMRES' and self.kind == 'L2'
        if P['method'] == 'CG' and P['precision'] == 'mixed':
            P['precision'] = 'fp64'
        if P['method'] == 'CG' and P['precond'] == 'block_jacobi':
            P['precond'] = 'jacobi'            # CG is built with a diagonal preconditioner
        self.params = P
        self.mat = fem.Matrix(self.space, jacobi64=P['precision'] == 'fp64' and P['precond'] == 'jacobi',
                              jacobi32=P['precision'] == 'mixed' and P['precond'] == 'jacobi')
        # A direct solve in OpenCMP is accurate to the conditioning of the system; here a Krylov
        # solve that stops short of 1e-12 at the FP64 round-off floor is accepted below 1e-9.
        self.accept = 1e-9 if model.solver_params['tol'] <= 1e-12 else P['tol']
        self.op = None                      # ODE-part operator, for explicit terms
        n = self.space.ndof
        self.u = torch.zeros(n, dtype=torch.float64, device='cuda')
        self.b = torch.zeros(n, dtype=torch.float64, device='cuda')
        # the NGSolve-side objects OpenCMP's Model/Solver methods pass around (forms.py)
        self.gfu = forms.GridFunction(self.space, self.u)
        self.a = forms.BilinearForm(self.space, self.mat)
        self.a.var = self
        self.L = forms.LinearForm(self.space, self.b)
        if direct_dg:
            P['precond'] = 'strip'
            try:
                self.pre = model.construct_preconditioners([self.a])[0]
            except LB.OcmpError as e:
                if e.status not in (LB.ERR_UNSUPPORTED, LB.ERR_NOMEM):
                    raise
                P['precond'] = model.solver_params['precond']
                self.pre = model.construct_preconditioners([self.a])[0]
        else:
            self.pre = model.construct_preconditioners([self.a])[0]
        self.solver = self.pre.solver
        self._qp = None
        self._fq = None
        self._flab = None
        self._bpts: Dict[int, np.ndarray] = {}

    # ---------------------------------------------------------------- geometry caches
    def quad_points(self):
        if self._qp is None:
            self._qp = self.space.quad_points()
        return self._qp

    def _facets(self):
        if self._fq is None:
            self._fq = self.space.facet_quad_points()
            self._flab = self.space.boundary_facets()[:, 2]
        return self._fq, self._flab

    def lab(self, marker: str) -> int:
        return self.model.mesh.bc_names.index(marker)

    def mask(self, markers) -> int:
        return self.model.mesh.label_mask(list(markers))

    # ---------------------------------------------------------------- boundary data
    def facet_data(self, d: Dict[str, object], t: float, scale: float = 1.0):
        """Per-label constants {label: scale*value}, or, when some value depends on x, y, z, the
        values at every boundary-facet quadrature point as a device tensor (labels outside `d` 0)."""
        consts, spatial = {}, False
        for marker, v in d.items():
            c = _scalar_at(v, t)
            if c is None:
                spatial = True
            else:
                consts[self.lab(marker)] = scale * c
        if not spatial:
            return consts, None
        X, labs = self._facets()
        vals = np.zeros(X.shape[:2])
        for marker, v in d.items():
            sel = labs == self.lab(marker)
            if sel.any():
                vals[sel] = scale * _at(v, X[sel], t)
        return consts, torch.as_tensor(vals, device='cuda')

    def set_dirichlet(self, t: float, u: Optional[torch.Tensor] = None):
        """gfu.Set(g_D, definedon=Dirichlet boundaries) (base_model.py:321-341) on u (default: the
        variable's solution)."""
        if self.kind != 'H1' or not self.dirichlet:
            return
        u = self.u if u is None else u
        consts = {}
        for marker, v in self.dirichlet.items():
            c = _scalar_at(v, t)
            if c is not None:
                consts[self.lab(marker)] = c
        if consts:
            self.space.set_boundary(consts, u)
        for marker, v in self.dirichlet.items():
            if _scalar_at(v, t) is None:
                lab = self.lab(marker)
                if lab not in self._bpts:
                    self._bpts[lab] = self.space.boundary_points(1 << lab)
                self.space.set_boundary_values(1 << lab, _at(v, self._bpts[lab], t), u)

    def project(self, value, t: float = 0.0):
        """Initial condition: the L2 projection of `value` onto the space (exact for constants)."""
        if value is None:
            self.u.zero_()
            return
        c = _scalar_at(value, t)
        if c is not None and self.kind == 'H1':
            h = np.zeros(self.space.ndof)
            h[:self.model.mesh.nv] = c
            self.u.copy_(torch.as_tensor(h))
            return
        sp = fem.Space(self.model.mesh, self.kind, self.model.interp_ord, (), gmesh=self.model.gmesh)
        M = fem.Matrix(sp)
        f = fem.make_form(mass=1.0)
        M.assemble(f)
        if c is not None:
            rhs = fem.make_rhs(src_const=c)
            fq = None
        else:
            fq = torch.as_tensor(_at(value, sp.quad_points(), t).reshape(self.model.mesh.ne, -1), device='cuda')
            rhs = fem.make_rhs(src_qp=fq)
        b = torch.zeros(sp.ndof, dtype=torch.float64, device='cuda')
        fem.assemble_rhs(sp, f, rhs, b)
        x = torch.zeros_like(b)
        fem.KrylovSolver(M, method='CG', tol=1e-13, maxit=20000).solve(b, x)
        self.u.copy_(x)

    def solve(self, x: Optional[torch.Tensor] = None):
        """Model.solve_single_step for this variable's system, into x (default: the solution)."""
        gfu = self.gfu if x is None or x.data_ptr() == self.u.data_ptr() else forms.GridFunction(self.space, x)
        return self.model.solve_single_step([self.a], [self.L], [self.pre], gfu)

    def source(self, t: float):
        """(constant, quadrature-point tensor) of the source; one of them is None."""
        fs = self.model.functions.get('source', {})
        f = fs.get(self.name, fs.get('all'))
        if f is None:
            return None, None
        if isinstance(f, Expr) and f.mvars:
            # the part that does not read the model variables (the rest is the reaction terms of
            # Model.reaction)
            names = list(self.model.vars) or list(self.model.components)
            X = self.quad_points()
            f0, _ = affine_parts(f, names, X, t)
            if np.ptp(f0) == 0.0:
                c0 = float(f0.reshape(-1)[0])
                return (c0 if c0 != 0.0 else None), None
            return None, torch.as_tensor(np.ascontiguousarray(f0.reshape(self.model.mesh.ne, -1)), device='cuda')
        c = _scalar_at(f, t)
        if c is not None:
            return (c if c != 0.0 else None), None
        X = self.quad_points()
        return None, torch.as_tensor(_at(f, X, t).reshape(self.model.mesh.ne, -1), device='cuda')


class Model:
    """Configuration, mesh, boundary/initial/model data (base_model.py:44-257)."""

    components: List[str] = []

    def __init__(self, config: ConfigParser):
        self.config = config
        self.run_dir = config.get_item(['OTHER', 'run_dir'], str)
        # the h-convergence test (post_processing.py) solves again on refined copies of the mesh
        refined = getattr(config, 'refined_mesh', None)
        self.mesh = refined if refined is not None else load_mesh(config.get_item(['MESH', 'filename'], str))
        self.gmesh = fem.GPUMesh(self.mesh)
        self.DG = config.get_item(['DG', 'DG'], bool)
        self.ipc = config.get_item(['DG', 'interior_penalty_coefficient'], float)
        self.interp_ord = config.get_item(['FINITE ELEMENT SPACE', 'interpolant_order'], int)
        self.elements = config.get_dict(['FINITE ELEMENT SPACE', 'elements'], all_str=True)
        set_import_dir(self.run_dir)        # IMPORT(...) in the sub-configurations reads this run's functions
        bc = load_sub_config(self.run_dir, 'bc')
        self.bc = {k.lower(): value_map(bc, k) for k in (bc.sections() if bc else [])}
        ic = load_sub_config(self.run_dir, 'ic')
        self.ic = value_map(ic, ic.sections()[0]) if ic and ic.sections() else {}
        mc = load_sub_config(self.run_dir, 'model')
        self.params = value_map(mc, 'PARAMETERS')
        self.functions = value_map(mc, 'FUNCTIONS')
        rs = load_sub_config(self.run_dir, 'ref_sol')
        self.ref_sol: Dict[str, object] = {}
        self.metrics: Dict[str, List[str]] = {}
        if rs is not None:
            if rs.has_section('REFERENCE SOLUTIONS'):
                self.ref_sol = {k: parse(v) for k, v in rs.items('REFERENCE SOLUTIONS')}
            if rs.has_section('METRICS'):
                self.metrics = {k: [s.strip() for s in v.split(',') if s.strip()] for k, v in rs.items('METRICS')}
        self.solver_params = self._solver_params()
        self.vars: Dict[str, Variable] = {}

    def _solver_params(self) -> dict:
        c = self.config
        ls = c.get_item(['SOLVER', 'linear_solver'], str)
        pre = c.get_item(['SOLVER', 'preconditioner'], str)
        tol = c.get_item(['SOLVER', 'linear_tolerance'], float)
        maxit = c.get_item(['SOLVER', 'linear_max_iterations'], int)
        # 'default' / 'direct' (a sparse LU in OpenCMP, base_model.py:918) run as FP64 Krylov to a 1e-12
        # relative residual: CG for symmetric operators, GMRES otherwise (chosen per variable)
        if ls in ('default', 'direct'):
            method, tol, maxit = 'auto', 1e-12, max(maxit, 20000)
        elif ls == 'CG':
            method = 'CG'
        elif ls in ('GMRes', 'GMRES', 'MinRes', 'Richardson'):
            method = 'GMRES'
        else:
            raise ValueError('No linear solver specified.')
        precond = {'default': 'jacobi', 'local': 'jacobi', 'None': 'none', 'block_jacobi': 'block_jacobi',
                   'direct': 'strip'}.get(pre)
        if precond is None:
            raise NotImplementedError('preconditioner {!r} is not on the GPU path'.format(pre))
        if self.DG and pre == 'default':
            precond = 'block_jacobi'
        prec = c.get_item(['SOLVER', 'gpu_precision'], str)
        return dict(method=method, precond=precond, tol=max(tol, 1e-12), maxit=max(maxit, 1000),
                    precision='mixed' if prec == 'mixed' else 'fp64',
                    restart=c.get_item(['SOLVER', 'gpu_restart'], int), inner_tol=1e-4)

    @classmethod
    def name(cls) -> str:
        """The model's name in file names: the class name in lower case, a trailing 'dim' removed
        (base_model.py:648-662)."""
        n = cls.__name__.lower()
        return n[:-3] if n.endswith('dim') else n

    # ---------------------------------------------------------------- state for solution files
    def state(self) -> Dict[str, np.ndarray]:
        """The solution, variable by variable (the content of a solution file)."""
        return {name: v.u.cpu().numpy() for name, v in self.vars.items()}

    def load_state(self, st: Dict[str, np.ndarray]):
        """Restore a state written by state() as the initial condition (base_model.py:218-221)."""
        for name, v in self.vars.items():
            if name not in st or st[name].size != v.u.numel():
                raise ValueError('the checkpoint holds no {}-dof solution of {!r}'.format(v.u.numel(), name))
            v.u.copy_(torch.as_tensor(st[name]))

    # ---------------------------------------------------------------- OpenCMP's solve hooks
    def construct_preconditioners(self, a_assembled: List[forms.BilinearForm]) -> List[forms.Preconditioner]:
        """One preconditioner per assembled bilinear form (base_model.py:365-383): the [SOLVER]
        preconditioner ('local' = point Jacobi, 'direct' = the strip direct factorisation, ...) in
        the Krylov method, precision and tolerances the form's variable solves with."""
        out = []
        for a in a_assembled:
            P = a.var.params
            out.append(forms.Preconditioner(a, P['precond'], method=P['method'], precision=P['precision'],
                                            tol=P['tol'], maxit=P['maxit'], restart=P['restart'],
                                            inner_tol=P['inner_tol']))
        return out

    def solve_single_step(self, a_lst: List[forms.BilinearForm], L_lst: List[forms.LinearForm],
                          precond_lst: List[forms.Preconditioner], gfu: forms.GridFunction, time_step: int = 0):
        """One linear solve of the step's system (base_model.py:868-884): linear_solve with the
        forms of this time step."""
        return self.linear_solve(a_lst[time_step], L_lst[time_step], precond_lst[time_step], gfu)

    def linear_solve(self, a_assembled: forms.BilinearForm, L_assembled: forms.LinearForm,
                     precond: forms.Preconditioner, gfu: forms.GridFunction):
        """Solve A x = L on the free dofs (base_model.py:886-947): gfu.vec holds the Dirichlet values
        and the initial guess and receives the solution. Returns the solve's info (OpenCMP returns
        nothing; the info carries iterations and the FP64 relative residual)."""
        accept = getattr(getattr(a_assembled, 'var', None), 'accept', precond.solver.params.tol)
        return checked_solve(precond.solver, L_assembled.vec, gfu.vec, accept)

    def symmetric(self, var: Variable) -> bool:
        """Whether the variable's operator is symmetric (no convection)."""
        return True

    # ---------------------------------------------------------------- per-model terms
    def operator(self, var: Variable) -> dict:
        """make_form keywords of the variable's operator (no mass, no dt)."""
        raise NotImplementedError

    def boundary_rhs(self, var: Variable, t: float):
        """((Neumann-type {label: value}, facet tensor or None), (DG Dirichlet {label: g}, tensor or None))."""
        raise NotImplementedError

    def boundary_mask(self, var: Variable) -> int:
        """Labels that carry Neumann-type data in the linear form."""
        raise NotImplementedError

    # ---------------------------------------------------------------- forms
    def reaction(self, var: Variable, t: float) -> Dict[str, float]:
        """{variable: k} of the variable's source terms that read the model's variables (f = f0 +
        sum_j k_j c_j); empty when the source reads none."""
        fs = self.functions.get('source', {})
        f = fs.get(var.name, fs.get('all'))
        if not (isinstance(f, Expr) and f.mvars):
            return {}
        _, ks = affine_parts(f, list(self.vars), var.quad_points()[:1], t)
        return ks

    def coupled(self) -> bool:
        """Whether a source reads another variable than its own (the variables' systems couple)."""
        return any(n != v.name for v in self.vars.values() for n in self.reaction(v, 0.0))

    def coupling_rhs(self, var: Variable, theta: float, dt: float, olds, cur):
        """The cross-variable reaction terms of a segregated sweep in the linear form:
        theta dt k_j (c_j, r) at the sweep's current c_j plus (1 - theta) dt k_j (c_j^n, r)."""
        for name, k in self.reaction(var, getattr(self, 't_form', 0.0)).items():
            if name == var.name or k == 0.0:
                continue
            for coef, vec in ((theta * dt * k, cur[name]), ((1.0 - theta) * dt * k, olds[name])):
                if coef != 0.0:
                    r = fem.make_rhs(mass=coef, uprev=vec)
                    r.accumulate = 1
                    fem.assemble_rhs(var.space, fem.make_form(), r, var.b)

    def form(self, var: Variable, mass: float, dt: float, skeleton_dt: float) -> LB.Form:
        # a source term k c that reads the variable itself goes into the bilinear form as
        # -dt k (c, r), with the operator's dt (multi_component_ins.py:243-257)
        k_own = self.reaction(var, getattr(self, 't_form', 0.0)).get(var.name, 0.0)
        f = fem.make_form(mass=mass - dt * k_own, dt=dt, **self.operator(var))
        f.skeleton_own_dt, f.skeleton_dt = 1, skeleton_dt
        return f

    def rhs(self, var: Variable, t: float, dt: float, mass: float = 0.0, uprev=None, accumulate: bool = False):
        """The linear form and the device tensors it points to (keep them alive until assembled)."""
        c, fq = var.source(t)
        (bc, bq), (gc, gq) = self.boundary_rhs(var, t)
        r = fem.make_rhs(dt=dt, src_const=c, src_qp=fq, mass=mass, uprev=uprev, bval=bc, gval=gc, bval_fq=bq,
                         gval_fq=gq, bval_mask=self.boundary_mask(var))
        r.accumulate = int(accumulate)
        return r, (fq, bq, gq)

    def setup(self):
        for name in self.components:
            self.vars[name] = Variable(self, name, self.elements.get(name, 'H1'))
        for name, v in self.vars.items():
            v.project(self.ic.get(name, {}).get('all', 0.0), 0.0)

    def l2_error_of(self, name: str, t: float) -> float:
        """|| u_h - u_ref ||_L2 of one model variable against its reference solution at time t
        (``norm('l2_norm', ...)``, opencmp/helpers/error.py:75-128)."""
        v = self.vars[name]
        ref = self.ref_sol.get(name, 0.0)
        c = _scalar_at(ref, t)
        if c is not None:
            return v.space.l2_error(v.u, c)
        fq = torch.as_tensor(_at(ref, v.quad_points(), t).reshape(self.mesh.ne, -1), device='cuda')
        return v.space.l2_error(v.u, fq)

    def errors(self, t: float) -> List[str]:
        """``L2 norm in <var>: <value>`` lines, as opencmp/helpers/error.py:238-301 prints them."""
        lines = []
        for metric, names in self.metrics.items():
            if metric.lower() != 'l2_norm':
                raise NotImplementedError('{} is not on the GPU path'.format(metric))
            for name in names:
                lines.append('{0} in {1}: {2}'.format(metric.replace('_', ' '), name, self.l2_error_of(name, t)))
        return lines


class Poisson(Model):
    components = ['u']

    def __init__(self, config):
        super().__init__(config)
        dc = self.params.get('diffusion_coefficient', {}).get('all', 1.0)
        self.dc = _scalar_at(dc, 0.0)
        if self.dc is None:
            raise NotImplementedError('a space-dependent diffusion coefficient is not on the GPU path')

    def robin_r(self, var, t: float) -> Dict[int, float]:
        """Per Robin label, the coefficient of its facet mass term, -dc r (poisson.py:93-97); r is
        the first entry of the marker's [r, q] and may vary in time, not in space."""
        out = {}
        for marker, v in var.robin.items():
            if isinstance(v, Expr) and v.depends_on_space:
                X, labs = var._facets()
                rq = np.asarray(v(X[labs == var.lab(marker)].reshape(-1, X.shape[-1]), t), float).reshape(-1, 2)
                if rq.size and np.ptp(rq[:, 0]) > 1e-14 * max(1.0, np.abs(rq[:, 0]).max()):
                    raise NotImplementedError('a space-dependent Robin coefficient r is not on the GPU path')
                r = float(rq[0, 0]) if rq.size else 0.0
            else:
                r = float(np.asarray(v(None, t) if isinstance(v, Expr) else v, float).reshape(-1)[0])
            out[var.lab(marker)] = -self.dc * r
        return out

    def operator(self, var):
        op = dict(diff=self.dc, ipc=self.ipc, dg=self.DG, nitsche_mask=var.mask(var.dirichlet) if self.DG else 0)
        if var.robin:
            op['robin'] = self.robin_r(var, getattr(self, 't_form', 0.0))
        return op

    def boundary_rhs(self, var, t):
        # Neumann data dc h, and the Robin markers' -dc r q (poisson.py:148-157)
        data = dict(var.neumann)
        for marker, v in var.robin.items():
            data[marker] = _RobinData(v)
        neu = var.facet_data(data, t, self.dc)
        dir_ = var.facet_data(var.dirichlet, t) if self.DG else ({}, None)
        return neu, dir_

    def boundary_mask(self, var):
        return var.mask(list(var.neumann) + list(var.robin))


class MultiComponentINS(Model):
    """Fixed-velocity transport of the configured components (``velocity_fixed = True``)."""

    def __init__(self, config):
        super().__init__(config)
        if not config.get_item(['OTHER', 'velocity_fixed'], bool):
            raise NotImplementedError('MultiComponentINS runs on the GPU path with velocity_fixed = True')
        self.components = config.get_list(['OTHER', 'component_names'], str)
        self.D = {k: _scalar_at(v, 0.0) for k, v in self.params.get('diffusion_coefficients', {}).items()}
        W = self.ic.get('u', {}).get('all')
        self._wind_vtx = None
        self._wind_const = None
        if isinstance(W, Expr) and W.depends_on_space:
            self._wind_vtx = torch.as_tensor(np.ascontiguousarray(W(self.mesh.coords, 0.0)), device='cuda')
        elif W is not None:
            self._wind_const = tuple(np.ravel(W(None, 0.0) if isinstance(W, Expr) else [float(W)]))
        # Oseen (the default) keeps the convection implicit; IMEX moves it to the linear form at the
        # previous step's concentration (multi_component_ins.py:390-430, euler_IMEX in
        # time_integration_schemes.py:193-250)
        self.linearize = config.get_item(['SOLVER', 'linearization_method'], str)
        if self.linearize == 'IMEX':
            if self.DG:
                raise NotImplementedError('the IMEX linearisation of MultiComponentINS is on the GPU path for '
                                          'continuous spaces')
            if any(self.bc.get('total_flux', {}).get(c) for c in self.components):
                raise ValueError('Cannot specify total flux for IMEX schemes since convection term is fully explicit.')

    def symmetric(self, var):
        if self.linearize == 'IMEX':
            return True                       # mass and diffusion only
        if self._wind_vtx is not None:
            return False
        return self._wind_const is None or not any(self._wind_const)

    def operator(self, var):
        if var.neumann and self.D[var.name] == 0:
            raise ValueError('Trying to apply a neuman boundary condition for purely advective flow '
                             '(diffusion coefficient is 0).')
        if self.linearize == 'IMEX':
            return dict(diff=self.D[var.name], ipc=self.ipc, dg=self.DG)
        flux = set(self.mesh.bc_names) - set(var.dirichlet) - set(var.neumann)
        return dict(diff=self.D[var.name], wind=self._wind_const, wind_vtx=self._wind_vtx, ipc=self.ipc, dg=self.DG,
                    outflow_mask=var.mask(flux), wn_mask=var.mask(var.neumann),
                    nitsche_mask=var.mask(var.dirichlet) if self.DG else 0)

    def imex_explicit(self, var, dt: float, t_new: float, uprev: torch.Tensor):
        """The explicit part of the IMEX linear form, added to var.b (multi_component_ins.py:390-430):
        dt (c^n, w . grad r) = -dt K_w c^n, K_w the convection matrix, and -dt (h, r) on the Neumann
        markers (a second time: OpenCMP's explicit part repeats the linear form's Neumann half)."""
        if self._wind_const is not None or self._wind_vtx is not None:
            conv = fem.make_form(wind=self._wind_const, wind_vtx=self._wind_vtx)
            if getattr(var, 'opx', None) is None:
                var.opx = fem.Matrix(var.space)
            var.opx.assemble(conv)
            LB.call('ocmp_spmv_axpby', var.opx.h, -dt, C.c_void_p(uprev.data_ptr()), 1.0,
                    C.c_void_p(var.b.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
        if var.neumann:
            consts, fq = var.facet_data(var.neumann, t_new, -1.0)
            r = fem.make_rhs(dt=dt, bval=consts, bval_fq=fq, bval_mask=var.mask(var.neumann))
            r.accumulate = 1
            fem.assemble_rhs(var.space, fem.make_form(), r, var.b)

    def boundary_rhs(self, var, t):
        d = dict(var.neumann)
        d.update(var.total_flux)
        neu = var.facet_data(d, t, -1.0)
        dir_ = var.facet_data(var.dirichlet, t) if self.DG else ({}, None)
        return neu, dir_

    def boundary_mask(self, var):
        return var.mask(list(var.neumann) + list(var.total_flux))


def _vec_at(v, X, t):
    """A vector-valued config value ([a, b] or vec(a, b)) at the points X (..., 2) -> (..., 2)."""
    if isinstance(v, Expr):
        r = v(X.reshape(-1, X.shape[-1]), t)
        return np.asarray(r).reshape(X.shape[:-1] + (2,))
    return np.broadcast_to(np.asarray(v, float), X.shape[:-1] + (2,)).copy()


class INS(Model):
    """Incompressible Navier-Stokes (opencmp/models/ins.py) on Taylor-Hood spaces: velocity order
    ``interpolant_order``, pressure one lower, velocity Dirichlet data per label, the Oseen
    linearisation (Picard iteration on the wind, ins.py:323-355) or IMEX (explicit convection,
    ins.py:302-314). Where OpenCMP factorises the system (ins.py with its direct default), the
    transient systems here are solved by flexible GMRES with the Cahouet-Chabard preconditioner
    (``saddle.SaddleSolver``: velocity Jacobi, pressure Laplacian CG plus pressure mass diagonal),
    whose iteration counts do not grow with the mesh. ``[SOLVER] preconditioner = local`` and the
    stationary systems use GMRES with the block-diagonal preconditioner of ocmp_th_block_diag
    (velocity Jacobi, pressure Schur-complement diagonal)."""

    components = ['u', 'p']

    def __init__(self, config):
        super().__init__(config)
        if self.DG:
            raise NotImplementedError('INS runs on the GPU path with continuous Taylor-Hood elements (DG = False)')
        self.kv = _scalar_at(self.params.get('kinematic_viscosity', {}).get('all', 1.0), 0.0)
        lin = config.get_item(['SOLVER', 'linearization_method'], str)
        self.linearize = lin if lin in ('Oseen', 'IMEX') else 'Oseen'
        if self.linearize == 'Oseen':
            tol = config.get_dict(['SOLVER', 'nonlinear_tolerance'])
            self.abs_tol, self.rel_tol = float(tol.get('absolute', 0.0)), float(tol['relative'])
            self.max_picard = config.get_item(['SOLVER', 'nonlinear_max_iterations'], int)
        for kind in ('stress', 'parallel', 'neumann', 'robin'):
            if self.bc.get(kind, {}).get('u'):
                raise NotImplementedError('{} boundary conditions for INS are not on the GPU path'.format(kind))
        self.dirichlet = self.bc.get('dirichlet', {}).get('u', {})
        self.scheme = config.get_item(['TRANSIENT', 'scheme'], str) if config.get_item(['TRANSIENT', 'transient'], bool) \
            else 'stationary'
        if self.scheme in ('CNLF', 'SBDF') and self.linearize != 'IMEX':
            raise NotImplementedError('{} needs the IMEX linearisation'.format(self.scheme))

    def setup(self):
        k = self.interp_ord
        self.th = fem.TaylorHood(self.mesh, k, list(self.dirichlet), gmesh=self.gmesh)
        th = self.th
        self.A = th.matrix()
        self.local_precond = self.config.get_item(['SOLVER', 'preconditioner'], str) == 'local'
        self.solver = None   # block-diagonal GMRES, made on first use
        self.saddle = None   # Cahouet-Chabard FGMRES, made on first use
        dev = 'cuda'
        self.u = torch.zeros(th.ndof, dtype=torch.float64, device=dev)
        self.b = torch.zeros_like(self.u)
        self.dinv = torch.zeros_like(self.u)
        self.W = torch.zeros_like(self.u)
        self._qp = None
        self._bpts = {}
        ic_u = self.ic.get('u', {}).get('all')
        ic_p = self.ic.get('p', {}).get('all')
        self._project(ic_u, ic_p)
        self.W.copy_(self.u)
        # previous solutions, most recent first (all the initial condition at the start, as OpenCMP's
        # gfu_0_list); the multistep IMEX schemes read them
        self.hist = [self.u.clone() for _ in range(3)]
        self.Kv = None
        self.vars = {}

    def quad_points(self):
        if self._qp is None:
            self._qp = self.th.quad_points()
        return self._qp

    def state(self):
        return {'u_p': self.u.cpu().numpy()}

    def load_state(self, st):
        if 'u_p' not in st or st['u_p'].size != self.u.numel():
            raise ValueError('the checkpoint holds no {}-dof Taylor-Hood solution'.format(self.u.numel()))
        self.u.copy_(torch.as_tensor(st['u_p']))
        self.W.copy_(self.u)
        for h in self.hist:
            h.copy_(self.u)

    def _project(self, vu, vp):
        """Initial condition: L2 projection of each velocity component and of the pressure."""
        th = self.th
        for c, (sp_, val) in enumerate(((th.V, vu), (th.V, vu), (th.Q, vp))):
            if val is None:
                continue
            M = fem.Matrix(sp_)
            f = fem.make_form(mass=1.0)
            M.assemble(f)
            X = sp_.quad_points()
            vals = _vec_at(val, X, 0.0)[..., c] if c < 2 else _at(val, X, 0.0)
            fq = torch.as_tensor(np.ascontiguousarray(vals.reshape(self.mesh.ne, -1)), device='cuda')
            bb = torch.zeros(sp_.ndof, dtype=torch.float64, device='cuda')
            fem.assemble_rhs(sp_, f, fem.make_rhs(src_qp=fq), bb)
            x = torch.zeros_like(bb)
            fem.KrylovSolver(M, method='CG', tol=1e-13, maxit=20000).solve(bb, x)
            th.component(self.u, c).copy_(x)

    def set_dirichlet(self, t: float):
        th = self.th
        for marker, v in self.dirichlet.items():
            lab = self.mesh.bc_names.index(marker)
            if lab not in self._bpts:
                self._bpts[lab] = th.V.boundary_points(1 << lab)
            g = _vec_at(v, self._bpts[lab], t)
            for c in range(2):
                th.V.set_boundary_values(1 << lab, g[:, c], th.component(self.u, c))

    def source(self, t):
        f = self.functions.get('source', {}).get('u')
        if f is None:
            return (0.0, 0.0), None
        if isinstance(f, Expr) and f.depends_on_space:
            return (0.0, 0.0), torch.as_tensor(_vec_at(f, self.quad_points(), t), device='cuda')
        v = _vec_at(f, np.zeros((1, 2)), t)[0]
        return (float(v[0]), float(v[1])), None

    def _solve(self, mass: float, dt: float, tcoef: Optional[float] = None):
        """Solve the system just assembled into A (mass coefficient `mass`, time step dt, divergence
        factor tcoef, default dt) for u; a stop at the iteration cap is accepted at the round-off
        floor (1e-9) when the requested tolerance is below it."""
        P = self.solver_params
        accept = 1e-9 if P['tol'] <= 1e-12 else P['tol']
        if mass > 0.0 and not self.local_precond:
            if self.saddle is None:
                self.saddle = SaddleSolver(self.th, self.A, restart=max(P['restart'], 50), tol=P['tol'],
                                           maxit=P['maxit'], precision=P['precision'])
            self.saddle.update(mass=mass, dt=dt, nu=self.kv, tcoef=tcoef)
            info = self.saddle.solve(self.b, self.u, raise_on_fail=False)
            if info.status != LB.OK and not (info.status == LB.NOT_CONVERGED and np.isfinite(info.relres)
                                             and info.relres <= accept):
                raise LB.OcmpError(info.status, 'INS solve: relative residual {:.3e} after {} FGMRES iterations'
                                   .format(info.relres, info.iterations))
            return info
        if self.solver is None:
            self.solver = fem.KrylovSolver(self.A, method='GMRES', restart=max(P['restart'], 50), precond='user',
                                           precision=P['precision'], tol=P['tol'], maxit=P['maxit'],
                                           inner_tol=P['inner_tol'])
        self.th.block_diag(self.A, self.dinv)
        self.solver.set_diag(self.dinv)
        self.solver.update()
        return checked_solve(self.solver, self.b, self.u, accept)

    def _push(self):
        self.hist = [self.u.clone()] + self.hist[:-1]

    def startup_step(self, dt, t_new, infos):
        """A start-up step of the multistep schemes (transient_multistep.py:51-100): implicit Euler
        with the IMEX linearisation (no convection term) and a tiny dt."""
        th = self.th
        uprev = self.u.clone()
        f, fq = self.source(t_new)
        self.set_dirichlet(t_new)
        th.assemble(self.A, mass=1.0, nu=self.kv, dt=dt)
        th.assemble_rhs(self.b, dt=dt, src=f, src_qp=fq, mass=1.0, uprev=uprev)
        infos.append(self._solve(1.0, dt))
        self._push()

    def step(self, theta, dt, t_new, t_old, transient, infos):
        """One time step: implicit Euler with Oseen Picard iterations, or one of the IMEX schemes
        (Euler IMEX, CNLF, SBDF of time_integration_schemes.py); the stationary solve when not
        transient."""
        if theta != 1.0 and not (theta == 0.5 and transient and self.linearize == 'Oseen'):
            raise NotImplementedError('INS runs on the GPU path with implicit Euler, Crank-Nicolson (Oseen), '
                                      'Euler IMEX, CNLF or SBDF')
        th = self.th
        uprev = self.u.clone() if transient else None
        mass = 1.0 if transient else 0.0
        f, fq = self.source(t_new)
        if theta == 0.5:
            # Crank-Nicolson with Oseen Picard iterations (time_integration_schemes.py:135-190): the
            # pressure / divergence terms implicit with the full dt, the viscous and linearised
            # convection terms halved, their old-time half moved to the linear form with the wind u^n
            # (ins.py:136-161: at the previous step the wind is that step's velocity):
            #   (M + coef(dt) + 1/2 ODE(.; W)) u = M u^n + dt/2 (f^{n+1} + f^n) - 1/2 ODE(u^n; u^n) u^n
            f0, fq0 = self.source(t_old)
            if self.Kv is None:
                self.Kv = th.matrix()
            th.assemble(self.Kv, mass=0.0, nu=self.kv, dt=dt, wind=uprev, tcoef=0.0)
            area = float(self.mesh_area())
            for it in range(self.max_picard):
                self.set_dirichlet(t_new)
                th.assemble(self.A, mass=1.0, nu=self.kv, dt=0.5 * dt, wind=self.W, tcoef=dt)
                th.assemble_rhs(self.b, dt=0.5 * dt, src=f, src_qp=fq, mass=1.0, uprev=uprev)
                th.assemble_rhs(self.b, dt=0.5 * dt, src=f0, src_qp=fq0, accumulate=True)
                LB.call('ocmp_spmv_axpby', self.Kv.h, -0.5, fem._ptr(uprev), 1.0, fem._ptr(self.b), None)
                infos.append(self._solve(1.0, 0.5 * dt, dt))
                d = self.u - self.W
                err, _ = th.errors(d)
                unorm, _ = th.errors(self.u)
                self.W.copy_(self.u)
                if err < self.abs_tol + self.rel_tol * unorm / math.sqrt(area):
                    break
            self._push()
            return
        if self.linearize == 'IMEX' and self.scheme == 'CNLF':
            # (2 coef + ODE + M) u = M u^{n-1} + L(t^{n-1}) - ODE(u^{n-1}) + 2 N(u^n)
            u1 = self.hist[1]
            f0, fq0 = self.source(t_old)
            self.set_dirichlet(t_new)
            th.assemble(self.A, mass=1.0, nu=self.kv, dt=dt, tcoef=2.0 * dt)
            th.assemble_rhs(self.b, dt=dt, src=f0, src_qp=fq0, mass=1.0, uprev=u1, imex=uprev, imex_coef=2.0)
            if self.Kv is None:
                self.Kv = th.matrix()
            th.assemble(self.Kv, mass=0.0, nu=self.kv, dt=dt, tcoef=0.0)
            LB.call('ocmp_spmv_axpby', self.Kv.h, -1.0, fem._ptr(u1), 1.0, fem._ptr(self.b), None)
            infos.append(self._solve(1.0, dt, 2.0 * dt))
            self._push()
            return
        if self.linearize == 'IMEX' and self.scheme == 'SBDF':
            # (coef + ODE + 11/6 M) u = L(t^{n+1}) + M (3 u^n - 3/2 u^{n-1} + 1/3 u^{n-2})
            #                            + 3 N(u^n) - 3 N(u^{n-1}) + N(u^{n-2})
            u1, u2 = self.hist[1], self.hist[2]
            comb = 3.0 * uprev - 1.5 * u1 + u2 / 3.0
            self.set_dirichlet(t_new)
            th.assemble(self.A, mass=11.0 / 6.0, nu=self.kv, dt=dt)
            th.assemble_rhs(self.b, dt=dt, src=f, src_qp=fq, mass=1.0, uprev=comb, imex=uprev, imex_coef=3.0)
            th.assemble_rhs(self.b, dt=dt, imex=u1, imex_coef=-3.0, accumulate=True)
            th.assemble_rhs(self.b, dt=dt, imex=u2, imex_coef=1.0, accumulate=True)
            infos.append(self._solve(11.0 / 6.0, dt))
            self._push()
            return
        if self.linearize == 'IMEX':
            self.set_dirichlet(t_new)
            th.assemble(self.A, mass=mass, nu=self.kv, dt=dt)
            th.assemble_rhs(self.b, dt=dt, src=f, src_qp=fq, mass=mass, uprev=uprev, imex=uprev)
            infos.append(self._solve(mass, dt))
            self._push()
            return
        area = float(self.mesh_area())
        for it in range(self.max_picard):
            self.set_dirichlet(t_new)
            th.assemble(self.A, mass=mass, nu=self.kv, dt=dt, wind=self.W)
            th.assemble_rhs(self.b, dt=dt, src=f, src_qp=fq, mass=mass, uprev=uprev)
            infos.append(self._solve(mass, dt))
            d = self.u - self.W
            err, _ = th.errors(d)
            unorm, _ = th.errors(self.u)
            self.W.copy_(self.u)
            if err < self.abs_tol + self.rel_tol * unorm / math.sqrt(area):
                break
        self._push()

    # ---------------------------------------------------------------- adaptive time stepping
    def adaptive_state(self):
        """What one step changes (solution, Picard wind, step history), for an attempt to be undone."""
        return self.u.clone(), self.W.clone(), [h.clone() for h in self.hist]

    def adaptive_restore(self, st):
        u, W, hist = st
        self.u.copy_(u)
        self.W.copy_(W)
        for h, h0 in zip(self.hist, hist):
            h.copy_(h0)

    def local_errors(self, kept, other):
        """[(|| kept - other ||, || kept ||)] over the components in OpenCMP's local error: the velocity
        only (ins.py:67-69)."""
        d, _ = self.th.errors(kept - other)
        n, _ = self.th.errors(kept)
        return [(d or 1e-10, n or 1e-10)]

    def mesh_area(self):
        X = self.mesh.coords[self.mesh.elements]
        a = X[:, 1] - X[:, 0]
        b = X[:, 2] - X[:, 0]
        return 0.5 * np.abs(a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]).sum()

    def l2_error_of(self, name: str, t: float) -> float:
        th = self.th
        if name == 'u':
            ref = self.ref_sol.get('u')
            rq = None if ref is None else torch.as_tensor(_vec_at(ref, self.quad_points(), t), device='cuda')
            return th.errors(self.u, rq)[0]
        if name == 'p':
            ref = self.ref_sol.get('p', 0.0)
            c = _scalar_at(ref, t)
            pv = th.component(self.u, 2)
            if c is not None:
                return th.Q.l2_error(pv, c)
            Xq = th.Q.quad_points()
            return th.Q.l2_error(pv, torch.as_tensor(_at(ref, Xq, t).reshape(self.mesh.ne, -1), device='cuda'))
        raise NotImplementedError('L2 error of {} is not on the GPU path'.format(name))

    def errors(self, t: float) -> List[str]:
        lines = []
        th = self.th
        for metric, names in self.metrics.items():
            for name in names:
                if metric.lower() == 'l2_norm' and name in ('u', 'p'):
                    lines.append('L2 norm in {}: {}'.format(name, self.l2_error_of(name, t)))
                elif metric == 'divergence' and name == 'u':
                    _, dv = th.errors(self.u)
                    lines.append('divergence of u: {}'.format(dv))
                else:
                    raise NotImplementedError('{} of {} is not on the GPU path'.format(metric, name))
        return lines


models_dict = {'Poisson': Poisson, 'MultiComponentINS': MultiComponentINS, 'INS': INS}


def get_model_class(model_name: str, dim_used: bool = False):
    """Model class by name (opencmp/models/misc.py:27-50)."""
    if dim_used:
        raise NotImplementedError('the diffuse interface method is not on the GPU path')
    try:
        return models_dict[model_name]
    except KeyError:
        raise KeyError('Tried to run with class {' + model_name + '}. \nThe available models are ' +
                       str(list(models_dict.keys())))
