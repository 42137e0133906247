"""Stand-ins for the NGSolve objects that OpenCMP's Model/Solver methods pass around, backed by the
GPU library, so that those methods keep their reference signatures on the GPU path:

* ``Model.construct_preconditioners(a_assembled)``   (opencmp/models/base_model.py:365-383)
* ``Model.solve_single_step(a_lst, L_lst, precond_lst, gfu, time_step=0)``   (base_model.py:868-884)
* ``Model.linear_solve(a_assembled, L_assembled, precond, gfu)``   (base_model.py:886-947)
* ``Solver._assemble`` (opencmp/solvers/base_solver.py:368-377): ``a.Assemble()``, ``L.Assemble()``,
  ``precond.Update()``.

NGSolve builds its forms from symbolic integrands; here the integrand of each form is the library's
form description (``ocmp_form_t``, ``ocmp_rhs_t``) that the model fills in for the current step, so
a form handle is (space, device storage, the description to assemble). A model subclass written
against OpenCMP's method API overrides these methods and receives these handles:

* :class:`GridFunction` - ``gfu.vec`` is the device vector (a ``torch.Tensor``), ``gfu.space`` the
  space; ``gfu.space.FreeDofs()`` and ``.ndof`` as in NGSolve;
* :class:`BilinearForm` - ``a.mat`` is the assembled matrix (``fem.Matrix``), ``a.Assemble()``
  assembles the current form on the device, ``a.mat.mult(x, y)`` is ``y = A x``;
* :class:`LinearForm` - ``L.vec`` is the device right-hand side, ``L.Assemble()`` assembles it;
* :class:`Preconditioner` - ``Preconditioner(a, 'local' | 'direct' | ...)`` builds the library's
  solver on ``a``'s matrix (point Jacobi, the strip direct factorisation, ...), ``Update()``
  refreshes it after a reassembly.
"""
from __future__ import annotations

from typing import Callable, Optional

import torch

from . import fem

# OpenCMP's preconditioner names (docs: None, local, direct, multigrid, h1amg, bddc) -> library's
PRECONDITIONERS = {'None': 'none', 'none': 'none', 'local': 'jacobi', 'default': 'jacobi', 'jacobi': 'jacobi',
                   'block_jacobi': 'block_jacobi', 'direct': 'strip', 'strip': 'strip'}


class GridFunction:
    """``ngsolve.GridFunction`` stand-in: the solution vector of one space on the device."""

    def __init__(self, space: fem.Space, vec: Optional[torch.Tensor] = None):
        self.space = space
        self.vec = vec if vec is not None else torch.zeros(space.ndof, dtype=torch.float64, device='cuda')

    @property
    def ndof(self) -> int:
        return self.space.ndof


class BilinearForm:
    """``ngsolve.BilinearForm`` stand-in: the space, the device matrix and the form to assemble.
    ``form`` is an ``ocmp_form_t`` (``fem.make_form``), or a callable returning one; it is what
    ``Assemble()`` assembles."""

    def __init__(self, space: fem.Space, mat: fem.Matrix, form=None):
        self.space = space
        self.mat = mat
        self.form = form

    def Assemble(self, stream=None):
        f = self.form() if callable(self.form) else self.form
        if f is None:
            raise RuntimeError('BilinearForm.Assemble: no form set')
        self.mat.assemble(f, stream=stream)
        return self


class LinearForm:
    """``ngsolve.LinearForm`` stand-in: the device right-hand side and how to assemble it.
    ``assemble`` is a callable that writes ``vec`` (the model's linear form for the current step)."""

    def __init__(self, space: fem.Space, vec: torch.Tensor, assemble: Optional[Callable[[torch.Tensor], None]] = None):
        self.space = space
        self.vec = vec
        self._assemble = assemble

    def Assemble(self):
        if self._assemble is None:
            raise RuntimeError('LinearForm.Assemble: no linear form set')
        self._assemble(self.vec)
        return self


class Preconditioner:
    """``ngsolve.Preconditioner(a, kind)`` stand-in: the library's Krylov solver on ``a``'s matrix
    with the preconditioner that OpenCMP's name maps to (``local`` is point Jacobi, ``direct`` the
    strip direct factorisation), and the Krylov method and tolerances of the model's [SOLVER]
    section. ``Update()`` is NGSolve's ``Preconditioner.Update()``."""

    def __init__(self, a: BilinearForm, kind: str = 'local', method: str = 'GMRES', precision: str = 'fp64',
                 tol: float = 1e-8, maxit: int = 1000, restart: int = 50, inner_tol: float = 1e-4):
        if kind not in PRECONDITIONERS:
            raise NotImplementedError('preconditioner {!r} is not on the GPU path'.format(kind))
        self.a = a
        self.kind = kind
        self.solver = fem.KrylovSolver(a.mat, method=method, restart=restart, precond=PRECONDITIONERS[kind],
                                       precision=precision, tol=tol, maxit=maxit, inner_tol=inner_tol)

    def Update(self, stream=None):
        self.solver.update(stream=stream)
        return self
