"""Flexible GMRES with a Cahouet-Chabard pressure preconditioner for the Taylor-Hood saddle-point
systems of the INS model.

OpenCMP solves these systems with a sparse direct solver (``opencmp/models/ins.py`` with
``linear_solver = default``); the GPU path solves them by Krylov iteration. Block Jacobi on the
saddle-point matrix (velocity Jacobi, a diagonal Schur approximation; ``ocmp_th_block_diag``) needs
iteration counts that grow like 1/h on the lid-driven cavity (about 2,500 GMRES(50) iterations on
a 64 x 64 x 2 mesh). The preconditioner here keeps velocity Jacobi and replaces the pressure block
with the Cahouet-Chabard approximation of the inverse Schur complement, which gives iteration
counts that do not grow with the mesh.

The compound system (``oracle/ins.py``, the forms of ``opencmp/models/ins.py:178-250``) is

    [ A_u      tc B^T         ] [u]   [f]
    [ tc B    -tc eps M_p     ] [p] = [g],   A_u = alpha M + beta K (+ convection),

with alpha the mass coefficient of the time scheme, beta = dt nu, tc the factor of the divergence
terms (dt; 2 dt for CNLF) and eps = 1e-10. Its Schur complement is
-(tc^2 B A_u^-1 B^T + tc eps M_p), and

    (B (alpha M + beta K)^-1 B^T)^-1  ~  alpha L_p^-1 + beta M_p^-1

(Cahouet & Chabard 1988), L_p the pressure Laplacian. The pressure block of the preconditioner is
therefore

    z_p = -(alpha (L_p + delta M_p)^-1 r_p + beta D(M_p)^-1 r_p) / tc^2,   delta = alpha eps / tc,

where delta makes the preconditioner exact on constant pressures (the one mode that L_p does not
see and that the eps term alone fixes).

Two implementations. The default runs entirely in the library (``SaddleSolver(impl='library')``):
GMRES with OCMP_PRE_CAHOUET_CHABARD, the Laplacian solve applied exactly by the strip direct
factorisation of the pressure operator, so the preconditioner is fixed and plain GMRES suffices.
The host implementation (``impl='host'``) applies (L_p + delta M_p)^-1 by an inexact Jacobi-CG
solve (``ocmp_solve``) and therefore runs flexible GMRES (Saad 1993), which stores the
preconditioned directions; its Arnoldi algebra runs as torch tensor operations.
"""
from __future__ import annotations

import math
from typing import Callable, Optional

import numpy as np
import torch

from . import _lib as LB
from . import fem


class FGMRESInfo:
    """Result of :func:`fgmres`, with the fields of the library's ``ocmp_solve_info_t``."""

    def __init__(self, status, iterations, outer_iterations, relres0, relres, inner_iterations=0):
        self.status, self.iterations, self.outer_iterations = status, iterations, outer_iterations
        self.relres0, self.relres, self.inner_iterations = relres0, relres, inner_iterations


def fgmres(matvec: Callable[[torch.Tensor, torch.Tensor], None],
           precond: Callable[[torch.Tensor, torch.Tensor], None],
           b: torch.Tensor, x: torch.Tensor, free: torch.Tensor, restart: int = 50, tol: float = 1e-8,
           maxit: int = 2000, target_margin: float = 0.9) -> FGMRESInfo:
    """Right-preconditioned flexible GMRES(m) on the free dofs of A x = b, in place on x.

    ``matvec(v, out)`` writes A v over all rows; ``precond(r, z)`` writes an approximation of
    A^-1 r that may change from call to call, zero on constrained dofs. The constrained entries of
    x hold the Dirichlet values and are kept. The relative residual is |free (b - A x)| over
    |free (b - A x_D)|, x_D the Dirichlet part of x (the library's definition). Orthogonalisation is
    classical Gram-Schmidt with a second pass; a cycle stops when its residual estimate falls below
    ``target_margin`` times the tolerance, and the true residual decides convergence.
    """
    n = b.numel()
    dev, dt = b.device, b.dtype
    f = free.to(dt)
    w = torch.empty(n, dtype=dt, device=dev)
    xd = x * (1.0 - f)
    matvec(xd, w)
    nb = float(torch.linalg.vector_norm(f * (b - w)))
    if nb == 0.0:
        nb = 1.0

    def residual(out):
        matvec(x, w)
        torch.sub(b, w, out=out)
        out.mul_(f)
        return float(torch.linalg.vector_norm(out))

    m = restart
    V = torch.empty((m + 1, n), dtype=dt, device=dev)
    Z = torch.empty((m, n), dtype=dt, device=dev)
    beta = residual(V[0])
    relres0 = beta / nb
    it = cycles = 0
    status = LB.OK if beta <= tol * nb else LB.NOT_CONVERGED
    while status != LB.OK and it < maxit and math.isfinite(beta):
        cycles += 1
        V[0].div_(beta)
        H = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        g = np.zeros(m + 1)
        g[0] = beta
        k = 0
        for j in range(m):
            precond(V[j], Z[j])
            matvec(Z[j], w)
            w.mul_(f)
            Vj = V[:j + 1]
            h = Vj @ w
            w.sub_(h @ Vj)
            h2 = Vj @ w
            w.sub_(h2 @ Vj)
            hcol = (h + h2).cpu().numpy()
            hn = float(torch.linalg.vector_norm(w))
            it += 1
            col = np.append(hcol, hn)
            for i in range(j):
                a, c = col[i], col[i + 1]
                col[i], col[i + 1] = cs[i] * a + sn[i] * c, -sn[i] * a + cs[i] * c
            r = math.hypot(col[j], col[j + 1])
            if r == 0.0:
                status = LB.BREAKDOWN
                break
            k = j + 1
            cs[j], sn[j] = col[j] / r, col[j + 1] / r
            col[j], col[j + 1] = r, 0.0
            H[:j + 2, j] = col
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            if hn == 0.0 or abs(g[j + 1]) <= target_margin * tol * nb or it >= maxit:
                break
            V[j + 1] = w / hn
        if k == 0:
            break
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:k] @ y[i + 1:k]) / H[i, i]
        x.add_(torch.as_tensor(y, dtype=dt, device=dev) @ Z[:k])
        beta = residual(V[0])
        if beta <= tol * nb:
            status = LB.OK
        elif status == LB.BREAKDOWN:
            break
        else:
            status = LB.NOT_CONVERGED
    if not math.isfinite(beta):
        status = LB.ERR_NONFINITE
    return FGMRESInfo(status, it, cycles, relres0, beta / nb)


def _diag_positions(space) -> np.ndarray:
    """Index of each row's diagonal entry in the space's CSR values."""
    rp, col = space.pattern()
    rows = np.repeat(np.arange(space.ndof, dtype=np.int64), np.diff(rp))
    pos = np.flatnonzero(col == rows)
    if pos.size != space.ndof:
        raise ValueError('the pattern lacks diagonal entries')
    return pos


class SaddleSolver:
    """GMRES(m) with the Cahouet-Chabard block-diagonal preconditioner for a Taylor-Hood system
    (``fem.TaylorHood``) assembled into ``A``.

    ``impl='library'`` (the default): the library's GMRES with OCMP_PRE_CAHOUET_CHABARD, the whole
    iteration on the device. The pressure block's Laplacian solve is exact: the strip direct
    factorisation of L_p + sigma M_p, sigma = max(delta, 1), computed in FP32 once per pressure
    operator (delta alone would leave the FP32 factorisation singular on the constant pressure, the
    mode the outer FP64 GMRES resolves; sigma = 1 keeps the operator's condition near 1/h^2).
    ``precision='mixed'`` runs the inner GMRES in FP32 with FP64 refinement.

    ``impl='host'``: flexible GMRES on the host (``fgmres``), whose pressure block is an inexact
    Jacobi-CG solve of (L_p + delta M_p) z = r_p to ``inner_tol`` (``ocmp_solve``), the outer
    Arnoldi algebra in torch.
    """

    def __init__(self, th, A, restart: int = 50, tol: float = 1e-8, maxit: int = 2000, inner_tol: float = 0.1,
                 inner_maxit: int = 1000, precision: str = 'fp64', eps_p: float = 1e-10, impl: str = 'library'):
        if impl not in ('library', 'host'):
            raise ValueError("impl is 'library' or 'host'")
        self.impl = impl
        self.th, self.A = th, A
        self.restart, self.tol, self.maxit = restart, tol, maxit
        self.inner_tol, self.inner_maxit = inner_tol, inner_maxit
        self.precision, self.eps_p = precision, eps_p
        nd, nu2 = th.ndof, 2 * th.nu
        self.nu2 = nu2
        self.free = torch.as_tensor(th.C.FreeDofs(), device='cuda')
        self.dinv = torch.zeros(nd, dtype=torch.float64, device='cuda')
        self.Mp = fem.Matrix(th.Q)
        self.Mp.assemble(fem.make_form(mass=1.0))
        pos = torch.as_tensor(_diag_positions(th.Q), device='cuda')
        self.mp_dinv = 1.0 / self.Mp.device_values()[0][pos]
        self.Lp = fem.Matrix(th.Q, fp32=precision == 'mixed')
        self.inner = None
        self.delta = None
        self.zp = torch.zeros(th.np, dtype=torch.float64, device='cuda')
        self.inner_iterations = 0
        self.coef = (1.0, 0.0, 1.0)
        self.lib = None
        if impl == 'library':
            self.lib = fem.KrylovSolver(A, method='GMRES', restart=restart, precond='cahouet_chabard',
                                        precision=precision, tol=tol, maxit=maxit, inner_tol=1e-4, check_every=1)

    def _pressure_operator(self, delta: float) -> bool:
        """(Re)assemble the pressure operator and, on the host path, its inner CG solver when delta
        changes; True when it changed."""
        if self.delta == delta:
            return False
        if self.impl == 'library':
            self.Lp.assemble(fem.make_form(mass=max(delta, 1.0), diff=1.0))
        else:
            self.Lp.assemble(fem.make_form(mass=delta, diff=1.0))
            self.inner = fem.KrylovSolver(self.Lp, method='CG', precond='jacobi', precision=self.precision,
                                          tol=self.inner_tol, maxit=self.inner_maxit, inner_tol=self.inner_tol)
        self.delta = delta
        return True

    def update(self, mass: float, dt: float, nu: float, tcoef: Optional[float] = None):
        """Take the coefficients of the system just assembled into A: the mass coefficient alpha,
        beta = dt nu, and tc = tcoef (default dt); refresh the velocity Jacobi diagonal."""
        tc = dt if tcoef is None else tcoef
        self.coef = (float(mass), float(dt) * float(nu), float(tc))
        changed = False
        if mass > 0.0:
            changed = self._pressure_operator(mass * self.eps_p / tc)
        self.th.block_diag(self.A, self.dinv)
        if self.lib is not None:
            if mass <= 0.0:
                raise NotImplementedError('the library saddle-point solve needs a mass term (transient systems)')
            self.lib.update()
            n2 = self.nu2
            self.lib.set_cahouet_chabard(self.Lp, self.dinv[:n2].contiguous(), self.mp_dinv, self.coef[0],
                                         self.coef[1], self.coef[2], changed)

    def precond(self, r: torch.Tensor, z: torch.Tensor):
        alpha, beta, tc = self.coef
        n2 = self.nu2
        torch.mul(self.dinv[:n2], r[:n2], out=z[:n2])
        rp, zp = r[n2:], z[n2:]
        if alpha > 0.0:
            self.zp.zero_()
            info = self.inner.solve(rp.contiguous(), self.zp, raise_on_fail=False)
            if info.status not in (LB.OK, LB.NOT_CONVERGED):
                LB.check(info.status)
            self.inner_iterations += info.iterations
            torch.mul(self.mp_dinv, rp, out=zp)
            zp.mul_(beta)
            zp.add_(self.zp, alpha=alpha)
        else:
            torch.mul(self.mp_dinv, rp, out=zp)
            zp.mul_(beta)
        zp.mul_(-1.0 / (tc * tc))

    def match_pressure_mean(self, u: torch.Tensor, ref: torch.Tensor):
        """Shift the pressure part of u so that its pressure-mass-weighted mean equals ref's. The
        constant pressure is determined only by the 1e-10 p q term, so a guess extrapolated in time
        carries whatever the previous steps left in it, amplified by the extrapolation; left alone it
        grows from step to step until the FP32 inner iteration loses the pressure gradients to
        cancellation. The shift changes the residual by far less than the tolerance."""
        n2 = self.nu2
        w = 1.0 / self.mp_dinv
        du = torch.dot(w, u[n2:] - ref[n2:]) / w.sum()
        u[n2:] -= du

    def matvec(self, v: torch.Tensor, out: torch.Tensor):
        self.A.mult(v, out)

    def solve(self, b: torch.Tensor, x: torch.Tensor, raise_on_fail: bool = True) -> FGMRESInfo:
        """Solve A x = b on the free dofs from the initial guess x (its constrained entries hold the
        Dirichlet values)."""
        self.inner_iterations = 0
        if self.lib is not None:
            li = self.lib.solve(b, x, raise_on_fail=False)
            info = FGMRESInfo(li.status, li.iterations, li.outer_iterations, li.relres0, li.relres)
        else:
            info = fgmres(self.matvec, self.precond, b, x, self.free, restart=self.restart, tol=self.tol,
                          maxit=self.maxit)
        info.inner_iterations = self.inner_iterations
        if raise_on_fail and info.status != LB.OK:
            raise LB.OcmpError(info.status, 'FGMRES (Cahouet-Chabard): relative residual {:.3e} after {} '
                                            'iterations'.format(info.relres, info.iterations))
        return info
