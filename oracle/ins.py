"""Oracle (test infrastructure only): CPU restatement of OpenCMP's incompressible Navier-Stokes model
on Taylor-Hood spaces (velocity H1 order k per component, pressure H1 order k-1, triangles).

Follows ``opencmp/models/ins.py``:

* time-coefficient form (lines 238-250): dt * (-div(u) q - div(v) p - 1e-10 p q);
* ODE form (lines 178-196): dt * nu * grad(u) : grad(v), plus for the Oseen linearisation
  -dt * (u (x) w) : grad(v) = -dt * sum_c u_c (w . grad v_c);
* linear form (lines 282-296): dt * f . v; IMEX explicit part (lines 302-314):
  -dt * (grad(u^n) u^n) . v;
* the time-derivative mass term u . v (base_model.py:418-497).

The compound vector is [u_x (n_u), u_y (n_u), p (n_p)], each block numbered like the oracle's scalar
spaces. Element integrals use the collapsed (k + 2)-point simplex rule; the per-element numpy
contractions are checked against the oracle's scalar element matrices in the tests.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import oracle as O


class TaylorHood:
    def __init__(self, mesh, k: int, dirichlet_mask: int):
        if mesh.dim != 2:
            raise ValueError('the Taylor-Hood oracle is two-dimensional')
        self.mesh, self.k = mesh, k
        self.V = O.Space(mesh, O.H1, k, dirichlet_mask)
        self.Q = O.Space(mesh, O.H1, k - 1, 0)
        self.nu, self.np_ = self.V.ndof, self.Q.ndof
        self.ndof = 2 * self.nu + self.np_
        self.dv, self.dq = self.V.dofs(), self.Q.dofs()
        conn = self.V.sorted_conn()
        X = mesh.coords[conn]                                   # (ne, 3, 2)
        J = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]], axis=2)   # J[e, r, c] = dx_r / dxi_c
        self.det = np.abs(np.linalg.det(J))
        self.Jinv = np.linalg.inv(J)                              # (ne, 2, 2): dxi_c / dx_r = Jinv[c, r]
        self.x0 = X[:, 0]
        self.J = J
        self.xq, self.wq = O.rule(2, k + 2)
        self.phi, gref = O.tabulate(2, O.H1, k, self.xq)          # (nq, Lu), (nq, Lu, 2)
        self.psi, _ = O.tabulate(2, O.H1, k - 1, self.xq)         # (nq, Lp)
        # physical gradients (ne, nq, Lu, 2): grad phi = Jinv^T gref
        self.gphi = np.einsum('ecr,qic->eqir', self.Jinv, gref)
        self.free = np.concatenate([self.V.freedofs(), self.V.freedofs(), np.ones(self.np_, bool)])
        self.W = self.wq[None, :] * self.det[:, None]             # (ne, nq) weights

    def quad_points(self):
        """Physical quadrature points (ne, nq, 2)."""
        return self.x0[:, None, :] + np.einsum('erc,qc->eqr', self.J, self.xq)

    def _field(self, u):
        """Velocity values (ne, nq, 2) and gradients (ne, nq, 2 comp, 2 dir) of a compound vector."""
        ue = np.stack([u[self.dv], u[self.nu + self.dv]], axis=1)      # (ne, 2, Lu)
        val = np.einsum('qi,eci->eqc', self.phi, ue)
        grad = np.einsum('eqir,eci->eqcr', self.gphi, ue)
        return val, grad

    def matrix(self, mass: float, nu: float, dt: float, wind=None, eps_p: float = 1e-10, tcoef=None):
        """The compound system matrix (scipy CSR); `wind` a compound vector whose velocity is the
        Oseen wind, or None (Stokes / IMEX); tcoef the factor of the divergence and pressure terms
        (default dt; OpenCMP's CNLF doubles them)."""
        tc = dt if tcoef is None else tcoef
        W = self.W
        M = np.einsum('eq,qi,qj->eij', W, self.phi, self.phi)
        K = np.einsum('eq,eqir,eqjr->eij', W, self.gphi, self.gphi)
        Kuu = mass * M + dt * nu * K
        if wind is not None:
            wv, _ = self._field(wind)
            wg = np.einsum('eqc,eqic->eqi', wv, self.gphi)            # w . grad phi_i
            Kuu = Kuu - dt * np.einsum('eq,eqi,qj->eij', W, wg, self.phi)
        B = [-tc * np.einsum('eq,qi,eqj->eij', W, self.psi, self.gphi[..., c]) for c in range(2)]   # (ne, Lp, Lu)
        Kpp = -tc * eps_p * np.einsum('eq,qi,qj->eij', W, self.psi, self.psi)
        rows, cols, vals = [], [], []

        def add(rd, cd, blocks):
            ne, a, b = blocks.shape
            rows.append(np.repeat(rd, b, axis=1).ravel())
            cols.append(np.tile(cd, (1, a)).ravel())
            vals.append(blocks.ravel())
        ux, uy, p = self.dv, self.nu + self.dv, 2 * self.nu + self.dq
        add(ux, ux, Kuu)
        add(uy, uy, Kuu)
        add(p, ux, B[0])
        add(p, uy, B[1])
        add(ux, p, np.transpose(B[0], (0, 2, 1)))
        add(uy, p, np.transpose(B[1], (0, 2, 1)))
        add(p, p, Kpp)
        A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(self.ndof, self.ndof)).tocsr()
        A.sum_duplicates()
        return A

    def rhs(self, dt: float, f=(0.0, 0.0), mass: float = 0.0, uprev=None, imex=None, imex_coef: float = 1.0):
        """dt f . v + mass u_prev . v - imex_coef dt (grad(w) w) . v (the last with imex = w)."""
        W = self.W
        Fe = np.zeros((self.mesh.ne, 2, self.phi.shape[1]))
        fq = np.zeros((self.mesh.ne, len(self.wq), 2))
        fq[...] = np.asarray(f, float)
        q = dt * fq
        if uprev is not None:
            val, _ = self._field(uprev)
            q = q + mass * val
        if imex is not None:
            val, grad = self._field(imex)
            q = q - imex_coef * dt * np.einsum('eqcr,eqr->eqc', grad, val)
        Fe = np.einsum('eq,qi,eqc->eci', W, self.phi, q)
        b = np.zeros(self.ndof)
        np.add.at(b, self.dv, Fe[:, 0])
        np.add.at(b, self.nu + self.dv, Fe[:, 1])
        return b

    def set_boundary(self, mask: int, gvals: dict, u):
        """Constant per-label Dirichlet velocity {label: (gx, gy)} on both components."""
        for c in range(2):
            part = u[c * self.nu:(c + 1) * self.nu].copy()
            self.V.set_boundary(mask, {lab: g[c] for lab, g in gvals.items()}, part)
            u[c * self.nu:(c + 1) * self.nu] = part

    def solve(self, A, b, x):
        """Exact solve on the free dofs with the constrained values of x lifted."""
        import scipy.sparse.linalg as spla
        fr = self.free
        x = x.copy()
        x[fr] = spla.spsolve(A[fr][:, fr].tocsc(), b[fr] - A[fr][:, ~fr] @ x[~fr])
        return x

    def l2_error(self, u, ref=None):
        """sqrt(int |u_h - ref|^2), ref a callable of the points (..., 2) -> (..., 2) or None."""
        val, _ = self._field(u)
        r = 0.0 if ref is None else ref(self.quad_points())
        return float(np.sqrt(np.einsum('eq,eqc->', self.W, (val - r) ** 2)))

    def divergence(self, u):
        _, grad = self._field(u)
        d = grad[..., 0, 0] + grad[..., 1, 1]
        return float(np.sqrt(np.einsum('eq,eq->', self.W, d * d)))
