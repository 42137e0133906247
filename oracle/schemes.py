"""Oracle (test infrastructure only): CPU restatement of OpenCMP's one-step time schemes.

``opencmp/solvers/time_integration_schemes.py`` builds, for explicit Euler (lines 25-76),
implicit Euler (79-132) and Crank-Nicolson (134-191), the system

    (M + theta dt K_ode + dt K_skel) u^{n+1} = M u^n - (1 - theta) dt K_ode u^n
                                              + theta dt L(t^{n+1}) + (1 - theta) dt L(t^n)

with theta = 0, 1, 1/2. K_skel is the model's time-coefficient form (the interior-facet DG terms,
``poisson.py:100-131``, ``multi_component_ins.py:158-199``), K_ode the rest of its operator
(``poisson.py:71-98``, ``multi_component_ins.py:201-303``) and L the linear form with dt = 1.
Dirichlet data of H1 spaces is set on the constrained dofs at t^{n+1} before the solve
(``base_model.py:321-341``), and the free block is solved exactly (sparse LU) with the constrained
values lifted to the right-hand side (``base_model.py:918-922``).

The oracle's own assembly (``oracle.c``) supplies M, K and L; K_skel is the difference of the
assembled operator with and without its interior-facet terms.
"""
from __future__ import annotations

from typing import Callable, Dict, Optional

import numpy as np

from . import oracle as O

THETA = {'explicit euler': 0.0, 'crank nicolson': 0.5, 'implicit euler': 1.0}


def theta_run(mesh, kind: int, order: int, scheme: str, dt: float, nsteps: int, fkw: dict,
              dirichlet: Dict[int, Callable[[float], float]], u0_src, bval: Optional[Dict[int, float]] = None,
              t0: float = 0.0):
    """Run `nsteps` steps of `scheme`; returns (oracle space, final solution).

    fkw: make_form keywords of the operator (diff, wind, ipc, dg, outflow/wn/nitsche masks);
    dirichlet: {label: g(t)} (H1: constrained dofs; L2: the DG Dirichlet datum of the linear form);
    u0_src: (source kind, params) of the initial condition's L2 projection;
    bval: constant Neumann-type data per label (already multiplied by the model's coefficient)."""
    import scipy.sparse.linalg as spla
    theta = THETA[scheme]
    dmask = 0
    for lab in dirichlet:
        dmask |= 1 << lab
    s = O.Space(mesh, kind, order, dmask if kind == O.H1 else 0)
    form = O.make_form(dt=1.0, **fkw)
    K = s.assemble(form)
    Kn = s.assemble(O.make_form(dt=1.0, **dict(fkw, dg=False)))
    Ks = K - Kn
    Mm = s.assemble(O.make_form(mass=1.0, dt=0.0))
    A = s.csr(Mm + theta * dt * Kn + dt * Ks)
    Mc, Knc = s.csr(Mm), s.csr(Kn)
    free = s.freedofs()
    lu = spla.splu(A[free][:, free].tocsc())
    Afd = A[free][:, ~free]

    def L(t):
        g = {lab: fn(t) for lab, fn in dirichlet.items()} if kind == O.L2 else None
        return s.rhs(form, O.make_rhs(dt=1.0, bval=bval, gval=g))

    u = s.project(*u0_src)
    t = t0
    for _ in range(nsteps):
        t_new = t + dt
        b = Mc @ u + theta * dt * L(t_new)
        if theta < 1.0:
            b += (1.0 - theta) * dt * (L(t) - Knc @ u)
        x = u.copy()
        if kind == O.H1 and dirichlet:
            s.set_boundary(dmask, {lab: fn(t_new) for lab, fn in dirichlet.items()}, x)
        x[free] = lu.solve(b[free] - Afd @ x[~free])
        u = x
        t = t_new
    return s, u


def ramp(t, p1=0.0, p2=1.0, tr=1.0):
    """OpenCMP's ramp (opencmp/helpers/math.py:116-131): cosine blend from p1 to p2 over [0, tr], then p2."""
    return 0.5 * (p1 - p2) * np.cos(t * np.pi / tr) + 0.5 * (p1 + p2) if tr - t > 0 else p2
