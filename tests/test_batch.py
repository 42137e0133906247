"""Batched solves (ocmp_matrix_create_batch / ocmp_assemble_matrix_batch / ocmp_solve_batch): each
instance of a batch must match the same system solved on its own and the CPU oracle."""
import numpy as np
import pytest

from opencmp_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _forms(fem, B, rng):
    eps = 10 ** rng.uniform(-2, 0, B)
    ang = rng.uniform(0, 2 * np.pi, B)
    return [(float(e), (float(np.cos(a)), float(np.sin(a)))) for e, a in zip(eps, ang)]


@pytest.mark.parametrize('precision,graph', [('fp64', False), ('mixed', False), ('mixed', True)])
def test_batched_gmres_matches_single_solves(gpu_lib, oracle, precision, graph):
    import torch
    from opencmp_gb300 import fem
    rng = np.random.default_rng(0)
    m = M.unit_square(12)
    sp = fem.Space(m, 'H1', 2, m.bc_names)
    B = 5
    coefs = _forms(fem, B, rng)
    forms = [fem.make_form(diff=e, dt=1.0, wind=w) for e, w in coefs]
    kw = dict(jacobi64=precision == 'fp64', jacobi32=precision == 'mixed')
    A = fem.Matrix(sp, batch=B, **kw)
    A.assemble_batch(forms)
    b1 = torch.zeros(sp.ndof, dtype=torch.float64, device='cuda')
    fem.assemble_rhs(sp, forms[0], fem.make_rhs(src_const=1.0), b1)
    b = b1.repeat(B)
    x = torch.zeros_like(b)
    sv = fem.KrylovSolver(A, method='GMRES', restart=40, precision=precision, tol=1e-10, maxit=4000, inner_tol=1e-4)
    if graph:
        sv.set_graph(True)
    infos = sv.solve_batch(b, x)
    assert all(i.status == 0 and i.relres <= 1e-10 for i in infos)
    o = oracle.Space(m, oracle.H1, 2, m.label_mask(m.bc_names))
    xb = x.view(B, -1).cpu().numpy()
    for q, (e, w) in enumerate(coefs):
        A1 = fem.Matrix(sp, **kw)
        A1.assemble(forms[q])
        x1 = torch.zeros_like(b1)
        fem.KrylovSolver(A1, method='GMRES', restart=40, precision=precision, tol=1e-10, maxit=4000,
                         inner_tol=1e-4).solve(b1, x1)
        x1 = x1.cpu().numpy()
        assert np.linalg.norm(xb[q] - x1) <= 1e-8 * np.linalg.norm(x1)
        of = oracle.make_form(diff=e, dt=1.0, wind=w)
        ao = o.assemble(of)
        bo = o.rhs(of, oracle.make_rhs(src_kind=oracle.SRC_CONST, src=(1.0,)))
        assert o.relres(ao, bo, xb[q]) <= 1.05e-10
