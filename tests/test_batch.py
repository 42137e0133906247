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


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_group_solve_over_uneven_instances_matches_batches(gpu_lib, oracle, precision):
    """A solver group (ocmp_group_*) over uneven instances: three members of different meshes and
    orders (two of them batched), solved by one kernel sequence. Every instance meets the tolerance,
    satisfies the oracle's system, and agrees with its member's own batched solve (the same GMRES;
    the group sums its dot products over fewer blocks, so the iteration counts may differ by
    rounding: within two) to what the tolerance allows."""
    import torch
    from opencmp_gb300 import fem
    rng = np.random.default_rng(3)
    kw = dict(jacobi64=precision == 'fp64', jacobi32=precision == 'mixed')
    classes = [(8, 1, 3), (12, 2, 1), (16, 3, 2)]   # (n, p, instances)
    members, bs, xs, ref, cases = [], [], [], [], []
    for n, p, B in classes:
        m = M.unit_square(n)
        sp = fem.Space(m, 'H1', p, m.bc_names)
        coefs = _forms(fem, B, rng)
        forms = [fem.make_form(diff=e, dt=1.0, wind=w) for e, w in coefs]
        A = fem.Matrix(sp, batch=B, **kw)
        A.assemble_batch(forms)
        b1 = torch.zeros(sp.ndof, dtype=torch.float64, device='cuda')
        fem.assemble_rhs(sp, forms[0], fem.make_rhs(src_const=1.0), b1)
        sv = fem.KrylovSolver(A, method='GMRES', restart=30, precision=precision, tol=1e-10, maxit=3000,
                              inner_tol=1e-4)
        b = b1.repeat(B)
        xr = torch.zeros_like(b)
        ref.append((sv.solve_batch(b, xr), xr.clone()))
        members.append((sv, A))
        bs.append(b)
        xs.append(torch.zeros_like(b))
        cases.append((m, sp, p, coefs, B))
    group = fem.KrylovGroup([sv for sv, _ in members])
    infos = group.solve(bs, xs)
    assert len(infos) == sum(c[-1] for c in cases)
    assert all(i.status == 0 and i.relres <= 1e-10 for i in infos)
    k = 0
    for (m, sp, p, coefs, B), (rinfos, xr), x in zip(cases, ref, xs):
        assert (x - xr).abs().max().item() <= 1e-8 * xr.abs().max().item()
        for q in range(B):
            assert abs(infos[k].iterations - rinfos[q].iterations) <= 2
            k += 1
        o = oracle.Space(m, oracle.H1, p, m.label_mask(m.bc_names))
        xb = x.view(B, -1).cpu().numpy()
        for q, (e, w) in enumerate(coefs):
            of = oracle.make_form(diff=e, dt=1.0, wind=w)
            ao = o.assemble(of)
            bo = o.rhs(of, oracle.make_rhs(src_kind=oracle.SRC_CONST, src=(1.0,)))
            assert o.relres(ao, bo, xb[q]) <= 1.05e-10
    # a second solve from the same zero start reuses the captured cycle and gives the same result
    x2 = [torch.zeros_like(b) for b in bs]
    infos2 = group.solve(bs, x2)
    assert all(torch.equal(a, c) for a, c in zip(x2, xs))
    assert [i.iterations for i in infos2] == [i.iterations for i in infos]


def test_group_refuses_mismatched_members(gpu_lib):
    import torch
    from opencmp_gb300 import fem, _lib
    m = M.unit_square(6)
    sp = fem.Space(m, 'H1', 1, m.bc_names)
    A = fem.Matrix(sp, jacobi64=True)
    A.assemble(fem.make_form(diff=1.0, dt=1.0))
    s1 = fem.KrylovSolver(A, method='GMRES', restart=20, precision='fp64')
    s2 = fem.KrylovSolver(A, method='GMRES', restart=30, precision='fp64')
    s3 = fem.KrylovSolver(A, method='CG', precision='fp64')
    for bad in ([s1, s2], [s1, s3]):
        with pytest.raises(_lib.OcmpError) as e:
            fem.KrylovGroup(bad)
        assert e.value.status == _lib.ERR_UNSUPPORTED
