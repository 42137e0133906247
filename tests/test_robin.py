"""Robin boundary conditions of the Poisson model (opencmp/models/poisson.py:93-97, 153-157):
-dt dc r (u, v) in the bilinear form and -dt dc r q (v) in the linear form on a marker whose value
is [r, q]. With the weak form's boundary term dc (n.grad u, v) these impose n.grad u = r (u - q),
as the Neumann data h of the same forms is n.grad u (poisson.py:148-151).

CPU: the linear-form data -r q of constant and space-dependent [r, q]. GPU: matrix entries with
Robin terms on two labels against the oracle (1e-12 relative to the largest entry, FP64 and
double-float assembly, continuous and DG spaces); and a manufactured solution through run():
u = sin(pi x) cos(pi y) with eta = 0.5, the reference's h-convergence problem with the left
boundary turned into a Robin boundary (r = -2, q = u - n.grad u / r), refined three times:
the L2 error falls at the order-4 rate of P3.
"""
import math
import os
import shutil

import numpy as np
import pytest

from opencmp_gb300 import mesh as M
from opencmp_gb300.config import ConfigParser, parse

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
FIX = os.path.join(GOLDEN, 'fixtures')


def test_robin_linear_form_data():
    from opencmp_gb300.models import _RobinData, _at, _scalar_at
    X = np.array([[[0.5, 0.25], [0.2, 0.4]]])
    d = _RobinData(parse('[-2, x*y]'))
    assert d.depends_on_space and _scalar_at(d, 0.0) is None
    assert np.allclose(_at(d, X, 0.0), 2 * X[..., 0] * X[..., 1])
    c = _RobinData(parse('[-3, 2*t + 1]'))
    assert not c.depends_on_space and abs(_scalar_at(c, 0.5) - 6.0) < 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize('dfloat', [False, True], ids=['fp64', 'dfloat'])
@pytest.mark.parametrize('kind,order', [(0, 2), (0, 3), (1, 2)], ids=['h1-p2', 'h1-p3', 'dg-p2'])
def test_robin_matrix_matches_oracle(gpu_lib, oracle, kind, order, dfloat):
    from opencmp_gb300 import fem
    m = M.unit_square(6)
    rob = {1: 0.7, 3: -1.3}
    kw = dict(mass=0.5, diff=0.8, dt=0.4, robin=rob)
    if kind == 1:
        kw.update(dg=True, ipc=10.0, nitsche_mask=m.label_mask(m.bc_names[:1]))
    g = fem.Space(m, 'H1' if kind == 0 else 'L2', order, m.bc_names[:1] if kind == 0 else ())
    o = oracle.Space(m, kind, order, m.label_mask(m.bc_names[:1]) if kind == 0 else 0)
    A = fem.Matrix(g, dfloat=dfloat)
    A.assemble(fem.make_form(**kw))
    ao = o.assemble(oracle.make_form(**kw))
    v = A.values()
    assert np.abs(v - ao).max() <= 1e-12 * np.abs(ao).max()
    # the Robin term changed the matrix: without it the entries differ
    kw0 = dict(kw)
    kw0.pop('robin')
    assert np.abs(o.assemble(oracle.make_form(**kw0)) - ao).max() > 1e-3 * np.abs(ao).max()


@pytest.mark.gpu
@pytest.mark.parametrize('dg', [False, True], ids=['cg', 'dg'])
def test_robin_manufactured_solution_through_run(gpu_lib, tmp_path, capsys, dg):
    from opencmp_gb300.run import run
    run_dir = os.path.join(str(tmp_path), 'robin')
    shutil.copytree(os.path.join(FIX, 'poisson_h_convergence'), run_dir)
    # left boundary (x = 0, n = (-1, 0)): n.grad u = -pi cos(pi y), u = 0, so with r = -2
    # q = u - n.grad u / r = -(pi / 2) cos(pi y)
    with open(os.path.join(run_dir, 'bc_dir', 'bc_config'), 'w') as fh:
        fh.write('[DIRICHLET]\nu = right  ->  sin(pi * x) * cos(pi * y)\n\n'
                 '[NEUMANN]\nu = top    ->  -pi * sin(pi * x) * sin(pi * y)\n'
                 '    bottom ->  pi * sin(pi * x) * sin(pi * y)\n\n'
                 '[ROBIN]\nu = left   ->  [-2, -pi / 2 * cos(pi * y)]\n')
    cfg = ConfigParser(os.path.join(run_dir, 'config'))
    cfg['MESH']['filename'] = os.path.join(GOLDEN, 'unit_square_coarse.npz')
    cfg['OTHER']['run_dir'] = run_dir
    cfg['DG']['DG'] = str(dg)
    cfg['ERROR ANALYSIS']['num_refinements'] = '3'
    run('', cfg)
    out = capsys.readouterr().out.strip().split('\n')
    errs = [float(l.split(': ')[1]) for l in out if l.startswith('L2 norm at refinement')]
    assert len(errs) == 3
    rates = [math.log(errs[k] / errs[k + 1]) / math.log(2) for k in range(2)]
    assert errs[-1] < 1e-4 and rates[-1] >= 3.5, (errs, rates)
