"""The IMEX linearisation of MultiComponentINS (opencmp/models/multi_component_ins.py:390-430) with
the euler IMEX scheme (opencmp/solvers/time_integration_schemes.py:193-250): mass and diffusion
implicit, the convection dt (c^n, w . grad r) explicit at the previous step.

The reference's own euler IMEX fixture (test_mcins.py::TestDiffusion::test_imex_euler_cg) has no
velocity, so the explicit term vanishes there; this test runs one component in a constant wind
w = (1, 0.5) for five steps through the GPU solver and the same scheme restated with the oracle's
matrices (A = M + dt D K, b = M c^n - dt K_w c^n, Dirichlet 0), from the same initial vector:
the solutions agree to 1e-8 relative.
"""
import os
import shutil

import numpy as np
import pytest

from opencmp_gb300 import mesh as M
from opencmp_gb300.config import ConfigParser

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
FIX = os.path.join(GOLDEN, 'fixtures')


@pytest.mark.gpu
def test_imex_euler_explicit_convection_matches_oracle(gpu_lib, oracle, tmp_path):
    from opencmp_gb300.models import get_model_class
    from opencmp_gb300.solvers import get_solver_class
    run_dir = os.path.join(str(tmp_path), 'imex')
    shutil.copytree(os.path.join(FIX, 'mcins_diffusion'), run_dir)
    with open(os.path.join(run_dir, 'bc_dir', 'bc_config'), 'w') as fh:
        fh.write('[DIRICHLET]\na = left -> 0\n    right -> 0\n    top -> 0\n    bottom -> 0\n')
    with open(os.path.join(run_dir, 'ic_dir', 'ic_config'), 'w') as fh:
        fh.write('[MultiComponentINS]\nu = all -> [1.0, 0.5]\np = all -> 0\na = all -> sin(pi * x) * sin(pi * y)\n')
    with open(os.path.join(run_dir, 'model_dir', 'model_config'), 'w') as fh:
        fh.write('[PARAMETERS]\nkinematic_viscosity = all -> 1\ndiffusion_coefficients = a -> 0.1\n\n'
                 '[FUNCTIONS]\nsource = a -> 0\n')
    with open(os.path.join(run_dir, 'ref_sol_dir', 'ref_sol_config'), 'w') as fh:
        fh.write('[REFERENCE SOLUTIONS]\n\n[METRICS]\n')
    m = M.unit_square(12)
    mp = os.path.join(str(tmp_path), 'sq.npz')
    np.savez(mp, coords=m.coords, elements=m.elements, bfacets=m.bfacets, blabels=m.blabels,
             bc_names=np.array(m.bc_names))
    cfg = ConfigParser(os.path.join(run_dir, 'config'))
    cfg['MESH']['filename'] = mp
    cfg['OTHER']['run_dir'] = run_dir
    cfg['OTHER']['component_names'] = 'a'
    cfg['OTHER']['component_in_error_calc'] = 'a -> False'
    cfg['OTHER']['component_in_time_deriv'] = 'a -> True'
    cfg['FINITE ELEMENT SPACE']['elements'] = 'u -> VectorH1\np -> H1\na -> H1'
    cfg['FINITE ELEMENT SPACE']['interpolant_order'] = '2'
    cfg['SOLVER']['linearization_method'] = 'IMEX'
    cfg['TRANSIENT']['scheme'] = 'euler IMEX'
    dt, nsteps = 0.01, 5
    cfg['TRANSIENT']['time_range'] = '0.0, {}'.format(dt * nsteps)
    cfg['TRANSIENT']['dt'] = str(dt)
    cfg['ERROR ANALYSIS']['check_error'] = 'False'
    solver = get_solver_class(cfg)(get_model_class('MultiComponentINS'), cfg)
    v = solver.model.vars['a']
    c = v.u.cpu().numpy().copy()
    solver.solve()
    cg = v.u.cpu().numpy()
    # the oracle's restatement of the scheme, from the same initial vector
    o = oracle.Space(m, oracle.H1, 2, m.label_mask(m.bc_names))
    A = o.assemble(oracle.make_form(mass=1.0, diff=0.1, dt=dt))
    Kw = o.csr(o.assemble(oracle.make_form(wind=(1.0, 0.5))))
    free = o.freedofs().astype(bool)
    for _ in range(nsteps):
        b = o.rhs(oracle.make_form(mass=1.0, diff=0.1, dt=dt), oracle.make_rhs(dt=dt, mass=1.0, uprev=c))
        b = b - dt * Kw.dot(c)
        x = np.where(free, c, 0.0)
        o.cg(A, b, x, tol=1e-13)
        c = x
    assert np.linalg.norm(cg - c) <= 1e-8 * np.linalg.norm(c), np.linalg.norm(cg - c) / np.linalg.norm(c)
