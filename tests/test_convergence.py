"""OpenCMP's convergence tests ([ERROR ANALYSIS] convergence_test,
opencmp/post_processing/error_analysis.py:28-161) and the uniform refinement they run on
(netgen's Mesh.Refine).

CPU: refinement preserves area/volume and boundary labels, multiplies the element count by 2^D,
keeps the mesh conforming (every interior facet in exactly two elements, every boundary facet a
face of one element), keeps shapes from degrading over repeated refinements; the rate formulas and
the table. GPU: the reference's own h-convergence configuration (the coarse unstructured square,
order 3, space-dependent Dirichlet and Neumann data, five refinements) through run(), CG and DG:
the printed rates approach the order-(p + 1) = 4 rate of the L2 error.
"""
import math
import os

import numpy as np
import pytest

from opencmp_gb300 import mesh as M
from opencmp_gb300.config import ConfigParser
from opencmp_gb300 import post_processing as PP

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
FIX = os.path.join(GOLDEN, 'fixtures')


def _measure(m):
    X = m.coords[m.elements]
    d = X[:, 1:] - X[:, :1]
    return np.abs(np.linalg.det(d)) / math.factorial(m.dim)


def _facets(elements, D):
    loc = [np.delete(np.arange(D + 1), f) for f in range(D + 1)]
    F = np.concatenate([np.sort(elements[:, l], axis=1) for l in loc])
    keys, counts = np.unique(F, axis=0, return_counts=True)
    return keys, counts


def _check_conforming(m):
    keys, counts = _facets(m.elements, m.dim)
    assert counts.max() <= 2
    bf = np.sort(m.bfacets, axis=1)
    once = keys[counts == 1]
    a = {tuple(r) for r in once}
    b = {tuple(r) for r in bf}
    assert a == b          # boundary facets are exactly the facets of one element


@pytest.mark.parametrize('mk', [lambda: M.load_mesh(os.path.join(GOLDEN, 'unit_square_coarse.npz')),
                                lambda: M.unit_square(3), lambda: M.unit_cube(2)], ids=['coarse-square', 'square', 'cube'])
def test_uniform_refinement(mk):
    m = mk()
    r = M.refine_uniform(m)
    D = m.dim
    assert r.ne == m.ne * 2 ** D
    assert r.bfacets.shape[0] == m.bfacets.shape[0] * 2 ** (D - 1)
    assert abs(_measure(r).sum() - _measure(m).sum()) < 1e-13
    for lab in range(len(m.bc_names)):
        assert (r.blabels == lab).sum() == (m.blabels == lab).sum() * 2 ** (D - 1)
    _check_conforming(r)
    # the old vertices keep their numbers and places; the new ones are edge midpoints
    assert np.array_equal(r.coords[:m.nv], m.coords)
    r2 = M.refine_uniform(r)
    _check_conforming(r2)
    q0 = (_measure(m) / _measure(m).max()).min()
    q2 = (_measure(r2) / _measure(r2).max()).min()
    assert q2 >= 0.5 * q0
    # netgen's in-place form
    m.Refine()
    assert m.ne == r.ne and np.array_equal(m.elements, r.elements)


def test_rates_and_table():
    errs = [1e-2, 1e-2 / 16, 1e-2 / 256]
    assert np.allclose(PP.h_rates([10, 40, 160], errs, 2), [4.0, 4.0])
    assert np.allclose(PP.h_rates([10, 80, 640], errs, 3), [4.0, 4.0])
    assert np.allclose(PP.p_rates([10, 20], [1.0, 0.25]), [2.0])
    rows = [['Refinement Level', 'Mesh Elements', 'Error', 'Convergence Rate'], [1, 10, 1e-2, 0], ['1/2', 40, 6.25e-4, 4.0]]
    t = PP.format_table(rows, ('.1f', '.1f', '.3e', '.2f'))
    assert 'Convergence Rate' in t and '6.250e-04' in t and '4.00' in t


def test_convergence_test_keys():
    cfg = ConfigParser(os.path.join(FIX, 'poisson_h_convergence', 'config'))
    assert PP._tests(cfg) == {'h': ['u']}
    assert cfg.get_item(['ERROR ANALYSIS', 'num_refinements'], int) == 5
    cfg.remove_option('ERROR ANALYSIS', 'convergence_test')
    assert PP._tests(cfg) == {}


@pytest.mark.gpu
@pytest.mark.parametrize('dg', [False, True], ids=['cg', 'dg'])
def test_reference_h_convergence_through_run(gpu_lib, capsys, dg):
    """The reference's test_h_convergence_{cg,dg} (pytests/full_system/poisson/test_poisson.py:46-54)
    prints this table for a person to read; here its rates are checked: the last two refinements
    reach at least 3.5 (order 3: the L2 error falls like h^4)."""
    from opencmp_gb300.run import run
    cfg = ConfigParser(os.path.join(FIX, 'poisson_h_convergence', 'config'))
    cfg['MESH']['filename'] = os.path.join(GOLDEN, 'unit_square_coarse.npz')
    cfg['OTHER']['run_dir'] = os.path.join(FIX, 'poisson_h_convergence')
    cfg['DG']['DG'] = str(dg)
    run('', cfg)
    out = capsys.readouterr().out.strip().split('\n')
    errs = [float(l.split(': ')[1]) for l in out if l.startswith('L2 norm at refinement')]
    assert len(errs) == 5
    assert any('Convergence Rate' in l for l in out)
    n = [6 * 4 ** k for k in range(6)]
    assert n[-1] == 6144
    rates = [math.log(errs[k] / errs[k + 1]) / math.log(2) for k in range(len(errs) - 1)]
    assert min(rates[-2:]) >= 3.5, (errs, rates)
