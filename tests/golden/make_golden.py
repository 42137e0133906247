"""Generates the golden fixtures under tests/golden/ from the OpenCMP reference tree.

Run where the OpenCMP source tree is available: pass its path as the first argument, or set
OPENCMP_REFERENCE. The reference's Python package cannot be imported there (NGSolve and
pyparsing are absent), so the fixtures are its test inputs and pinned numbers, read as data:

* unit_square_coarse.npz - pytests/mesh_files/unit_square_coarse.vol (the mesh both the
  transient Poisson and the MultiComponentINS diffusion-convection tests run on), parsed by
  opencmp_gb300.mesh.load_mesh;
* reference_bounds.json  - the error bounds those tests assert (automated_output_check compares
  with isclose(rtol=3, atol=1e-12), opencmp/helpers/testing.py:58-86), with their file:line;
* square.npz, coarse_large_square_4bcs.npz - pytests/mesh_files/square.msh (the purely convective
  MCINS test's mesh) and coarse_large_square_4bcs.vol (the transient INS test's);
* fixtures/<group>_<case>/ - the run directories of the full-system tests the GPU path runs
  (config plus bc/ic/model/ref_sol sub-configs), copied as data; restart_transient_poisson is the
  run directory of the restart test (pytests/full_system/restart/test_restart.py). The tests point their mesh file
  and run_dir at this tree before running them.
"""
import ast
import json
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from opencmp_gb300.mesh import load_mesh  # noqa: E402


FIXTURES = ['poisson/transient_coarse', 'poisson/h_convergence', 'mcins/diffusion', 'mcins/diffusion_convection',
            'mcins/purely_convective', 'mcins/0th_rxn', 'mcins/1st_rxn', 'mcins/1st_rxn_coupled',
            'ins/sinusoidal_transient', 'restart/transient_poisson']
MESHES = ['unit_square_coarse.vol', 'square.msh', 'coarse_large_square_4bcs.vol']


def main(ref=None):
    ref = ref or os.environ.get('OPENCMP_REFERENCE')
    if not ref:
        raise SystemExit('usage: make_golden.py <path of the OpenCMP source tree> (or set OPENCMP_REFERENCE)')
    m = load_mesh(os.path.join(ref, 'pytests/mesh_files/unit_square_coarse.vol'))
    np.savez(os.path.join(HERE, 'unit_square_coarse.npz'), coords=m.coords, elements=m.elements,
             bfacets=m.bfacets, blabels=m.blabels, bc_names=np.array(m.bc_names))
    for name in MESHES[1:]:
        m = load_mesh(os.path.join(ref, 'pytests/mesh_files', name))
        np.savez(os.path.join(HERE, os.path.splitext(name)[0] + '.npz'), coords=m.coords, elements=m.elements,
                 bfacets=m.bfacets, blabels=m.blabels, bc_names=np.array(m.bc_names))
    for case in FIXTURES:
        src = os.path.join(ref, 'pytests/full_system', case)
        dst = os.path.join(HERE, 'fixtures', case.replace('/', '_'))
        os.makedirs(dst, exist_ok=True)
        shutil.copyfile(os.path.join(src, 'config'), os.path.join(dst, 'config'))
        for sub in ('bc', 'ic', 'model', 'ref_sol'):
            f = os.path.join(src, sub + '_dir', sub + '_config')
            if os.path.isfile(f):
                os.makedirs(os.path.join(dst, sub + '_dir'), exist_ok=True)
                shutil.copyfile(f, os.path.join(dst, sub + '_dir', sub + '_config'))
    bounds = {'rtol': {'value': 3.0, 'atol': 1e-12, 'source': 'opencmp/helpers/testing.py:82'},
              'tests': []}
    for tf in ('pytests/full_system/poisson/test_poisson.py', 'pytests/full_system/mcins/test_mcins.py',
               'pytests/full_system/ins/test_ins.py'):
        bounds['tests'] += reference_tests(ref, tf)
    with open(os.path.join(HERE, 'reference_bounds.json'), 'w') as fh:
        json.dump(bounds, fh, indent=1)
    print(json.dumps(bounds, indent=1))


def _const(node):
    return ast.literal_eval(node)


def reference_tests(ref, rel):
    """Every (uncommented) test of a full-system test file whose fixture is one of FIXTURES: the
    config overrides it applies, the error bounds it asserts, and its file:line."""
    src = open(os.path.join(ref, rel)).read()
    tree = ast.parse(src)
    fixtures = {}
    for node in tree.body:
        if isinstance(node, ast.FunctionDef):
            for sub in ast.walk(node):
                if isinstance(sub, ast.Call) and getattr(sub.func, 'id', '') == 'ConfigParser' and sub.args:
                    path = _const(sub.args[0])
                    case = os.path.dirname(path).replace('pytests/full_system/', '')
                    if case in FIXTURES:
                        fixtures[node.name] = case.replace('/', '_')
    out = []
    for cls in tree.body:
        if not isinstance(cls, ast.ClassDef):
            continue
        for fn in cls.body:
            if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith('test_'):
                continue
            args = [a.arg for a in fn.args.args]
            fx = [fixtures[a] for a in args if a in fixtures]
            if not fx:
                continue
            overrides, expected = {}, None
            for st in fn.body:
                if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Subscript):
                    t = st.targets[0]
                    key, sec = _const(t.slice), _const(t.value.slice)
                    overrides.setdefault(sec, {})[key] = _const(st.value)
                elif isinstance(st, ast.Assign) and getattr(st.targets[0], 'id', '') == 'expected_errors':
                    expected = _const(st.value)
                elif isinstance(st, ast.Expr) and isinstance(st.value, ast.Call) and \
                        getattr(st.value.func, 'id', '') == 'automated_output_check':
                    a = st.value.args[2]
                    if isinstance(a, ast.List):
                        expected = _const(a)
            if expected is None:
                continue
            out.append({'id': '{}::{}::{}'.format(os.path.basename(rel), cls.name, fn.name), 'fixture': fx[0],
                        'overrides': overrides, 'bounds': expected,
                        'source': '{}:{}'.format(rel, fn.lineno)})
    return out


if __name__ == '__main__':
    main(*sys.argv[1:])
