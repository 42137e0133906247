"""Generates the golden fixtures under tests/golden/ from the OpenCMP reference tree.

Run in a container where the reference is mounted (default path /root/reference, or pass it as
the first argument). The reference's Python package cannot be imported there (NGSolve and
pyparsing are absent), so the fixtures are its test inputs and pinned numbers, read as data:

* unit_square_coarse.npz - pytests/mesh_files/unit_square_coarse.vol (the mesh both the
  transient Poisson and the MultiComponentINS diffusion-convection tests run on), parsed by
  opencmp_gb300.mesh.load_mesh;
* reference_bounds.json  - the error bounds those tests assert (automated_output_check compares
  with isclose(rtol=3, atol=1e-12), opencmp/helpers/testing.py:58-86), with their file:line.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from opencmp_gb300.mesh import load_mesh  # noqa: E402


def main(ref='/root/reference'):
    m = load_mesh(os.path.join(ref, 'pytests/mesh_files/unit_square_coarse.vol'))
    np.savez(os.path.join(HERE, 'unit_square_coarse.npz'), coords=m.coords, elements=m.elements,
             bfacets=m.bfacets, blabels=m.blabels, bc_names=np.array(m.bc_names))
    bounds = {}
    tp = os.path.join(ref, 'pytests/full_system/poisson/test_poisson.py')
    src = open(tp).read().splitlines()
    for i, ln in enumerate(src):
        if 'def test_implicit_euler_cg' in ln:
            for k in range(i, i + 8):
                mm = re.search(r'automated_output_check\(capsys, \w+, \[([^\]]+)\]\)', src[k])
                if mm:
                    bounds['poisson_transient_implicit_euler_cg'] = {
                        'bounds': [float(v) for v in mm.group(1).split(',')],
                        'source': 'pytests/full_system/poisson/test_poisson.py:{}'.format(k + 1),
                        'config': 'pytests/full_system/poisson/transient_coarse/config'}
                    break
    tm = os.path.join(ref, 'pytests/full_system/mcins/test_mcins.py')
    src = open(tm).read().splitlines()
    for i, ln in enumerate(src):
        if 'class TestDiffusionConvection' in ln:
            for k in range(i, i + 8):
                mm = re.search(r'expected_errors = \[([^\]]+)\]', src[k])
                if mm:
                    bounds['mcins_diffusion_convection_implicit_euler_cg'] = {
                        'bounds': [float(v) for v in mm.group(1).split(',')],
                        'source': 'pytests/full_system/mcins/test_mcins.py:{}'.format(k + 1),
                        'config': 'pytests/full_system/mcins/diffusion_convection/config'}
                    break
            break
    bounds['rtol'] = {'value': 3.0, 'atol': 1e-12, 'source': 'opencmp/helpers/testing.py:82'}
    with open(os.path.join(HERE, 'reference_bounds.json'), 'w') as fh:
        json.dump(bounds, fh, indent=1)
    print(json.dumps(bounds, indent=1))


if __name__ == '__main__':
    main(*sys.argv[1:])
