import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')
    config.addinivalue_line('markers', 'slow: long-running')


@pytest.fixture(scope='session')
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope='session')
def coarse_mesh():
    from opencmp_gb300.mesh import load_mesh
    return load_mesh(os.path.join(ROOT, 'tests', 'golden', 'unit_square_coarse.npz'))


@pytest.fixture(scope='session')
def ref_bounds():
    import json
    with open(os.path.join(ROOT, 'tests', 'golden', 'reference_bounds.json')) as fh:
        d = json.load(fh)
    d['by_id'] = {t['id']: t for t in d['tests']}
    return d


@pytest.fixture(scope='session')
def gpu_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from opencmp_gb300 import build, _lib
    build.build()
    _lib.load()
    return _lib
