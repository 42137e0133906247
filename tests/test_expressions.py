"""Config expressions: IMPORT(name) (opencmp/config_functions/parse_arithmetic.py:105, 238-256) reads
`name` from the run directory's import_functions.py and calls it as OpenCMP does,
f(t_param, new_variables, mesh, time_step); here the result is a number, an array over the points, or
a callable of the points (and time) evaluated there. CPU only."""
import os

import numpy as np
import pytest

from opencmp_gb300.config import parse, set_import_dir


@pytest.fixture
def import_dir(tmp_path):
    with open(os.path.join(str(tmp_path), 'import_functions.py'), 'w') as fh:
        fh.write(
            'import numpy as np\n\n'
            'def coefficient(t_param, new_variables, mesh, time_step):\n'
            '    return 2.5\n\n'
            'def source(t_param, new_variables, mesh, time_step):\n'
            '    return lambda X, t: X[..., 0] ** 2 + t\n\n'
            'def wave(t_param, new_variables, mesh, time_step):\n'
            '    return lambda X: np.sin(np.pi * X[..., 1])\n')
    set_import_dir(str(tmp_path))
    yield str(tmp_path)
    set_import_dir(None)


def test_import_constant(import_dir):
    e = parse('2 * IMPORT(coefficient) + 1')
    assert not e.depends_on_space
    assert float(e(None, 0.3)) == 6.0


def test_import_space_and_time(import_dir):
    X = np.array([[0.5, 0.25], [1.0, 0.5]])
    e = parse('IMPORT(source) - 1')
    assert e.depends_on_space
    assert np.allclose(e(X, 0.75), X[:, 0] ** 2 + 0.75 - 1)
    w = parse('[IMPORT(wave), 0]')
    assert np.allclose(w(X, 0.0), np.stack([np.sin(np.pi * X[:, 1]), np.zeros(2)], 1))


def test_import_errors(tmp_path):
    set_import_dir(str(tmp_path))
    try:
        with pytest.raises(FileNotFoundError):
            parse('IMPORT(missing)')
    finally:
        set_import_dir(None)
    with pytest.raises(ValueError):
        parse('IMPORT(source)')          # no run directory
