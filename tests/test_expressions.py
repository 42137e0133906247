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


def test_model_variables_in_expressions():
    """A source such as `-5*a + 0.9*5*b` reads the model's variables: parsed as such, evaluated
    with their values, and split into the part without them and constant coefficients
    (OpenCMP puts the part that reads the unknowns into the bilinear form)."""
    from opencmp_gb300.models import affine_parts
    e = parse('-5*a + 0.9*5*b + 2*x')
    assert e.mvars == {'a', 'b'}
    X = np.array([[0.5, 0.0], [0.25, 1.0]])
    assert np.allclose(e(X, 0.0, {'a': 1.0, 'b': 2.0}), -5 + 9 + 2 * X[:, 0])
    with pytest.raises(ValueError):
        e(X, 0.0)                                      # no values for a, b
    f0, ks = affine_parts(e, ['a', 'b', 'c'], X, 0.0)
    assert np.allclose(f0, 2 * X[:, 0]) and ks == pytest.approx({'a': -5.0, 'b': 4.5})
    with pytest.raises(NotImplementedError):
        affine_parts(parse('a*b'), ['a', 'b'], X, 0.0)  # not affine
    with pytest.raises(NotImplementedError):
        affine_parts(parse('x*a'), ['a'], X, 0.0)       # coefficient varies in space
    with pytest.raises(NotImplementedError):
        affine_parts(parse('q + 1'), ['a'], X, 0.0)     # not a model variable here
