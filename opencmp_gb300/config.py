"""OpenCMP configuration files, read without pyparsing or NGSolve.

:class:`ConfigParser` keeps the interface of ``opencmp/config_functions/expanded_config_parser.py``
(``get_item``, ``get_list``, ``get_dict`` with the defaults table of lines 26-90 and ``REQUIRED``
markers). Values are infix expressions in x, y, z, t with the function set of
``opencmp/config_functions/parse_arithmetic.py:153-177`` (sin, cos, tan, exp, tanh, sig, H, abs,
trunc, round, sqrt, sgn, vec, ramp) and the constants pi and e; ``[a, b]`` builds a vector. Here an
expression becomes an :class:`Expr`, a callable evaluated with numpy on an array of points
``X`` (N x dim) at time ``t``; the GPU path samples it at quadrature points or dofs.
"""
from __future__ import annotations

import configparser
import math
import os
import re
from typing import Any, Dict, List, Optional

import numpy as np

CONFIG_DEFAULTS: Dict[str, Dict[str, Any]] = {
    'MESH': {'filename': 'REQUIRED', 'curved_elements': False},
    'FINITE ELEMENT SPACE': {'elements': 'REQUIRED', 'interpolant_order': 'REQUIRED', 'no_constrained_dofs': False},
    'DG': {'DG': False, 'interior_penalty_coefficient': 10.0},
    'SOLVER': {'linear_solver': 'default', 'preconditioner': 'default', 'linear_tolerance': 1e-15,
               'linear_max_iterations': 100, 'linearization_method': 'Oseen', 'nonlinear_solver': 'default',
               'nonlinear_tolerance': {'absolute': 0.0, 'relative': 'REQUIRED'}, 'nonlinear_max_iterations': 10,
               # GPU path (new keys; absent from OpenCMP's table)
               'gpu_precision': 'fp64', 'gpu_restart': 50, 'initial_guess': 'previous',
               'learned_train_steps': 20, 'learned_train_iters': 300},
    'TRANSIENT': {'transient': False, 'scheme': 'implicit euler', 'time_range': [0.0, 5.0], 'dt': 0.001,
                  'dt_tolerance': {'absolute': 0.0, 'relative': 'REQUIRED'}, 'dt_range': [1e-6, 0.1],
                  'maximum_rejected_solves': 1000},
    'ERROR ANALYSIS': {'check_error': False, 'check_error_every_timestep': False, 'save_error_every_timestep': False,
                       'convergence_test': {'h': False, 'p': False}, 'error_average': [], 'num_refinements': 4},
    'OTHER': {'num_threads': 1, 'messaging_level': 0, 'model': 'REQUIRED', 'component_names': [],
              'parameter_names': [], 'velocity_fixed': False, 'run_dir': 'REQUIRED', 'resume_from_previous': False,
              'restart_from': ''},
    'VISUALIZATION': {'save_to_file': False, 'save_type': '.sol', 'save_frequency': ['1', 'numit'],
                      'subdivision': -1, 'split_components': False},
    'DIM': {'diffuse_interface_method': False},
    'CONTROLLER': {'active': False},
}

# --------------------------------------------------------------------------------------------------
# expressions


def _sig(a):
    return 1.0 / (1.0 + np.exp(-a))


def _tanh(a):
    a = np.minimum(a, 350.0)
    return (np.exp(2 * a) - 1.0) / (np.exp(2 * a) + 1.0)


def _heaviside(a, w=0.1):
    shift = 9.21025
    return _sig((2 * shift) / w * a - shift)


def _ramp(t, p1=0.0, p2=1.0, tr=1.0):
    return np.where(tr - t > 0, 0.5 * (p1 - p2) * np.cos(t * math.pi / tr) + 0.5 * (p1 + p2), p2)


def _sgn(a, eps=1e-12):
    return np.where(a < -eps, -1.0, np.where(a > eps, 1.0, 0.0))


# IMPORT(name) (opencmp/config_functions/parse_arithmetic.py:105, 238-256): the function `name` of
# the run directory's import_functions.py, called as OpenCMP calls it, f(t_param, new_variables,
# mesh, time_step), with t_param the list [t]. OpenCMP's functions return NGSolve coefficient
# functions; here the result is a number, an array over the points, or a callable f(X) or f(X, t)
# evaluated at the points X (N x dim). The run directory is the one whose configuration is being
# read (set_import_dir).
_IMPORT_DIR: Optional[str] = None
_IMPORTED: Dict[str, Any] = {}


def set_import_dir(path: Optional[str]) -> None:
    """Directory whose import_functions.py IMPORT(...) expressions read (the run directory)."""
    global _IMPORT_DIR
    _IMPORT_DIR = path


def _imported(name: str, import_dir: Optional[str]):
    if import_dir is None:
        raise ValueError('IMPORT({}): no run directory to import from'.format(name))
    path = os.path.join(import_dir, 'import_functions.py')
    mod = _IMPORTED.get(path)
    if mod is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location('import_functions_{}'.format(len(_IMPORTED)), path)
        if spec is None or not os.path.isfile(path):
            raise FileNotFoundError('IMPORT({}): {} not found'.format(name, path))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        _IMPORTED[path] = mod
    fn = getattr(mod, name)
    if not callable(fn):
        raise TypeError('IMPORT({}): not a function'.format(name))
    return fn


def _import_value(fn, X, t):
    v = fn([t], [{}], None, None)
    if callable(v):
        import inspect
        try:
            nargs = len(inspect.signature(v).parameters)
        except (TypeError, ValueError):
            nargs = 2
        v = v(X, t) if nargs >= 2 else v(X)
    return v


FUNCS = {'sin': np.sin, 'cos': np.cos, 'tan': np.tan, 'exp': np.exp, 'tanh': _tanh, 'sig': _sig, 'H': _heaviside,
         'abs': np.abs, 'trunc': np.trunc, 'round': np.round, 'sqrt': np.sqrt, 'sgn': _sgn, 'ramp': _ramp}
CONSTS = {'pi': math.pi, 'e': math.e}
_TOKEN = re.compile(r'\s*(?:(\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?)|([A-Za-z_][A-Za-z_0-9]*)|(\S))')


class Expr:
    """A parsed expression; ``expr(X, t)`` evaluates it at the points X (N x dim) and time t."""

    def __init__(self, text: str):
        self.text = text.strip()
        self._toks = [(m.group(1), m.group(2), m.group(3)) for m in _TOKEN.finditer(self.text) if any(m.groups())]
        self._pos = 0
        self._imports: List[Any] = []
        self.mvars: set = set()
        self.ast = self._expr()
        if self._pos != len(self._toks):
            raise ValueError('cannot parse expression: {!r}'.format(text))

    # recursive descent: expr := term (('+'|'-') term)*; term := factor (('*'|'/') factor)*;
    # factor := unary ('^' factor)?; unary := ('+'|'-')* atom
    def _peek(self):
        return self._toks[self._pos] if self._pos < len(self._toks) else (None, None, None)

    def _take(self, op=None):
        t = self._peek()
        if op is not None and t[2] != op:
            raise ValueError('expected {!r} in {!r}'.format(op, self.text))
        self._pos += 1
        return t

    def _expr(self):
        node = self._term()
        while self._peek()[2] in ('+', '-'):
            op = self._take()[2]
            node = (op, node, self._term())
        return node

    def _term(self):
        node = self._factor()
        while self._peek()[2] in ('*', '/'):
            op = self._take()[2]
            node = (op, node, self._factor())
        return node

    def _factor(self):
        node = self._unary()
        if self._peek()[2] == '^':
            self._take()
            node = ('^', node, self._factor())
        return node

    def _unary(self):
        sign = 1
        while self._peek()[2] in ('+', '-'):
            if self._take()[2] == '-':
                sign = -sign
        node = self._atom()
        return ('neg', node) if sign < 0 else node

    def _args(self, close):
        args = [self._expr()]
        while self._peek()[2] == ',':
            self._take()
            args.append(self._expr())
        self._take(close)
        return args

    def _atom(self):
        num, name, op = self._take()
        if num is not None:
            return ('num', float(num))
        if op == '(':
            node = self._expr()
            self._take(')')
            return node
        if op == '[':
            return ('vec', self._args(']'))
        if name is not None:
            if name == 'IMPORT' and self._peek()[2] == '(':
                self._take()
                _, fname, _ = self._take()
                self._take(')')
                if fname is None:
                    raise ValueError('IMPORT takes the name of a function: {!r}'.format(self.text))
                fn = _imported(fname, _IMPORT_DIR)
                self._imports.append(fn)
                return ('import', fn)
            if self._peek()[2] == '(':
                self._take()
                args = self._args(')')
                if name == 'vec':
                    return ('vec', args)
                if name not in FUNCS:
                    raise ValueError('unknown function {!r}'.format(name))
                return ('call', name, args)
            if name in ('x', 'y', 'z', 't'):
                return ('var', name)
            if name in CONSTS:
                return ('num', CONSTS[name])
            # any other name is a model variable (a component of the model's solution, e.g. the
            # concentration `a` in a reaction source `-1*a`): its value is supplied at evaluation
            self.mvars.add(name)
            return ('mvar', name)
        raise ValueError('cannot parse expression: {!r}'.format(self.text))

    def _eval(self, node, X, t, vals=None):
        k = node[0]
        if k == 'num':
            return node[1]
        if k == 'mvar':
            if vals is None or node[1] not in vals:
                raise ValueError('{!r} reads the model variable {!r}, which has no value here'.format(self.text, node[1]))
            return vals[node[1]]
        if k == 'var':
            if node[1] == 't':
                return t
            c = 'xyz'.index(node[1])
            return X[..., c] if X is not None and c < X.shape[-1] else 0.0
        if k == 'neg':
            return -self._eval(node[1], X, t, vals)
        if k == 'import':
            return _import_value(node[1], X, t)
        if k == 'call':
            return FUNCS[node[1]](*[self._eval(a, X, t, vals) for a in node[2]])
        if k == 'vec':
            return [self._eval(a, X, t, vals) for a in node[1]]
        a, b = self._eval(node[1], X, t, vals), self._eval(node[2], X, t, vals)
        return {'+': np.add, '-': np.subtract, '*': np.multiply, '/': np.divide, '^': np.power}[k](a, b)

    @property
    def is_vector(self) -> bool:
        return self.ast[0] == 'vec'

    @property
    def depends_on_space(self) -> bool:
        if re.search(r'\b[xyz]\b', self.text) is not None:
            return True
        # an imported function depends on space unless it returns a number
        return any(not np.isscalar(fn([0.0], [{}], None, None)) for fn in self._imports)

    def __call__(self, X=None, t=0.0, vals=None):
        """The value at the points X (N x dim, or None) and time t; `vals` gives the model
        variables the expression reads ({name: value})."""
        v = self._eval(self.ast, X, t, vals)
        if isinstance(v, list):
            n = X.shape[0] if X is not None else 1
            return np.stack([np.broadcast_to(np.asarray(c, np.float64), (n,)) for c in v], axis=-1)
        if X is not None:
            return np.broadcast_to(np.asarray(v, np.float64), X.shape[:-1]).copy()
        return float(v)

    def __repr__(self):
        return 'Expr({!r})'.format(self.text)


def parse(text: str) -> Any:
    """Parse a config value: booleans, None, numbers and expressions (as :class:`Expr`)."""
    s = text.strip()
    if s in ('True', 'False'):
        return s == 'True'
    if s == 'None':
        return None
    try:
        return float(s)
    except ValueError:
        return Expr(s)


# --------------------------------------------------------------------------------------------------
# configuration files


class ConfigParser(configparser.ConfigParser):
    """OpenCMP's ConfigParser interface over plain ``configparser``."""

    def __init__(self, config_file_path: Optional[str] = None):
        super().__init__()
        self.optionxform = str  # keys are case-sensitive, as in OpenCMP's files
        self.path = config_file_path
        if config_file_path is not None:
            if not os.path.isfile(config_file_path):
                raise FileNotFoundError('The given config file "{}" does not exist.'.format(config_file_path))
            self.read(config_file_path)

    @classmethod
    def from_parser(cls, other: configparser.ConfigParser) -> 'ConfigParser':
        """A copy of another configparser's sections (e.g. OpenCMP's own ConfigParser)."""
        c = cls()
        for sec in other.sections():
            c[sec] = {k: v for k, v in other.items(sec, raw=True)}
        c.path = getattr(other, 'path', None)
        return c

    def _raw(self, keys: List[str]):
        sec, key = keys[0], keys[1]
        if self.has_option(sec, key):
            return self.get(sec, key)
        default = CONFIG_DEFAULTS.get(sec, {}).get(key, 'REQUIRED')
        if default == 'REQUIRED':
            raise ValueError('{} {} is required in the config file'.format(sec, key))
        return default

    def get_item(self, keys: List[str], val_type=str, quiet: bool = False):
        v = self._raw(keys)
        if not isinstance(v, str):
            return v if val_type is None or isinstance(v, val_type) else val_type(v)
        v = v.strip()
        if val_type is bool:
            return v == 'True'
        return val_type(v)

    def get_list(self, keys: List[str], val_type=str, quiet: bool = False) -> List:
        v = self._raw(keys)
        if isinstance(v, list):
            return [val_type(x) for x in v]
        return [val_type(x.strip()) for x in v.split(',') if x.strip()]

    def get_dict(self, keys: List[str], quiet: bool = False, all_str: bool = False) -> Dict[str, Any]:
        """``a -> v1`` lines (continuation lines allowed) into {'a': parsed v1, ...}."""
        v = self._raw(keys)
        if isinstance(v, dict):
            return dict(v)
        out = {}
        for ln in v.splitlines():
            if '->' not in ln:
                continue
            k, val = ln.split('->', 1)
            out[k.strip()] = val.strip() if all_str else parse(val)
        return out

    def sections_dict(self) -> Dict[str, Dict[str, str]]:
        return {s: dict(self.items(s)) for s in self.sections()}


def load_sub_config(run_dir: str, sub: str) -> Optional[ConfigParser]:
    """The ``<run_dir>/<sub>_dir/<sub>_config`` files of a run (bc, ic, model, ref_sol)."""
    path = os.path.join(run_dir, '{}_dir'.format(sub), '{}_config'.format(sub))
    return ConfigParser(path) if os.path.isfile(path) else None


def value_map(cfg: ConfigParser, section: str) -> Dict[str, Dict[str, Any]]:
    """{variable: {marker: parsed value}} for every key of a section written as ``marker -> value``
    lines; a bare value maps to the marker 'all'."""
    out = {}
    if cfg is None or not cfg.has_section(section):
        return out
    for var, raw in cfg.items(section):
        d = {}
        if '->' in raw:
            for ln in raw.splitlines():
                if '->' in ln:
                    k, val = ln.split('->', 1)
                    d[k.strip()] = parse(val)
        elif raw.strip():
            d['all'] = parse(raw)
        out[var] = d
    return out
