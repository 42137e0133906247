"""ctypes wrapper of the C oracle (oracle.c).  TEST INFRASTRUCTURE ONLY.

Only the tests, the smoke check and the CPU-baseline leg of bench.py import this module; the
product package never does.  ``build()`` compiles ``oracle.c`` with gcc/OpenMP into
``oracle/_build/liboracle.so``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD, 'liboracle.so')

H1, L2 = 0, 1
WIND_NONE, WIND_CONST, WIND_VERTEX = 0, 1, 2
SRC_NONE, SRC_CONST, SRC_SINPROD, SRC_GAUSS, SRC_POLY_X1MX = 0, 1, 2, 3, 4


def build(force: bool = False) -> str:
    src = os.path.join(HERE, 'oracle.c')
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, 'oracle.h'))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    subprocess.check_call(['gcc', '-O2', '-fopenmp', '-fPIC', '-shared', '-o', LIB, src, '-lm'])
    return LIB


class Form(C.Structure):
    _fields_ = [('mass', C.c_double), ('diff', C.c_double), ('dt', C.c_double), ('wind_kind', C.c_int),
                ('wind', C.c_double * 3), ('wind_vtx', C.c_void_p), ('ipc', C.c_double), ('dg', C.c_int),
                ('outflow_mask', C.c_uint32), ('wn_mask', C.c_uint32), ('nitsche_mask', C.c_uint32),
                ('robin_mask', C.c_uint32), ('robin', C.c_double * 32)]


class Rhs(C.Structure):
    _fields_ = [('dt', C.c_double), ('src_kind', C.c_int), ('src', C.c_double * 8), ('mass', C.c_double),
                ('uprev', C.c_void_p), ('bval', C.c_double * 32), ('bval_mask', C.c_uint32),
                ('gval', C.c_double * 32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.or_space_create.restype = P
        L.or_space_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, P, C.c_int64, P, C.c_int64, P, P,
                                      C.c_uint32]
        for nm in ('or_space_ndof', 'or_space_nnz', 'or_space_ninterior_facets'):
            getattr(L, nm).restype = C.c_int64
            getattr(L, nm).argtypes = [P]
        L.or_space_nloc.restype = C.c_int
        L.or_space_nloc.argtypes = [P]
        for nm in ('or_space_get_dofs', 'or_space_get_sorted_conn', 'or_space_get_free'):
            getattr(L, nm).argtypes = [P, P]
        L.or_space_get_pattern.argtypes = [P, P, P]
        L.or_space_destroy.argtypes = [P]
        L.or_assemble_matrix.argtypes = [P, C.POINTER(Form), P]
        L.or_assemble_rhs.argtypes = [P, C.POINTER(Form), C.POINTER(Rhs), P]
        L.or_element_matrix.argtypes = [P, C.POINTER(Form), C.c_int64, P]
        L.or_set_boundary.argtypes = [P, C.c_uint32, P, P]
        L.or_project.argtypes = [P, C.c_int, P, P]
        L.or_l2_error.restype = C.c_double
        L.or_l2_error.argtypes = [P, P, C.c_int, P]
        L.or_cg.argtypes = [P, P, P, P, C.c_double, C.c_int, P, P]
        L.or_gmres.argtypes = [P, P, P, P, C.c_int, C.c_int, C.c_double, C.c_int, P, P]
        L.or_relres.restype = C.c_double
        L.or_relres.argtypes = [P, P, P, P]
        L.or_spmv.argtypes = [C.c_int64, P, P, P, P, P]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_tabulate.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, P, P, P]
        L.or_rule.argtypes = [C.c_int, C.c_int, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def make_form(mass=0.0, diff=0.0, dt=1.0, wind=None, wind_vtx=None, ipc=10.0, dg=False,
              outflow_mask=0, wn_mask=0, nitsche_mask=0, robin=None):
    f = Form()
    f.mass, f.diff, f.dt, f.ipc, f.dg = mass, diff, dt, ipc, int(dg)
    f.outflow_mask, f.wn_mask, f.nitsche_mask = outflow_mask, wn_mask, nitsche_mask
    for lab, c in (robin or {}).items():
        f.robin_mask |= 1 << lab
        f.robin[lab] = c
    f._keep = None
    if wind_vtx is not None:
        wv = np.ascontiguousarray(wind_vtx, np.float64)
        f.wind_kind, f.wind_vtx, f._keep = WIND_VERTEX, wv.ctypes.data, wv
    elif wind is not None:
        f.wind_kind = WIND_CONST
        for k, w in enumerate(wind):
            f.wind[k] = w
    return f


def make_rhs(dt=1.0, src_kind=SRC_NONE, src=(), mass=0.0, uprev=None, bval=None, gval=None):
    r = Rhs()
    r.dt, r.src_kind, r.mass = dt, src_kind, mass
    for k, v in enumerate(src):
        r.src[k] = v
    r._keep = None
    if uprev is not None:
        u = np.ascontiguousarray(uprev, np.float64)
        r.uprev, r._keep = u.ctypes.data, u
    if bval:
        for lab, v in bval.items():
            r.bval[lab] = v
            r.bval_mask |= 1 << lab
    if gval:
        for lab, v in gval.items():
            r.gval[lab] = v
    return r


def tabulate(D: int, kind: int, p: int, xi):
    """Reference basis values (npts, L) and reference gradients (npts, L, D) at the points xi."""
    xi = np.ascontiguousarray(xi, np.float64).reshape(-1, D)
    L = (p + 1) * (p + 2) // 2 if D == 2 else (p + 1) * (p + 2) * (p + 3) // 6
    v = np.empty((xi.shape[0], L))
    g = np.empty((xi.shape[0], L, D))
    lib().or_tabulate(D, kind, p, xi.shape[0], _p(xi), _p(v), _p(g))
    return v, g


def rule(D: int, n: int):
    """The collapsed simplex rule with n points per direction: (points (n^D, D), weights)."""
    x = np.empty((n ** D, D))
    w = np.empty(n ** D)
    lib().or_rule(D, n, _p(x), _p(w))
    return x, w


class Space:
    """Oracle finite-element space on a mesh (H1 order 1..3, L2 order 1..3 on triangles)."""

    def __init__(self, mesh, kind: int, order: int, dirichlet_mask: int = 0):
        L = lib()
        self.mesh = mesh
        self._c = np.ascontiguousarray(mesh.coords, np.float64)
        self._e = np.ascontiguousarray(mesh.elements, np.int32)
        self._bf = np.ascontiguousarray(mesh.bfacets, np.int32)
        self._bl = np.ascontiguousarray(mesh.blabels, np.int32)
        self.h = L.or_space_create(mesh.dim, kind, order, mesh.nv, _p(self._c), mesh.ne, _p(self._e),
                                   self._bf.shape[0], _p(self._bf), _p(self._bl), dirichlet_mask)
        if not self.h:
            raise ValueError('oracle: unsupported space')
        self.kind, self.order, self.dim = kind, order, mesh.dim
        self.ndof = L.or_space_ndof(self.h)
        self.nnz = L.or_space_nnz(self.h)
        self.nloc = L.or_space_nloc(self.h)

    def __del__(self):
        if getattr(self, 'h', None):
            lib().or_space_destroy(self.h)
            self.h = None

    def dofs(self):
        d = np.empty((self.mesh.ne, self.nloc), np.int32)
        lib().or_space_get_dofs(self.h, _p(d))
        return d

    def sorted_conn(self):
        d = np.empty((self.mesh.ne, self.dim + 1), np.int32)
        lib().or_space_get_sorted_conn(self.h, _p(d))
        return d

    def pattern(self):
        rp = np.empty(self.ndof + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        lib().or_space_get_pattern(self.h, _p(rp), _p(col))
        return rp, col

    def freedofs(self):
        f = np.empty(self.ndof, np.uint8)
        lib().or_space_get_free(self.h, _p(f))
        return f.astype(bool)

    def assemble(self, form):
        v = np.empty(self.nnz, np.float64)
        lib().or_assemble_matrix(self.h, C.byref(form), _p(v))
        return v

    def element_matrix(self, form, e):
        K = np.empty((self.nloc, self.nloc), np.float64)
        lib().or_element_matrix(self.h, C.byref(form), e, _p(K))
        return K

    def rhs(self, form, rhs):
        b = np.empty(self.ndof, np.float64)
        lib().or_assemble_rhs(self.h, C.byref(form), C.byref(rhs), _p(b))
        return b

    def set_boundary(self, mask, gvals, u):
        g = np.zeros(32, np.float64)
        for k, v in gvals.items():
            g[k] = v
        lib().or_set_boundary(self.h, mask, _p(g), _p(u))

    def project(self, src_kind, src=()):
        s = np.zeros(8, np.float64)
        s[:len(src)] = src
        u = np.zeros(self.ndof, np.float64)
        lib().or_project(self.h, src_kind, _p(s), _p(u))
        return u

    def l2_error(self, u, src_kind, src=()):
        s = np.zeros(8, np.float64)
        s[:len(src)] = src
        return lib().or_l2_error(self.h, _p(np.ascontiguousarray(u, np.float64)), src_kind, _p(s))

    def cg(self, vals, b, x, tol=1e-10, maxit=10000):
        it = C.c_int(0); rr = C.c_double(0)
        lib().or_cg(self.h, _p(vals), _p(b), _p(x), tol, maxit, C.byref(it), C.byref(rr))
        return it.value, rr.value

    def gmres(self, vals, b, x, restart=50, precond=1, tol=1e-10, maxit=10000):
        it = C.c_int(0); rr = C.c_double(0)
        lib().or_gmres(self.h, _p(vals), _p(b), _p(x), restart, precond, tol, maxit, C.byref(it), C.byref(rr))
        return it.value, rr.value

    def relres(self, vals, b, x):
        return lib().or_relres(self.h, _p(vals), _p(b), _p(x))

    def spmv(self, vals, x):
        rp, col = self.pattern()
        y = np.empty(self.ndof, np.float64)
        lib().or_spmv(self.ndof, _p(rp), _p(col), _p(vals), _p(np.ascontiguousarray(x, np.float64)), _p(y))
        return y

    def csr(self, vals):
        import scipy.sparse as sp
        rp, col = self.pattern()
        return sp.csr_matrix((vals, col, rp), shape=(self.ndof, self.ndof))
