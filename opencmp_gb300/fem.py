"""Host-side handles over libopencmp_gpu.so: the GPU stand-ins for the NGSolve objects OpenCMP passes
around (mesh, finite-element space with ``FreeDofs``, assembled matrix, linear-form vector,
preconditioned Krylov solver).

Device arrays are torch tensors (``device='cuda'``); torch only owns memory and streams. All
arithmetic happens in the library's kernels.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional, Sequence

import numpy as np
import torch

from . import _lib as LB
from .mesh import Mesh


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, torch.Tensor):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def _stream(stream):
    if stream is None:
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, torch.cuda.Stream):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(stream)


class GPUMesh:
    """Device copy of a :class:`Mesh` (``ocmp_mesh_create``)."""

    def __init__(self, mesh: Mesh):
        self.mesh = mesh
        self._keep = [np.ascontiguousarray(mesh.coords, np.float64), np.ascontiguousarray(mesh.elements, np.int32),
                      np.ascontiguousarray(mesh.bfacets, np.int32), np.ascontiguousarray(mesh.blabels, np.int32)]
        h = C.c_void_p()
        c, e, bf, bl = self._keep
        LB.call('ocmp_mesh_create', _ptr(c), mesh.nv, mesh.dim, _ptr(e), mesh.ne, _ptr(bf), _ptr(bl),
                bf.shape[0], C.byref(h))
        self.h = h

    def __del__(self):
        if getattr(self, 'h', None) and LB._lib is not None:
            LB._lib.ocmp_mesh_destroy(self.h)
            self.h = None


class Space:
    """H1 (order 1..3, triangles/tetrahedra) or L2 (order 1..3, triangles) space on the GPU.

    ``dirichlet`` names boundary labels whose dofs are constrained (``FreeDofs`` excludes them).
    """

    def __init__(self, mesh: Mesh, kind: str = 'H1', order: int = 1, dirichlet: Sequence[str] | str = (),
                 gmesh: Optional[GPUMesh] = None):
        self.mesh = mesh
        self.gmesh = gmesh or GPUMesh(mesh)
        self.kind = LB.H1 if kind in ('H1', LB.H1) else LB.L2
        self.order = order
        self.dirichlet_mask = mesh.label_mask(dirichlet) if self.kind == LB.H1 else 0
        h = C.c_void_p()
        LB.call('ocmp_space_create', self.gmesh.h, self.kind, order, self.dirichlet_mask, C.byref(h))
        self.h = h
        info = LB.SpaceInfo()
        LB.call('ocmp_space_info', self.h, C.byref(info))
        self.info = info
        self.ndof, self.nnz, self.nloc, self.nq = info.ndof, info.nnz, info.nloc, info.nq
        self._free = None

    def __del__(self):
        if getattr(self, 'h', None) and LB._lib is not None:
            LB._lib.ocmp_space_destroy(self.h)
            self.h = None

    def dofs(self) -> np.ndarray:
        d = np.empty((self.mesh.ne, self.nloc), np.int32)
        LB.call('ocmp_space_get_dofs', self.h, _ptr(d))
        return d

    def pattern(self):
        rp = np.empty(self.ndof + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        LB.call('ocmp_space_get_pattern', self.h, _ptr(rp), _ptr(col))
        return rp, col

    def FreeDofs(self) -> np.ndarray:
        if self._free is None:
            f = np.empty(self.ndof, np.uint8)
            LB.call('ocmp_space_get_free', self.h, _ptr(f))
            self._free = f.astype(bool)
        return self._free

    def quad_points(self) -> np.ndarray:
        x = np.empty((self.mesh.ne, self.nq, self.mesh.dim), np.float64)
        LB.call('ocmp_space_quad_points', self.h, _ptr(x))
        return x

    def l2_error(self, u: torch.Tensor, f=None, stream=None) -> float:
        """||u_h - f||_L2; f a constant, a (ne, nq) tensor of quadrature-point values, or None (= 0)."""
        out = C.c_double(0)
        if isinstance(f, torch.Tensor):
            LB.call('ocmp_l2_error', self.h, _ptr(u), _ptr(f), 0.0, C.byref(out), _stream(stream))
        else:
            LB.call('ocmp_l2_error', self.h, _ptr(u), None, float(f or 0.0), C.byref(out), _stream(stream))
        return out.value

    def boundary_facets(self) -> np.ndarray:
        """(element, local facet, label) of each boundary facet, in the space's facet order."""
        out = np.empty((self.info.n_boundary_facets, 3), np.int32)
        LB.call('ocmp_space_boundary_facets', self.h, _ptr(out))
        return out

    def facet_quad_points(self) -> np.ndarray:
        """(nbf, nfq, dim) quadrature points of the boundary facets (where bval_fq/gval_fq are sampled)."""
        x = np.empty((self.info.n_boundary_facets, self.info.nfq, self.mesh.dim), np.float64)
        LB.call('ocmp_space_facet_quad_points', self.h, _ptr(x))
        return x

    def boundary_points(self, mask: int) -> np.ndarray:
        """Points at which space-dependent Dirichlet data on the labels of `mask` is sampled."""
        n = C.c_int64(0)
        LB.call('ocmp_boundary_points', self.h, mask, C.byref(n), None)
        x = np.empty((n.value, self.mesh.dim), np.float64)
        if n.value:
            LB.call('ocmp_boundary_points', self.h, mask, C.byref(n), _ptr(x))
        return x

    def set_boundary_values(self, mask: int, g: np.ndarray, u: torch.Tensor, stream=None):
        """Dirichlet dofs of u on the labels of `mask` from samples g at ``boundary_points(mask)``."""
        g = np.ascontiguousarray(g, np.float64)
        if g.size:
            LB.call('ocmp_set_boundary_values', self.h, mask, _ptr(g), _ptr(u), _stream(stream))

    def set_boundary(self, labels: Dict[int, float], u: torch.Tensor, mask: Optional[int] = None, stream=None):
        g = np.zeros(32, np.float64)
        m = 0
        for lab, v in labels.items():
            g[lab] = v
            m |= 1 << lab
        if mask is not None:
            m = mask
        LB.call('ocmp_set_boundary', self.h, m, _ptr(g), _ptr(u), _stream(stream))


def make_form(mass=0.0, diff=0.0, dt=1.0, wind=None, wind_vtx: Optional[torch.Tensor] = None, ipc=10.0, dg=False,
              outflow_mask=0, wn_mask=0, nitsche_mask=0, robin: Optional[Dict[int, float]] = None) -> LB.Form:
    """The bilinear form; ``robin`` maps boundary labels to the coefficient c of a Robin facet term
    dt c (u, v) on them (OpenCMP's -dt dc r (u, v), so c = -dc r)."""
    f = LB.Form()
    f.mass, f.diff, f.dt, f.ipc, f.dg = mass, diff, dt, ipc, int(dg)
    f.outflow_mask, f.wn_mask, f.nitsche_mask = outflow_mask, wn_mask, nitsche_mask
    for lab, c in (robin or {}).items():
        f.robin_mask |= 1 << lab
        f.robin[lab] = c
    f.wind_kind = LB.WIND_NONE
    if wind_vtx is not None:
        f.wind_kind = LB.WIND_VERTEX
        f.wind_vtx = wind_vtx.data_ptr()
    elif wind is not None:
        f.wind_kind = LB.WIND_CONST
        for k, w in enumerate(wind):
            f.wind[k] = w
    return f


def make_rhs(dt=1.0, src_const=None, src_qp: Optional[torch.Tensor] = None, mass=0.0,
             uprev: Optional[torch.Tensor] = None, bval: Optional[Dict[int, float]] = None,
             gval: Optional[Dict[int, float]] = None, bval_fq: Optional[torch.Tensor] = None,
             gval_fq: Optional[torch.Tensor] = None, bval_mask: Optional[int] = None, dfloat: bool = False) -> LB.Rhs:
    r = LB.Rhs()
    r.dt, r.mass = dt, mass
    r.src_kind = LB.SRC_NONE
    if src_qp is not None:
        r.src_kind, r.src_qp = LB.SRC_QP, src_qp.data_ptr()
    elif src_const is not None:
        r.src_kind, r.src_const = LB.SRC_CONST, src_const
    if uprev is not None:
        r.uprev = uprev.data_ptr()
    for lab, v in (bval or {}).items():
        r.bval[lab] = v
        r.bval_mask |= 1 << lab
    for lab, v in (gval or {}).items():
        r.gval[lab] = v
    if bval_mask is not None:
        r.bval_mask = bval_mask
    r.dfloat = int(dfloat)
    if bval_fq is not None:
        r.bval_fq = bval_fq.data_ptr()
    if gval_fq is not None:
        r.gval_fq = gval_fq.data_ptr()
    return r


MAT_FP32, MAT_JACOBI64, MAT_JACOBI32, MAT_DFLOAT, MAT_SELL32 = 1, 2, 4, 8, 16


class Matrix:
    """Assembled sparse matrix in the space's CSR pattern: FP64 values, and optionally an FP32 copy
    (``fp32``) and the Jacobi-scaled Krylov matrices A D^-1 in FP64 / FP32 (``jacobi64`` /
    ``jacobi32``) written by the same assembly pass. ``dfloat`` assembles in double-float arithmetic
    on the FP32 pipes (about 1e-14 relative to the native FP64 assembly)."""

    def __init__(self, space: Space, fp32: bool = False, jacobi64: bool = False, jacobi32: bool = False,
                 dfloat: bool = False, batch: int = 1, sell: bool = False):
        self.space = space
        h = C.c_void_p()
        flags = (MAT_FP32 if fp32 else 0) | (MAT_JACOBI64 if jacobi64 else 0) | (MAT_JACOBI32 if jacobi32 else 0) \
            | (MAT_DFLOAT if dfloat else 0) | (MAT_SELL32 if sell else 0)
        self.batch = batch
        LB.call('ocmp_matrix_create_batch', space.h, batch, flags, C.byref(h))
        self.h = h
        self.fp32 = fp32
        self.flags = flags

    def __del__(self):
        if getattr(self, 'h', None) and LB._lib is not None:
            LB._lib.ocmp_matrix_destroy(self.h)
            self.h = None

    def assemble(self, form: LB.Form, stream=None):
        LB.call('ocmp_assemble_matrix', self.h, C.byref(form), _stream(stream))

    def assemble_batch(self, forms, stream=None):
        """Assemble every instance of a batched matrix, one form per instance."""
        arr = (LB.Form * len(forms))(*forms)
        self._forms_keep = arr
        LB.call('ocmp_assemble_matrix_batch', self.h, arr, _stream(stream))

    def device_values(self):
        """Zero-copy torch views of the FP64 (and FP32, or None) value arrays on the device."""
        p64, p32 = C.c_void_p(), C.c_void_p()
        LB.call('ocmp_matrix_values', self.h, C.byref(p64), C.byref(p32))
        v64 = _dev_view(p64.value, self.space.nnz, '<f8', self)
        v32 = _dev_view(p32.value, self.space.nnz, '<f4', self) if p32.value else None
        return v64, v32

    def scaled_values(self):
        """Host copies of (A D^-1 in FP64 or None, A D^-1 in FP32 or None, D^-1 or None)."""
        p64, p32, pd = C.c_void_p(), C.c_void_p(), C.c_void_p()
        LB.call('ocmp_matrix_scaled_values', self.h, C.byref(p64), C.byref(p32), C.byref(pd))
        torch.cuda.synchronize()
        n, nd = self.space.nnz, self.space.ndof
        v64 = _dev_view(p64.value, n, '<f8', self).cpu().numpy() if p64.value else None
        v32 = _dev_view(p32.value, n, '<f4', self).cpu().numpy() if p32.value else None
        d = _dev_view(pd.value, nd, '<f8', self).cpu().numpy() if pd.value else None
        return v64, v32, d

    def values(self) -> np.ndarray:
        """FP64 values copied to the host (for checks)."""
        torch.cuda.synchronize()
        return self.device_values()[0].cpu().numpy()

    def values32(self) -> np.ndarray:
        torch.cuda.synchronize()
        return self.device_values()[1].cpu().numpy()

    def autotune(self, stream=None):
        """Pick the SpMV row configuration by timing the candidates on this matrix."""
        x = torch.randn(self.space.ndof, dtype=torch.float64, device='cuda')
        y = torch.empty_like(x)
        tpr, u, ms = C.c_int32(0), C.c_int32(0), C.c_float(0)
        LB.call('ocmp_matrix_autotune', self.h, _ptr(x), _ptr(y), _stream(stream), C.byref(tpr), C.byref(u),
                C.byref(ms))
        return {'threads_per_row': tpr.value, 'unroll': u.value, 'spmv_ms': ms.value}

    def mult(self, x: torch.Tensor, y: torch.Tensor, stream=None):
        LB.call('ocmp_spmv', self.h, _ptr(x), _ptr(y), _stream(stream))


class _CudaArray:
    """Minimal __cuda_array_interface__ holder so torch can view library-owned device memory."""

    def __init__(self, ptr, n, typestr, owner):
        self.__cuda_array_interface__ = {'shape': (n,), 'typestr': typestr, 'data': (ptr, False), 'version': 3,
                                         'strides': None}
        self._owner = owner


def _dev_view(ptr, n, typestr, owner):
    return torch.as_tensor(_CudaArray(ptr, n, typestr, owner), device='cuda')


def assemble_rhs(space: Space, form: LB.Form, rhs: LB.Rhs, b: torch.Tensor, stream=None):
    LB.call('ocmp_assemble_rhs', space.h, C.byref(form), C.byref(rhs), _ptr(b), _stream(stream))


class KrylovSolver:
    """Preconditioned CG / GMRES(m) on the free dofs of an assembled matrix (``ocmp_solve``)."""

    def __init__(self, mat: Matrix, method='GMRES', restart=30, precond='jacobi', precision='fp64', tol=1e-8,
                 maxit=1000, inner_tol=1e-4, check_every=8):
        self.mat = mat
        p = LB.SolveParams()
        p.method = LB.CG if str(method).upper() == 'CG' else LB.GMRES
        p.restart = restart
        p.precond = {'none': LB.PRE_NONE, 'jacobi': LB.PRE_JACOBI, 'local': LB.PRE_JACOBI,
                     'block_jacobi': LB.PRE_BLOCK_JACOBI, 'block': LB.PRE_BLOCK_JACOBI,
                     'user': LB.PRE_USER, 'strip': LB.PRE_STRIP, 'direct': LB.PRE_STRIP,
                     'cahouet_chabard': LB.PRE_CAHOUET_CHABARD}[str(precond).lower()]
        p.precision = LB.MIXED if str(precision).lower() == 'mixed' else LB.FP64
        p.tol, p.maxit, p.inner_tol, p.check_every = tol, maxit, inner_tol, check_every
        self.params = p
        h = C.c_void_p()
        LB.call('ocmp_solver_create', mat.h, C.byref(p), C.byref(h))
        self.h = h

    def __del__(self):
        if getattr(self, 'h', None) and LB._lib is not None:
            LB._lib.ocmp_solver_destroy(self.h)
            self.h = None

    def update(self, stream=None):
        LB.call('ocmp_solver_update', self.h, _stream(stream))

    def set_diag(self, dinv: torch.Tensor, stream=None):
        """The inverse diagonal used by precond='user' (taken over by the next update())."""
        LB.call('ocmp_solver_set_diag', self.h, _ptr(dinv), _stream(stream))

    def spmv_timing(self, on: bool = True):
        """Time each GMRES SpMV launch with CUDA events (resets the totals)."""
        LB.call('ocmp_solver_spmv_timing', self.h, int(on))

    def spmv_stats(self):
        """(launches timed, total milliseconds) since spmv_timing(True)."""
        n, ms = C.c_int64(0), C.c_double(0)
        LB.call('ocmp_solver_spmv_stats', self.h, C.byref(n), C.byref(ms))
        return n.value, ms.value

    def strip_stats(self) -> dict:
        """Sizes and timings of the last strip factorisation (precond='strip')."""
        o = LB.StripStats()
        LB.call('ocmp_solver_strip_stats', self.h, C.byref(o))
        return {k: getattr(o, k) for k, _ in LB.StripStats._fields_}

    def set_cahouet_chabard(self, pop: 'Matrix', vdinv: torch.Tensor, mpinv: torch.Tensor, alpha: float, beta: float,
                            tc: float, refactor: bool, stream=None):
        """Data of precond='cahouet_chabard' (ocmp_solver_set_cahouet_chabard): the pressure operator
        pop, the inverse velocity diagonal (its length is the velocity dofs), the inverse pressure-mass
        diagonal and the coefficients; pop is factorised on the first call and when refactor is set."""
        LB.call('ocmp_solver_set_cahouet_chabard', self.h, pop.h, _ptr(vdinv), _ptr(mpinv), vdinv.numel(), alpha,
                beta, tc, int(refactor), _stream(stream))

    def strip_gemm(self, kind: str):
        """Dense products of the next strip factorisations: 'simt' (FP32 FMA) or 'tensor' (tcgen05)."""
        LB.call('ocmp_solver_strip_gemm', self.h, {'simt': 0, 'tensor': 1}[kind])

    def strip_schulz(self, on: bool = True):
        """Newton-Schulz interface inverses in the next strip factorisations (on by default; off:
        block Gauss-Jordan over every strip)."""
        LB.call('ocmp_solver_strip_schulz', self.h, int(on))

    def strip_timing(self, on: bool = True):
        """Time every dense product of the next strip factorisations with CUDA events."""
        LB.call('ocmp_solver_strip_timing', self.h, int(on))

    def set_graph(self, on: bool = True):
        """Replay each restart cycle from a captured CUDA graph (GMRES)."""
        LB.call('ocmp_solver_set_graph', self.h, int(on))

    def solve_batch(self, b: torch.Tensor, x: torch.Tensor, stream=None, raise_on_fail=True):
        """Solve all systems of a batched matrix; b and x hold batch x ndof values."""
        nb = self.mat.batch
        infos = (LB.SolveInfo * nb)()
        st = LB.load().ocmp_solve_batch(self.h, _ptr(b), _ptr(x), _stream(stream), infos)
        if raise_on_fail:
            LB.check(st)
        return list(infos)

    def solve(self, b: torch.Tensor, x: torch.Tensor, stream=None, raise_on_fail=True) -> LB.SolveInfo:
        info = LB.SolveInfo()
        st = LB.load().ocmp_solve(self.h, _ptr(b), _ptr(x), _stream(stream), C.byref(info))
        if raise_on_fail:
            LB.check(st)
        return info


class KrylovGroup:
    """GMRES over the instances of several solvers at once (``ocmp_group_*``): uneven sizes, orders
    and patterns in one kernel sequence. The members (``KrylovSolver``, single or batched matrices)
    must be GMRES with point Jacobi, share restart, precision and maxit, and stay alive with the
    group; their own ``update()`` refreshes what the group solves with."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h for s in self.solvers])
        h = C.c_void_p()
        LB.call('ocmp_group_create', arr, len(self.solvers), C.byref(h))
        self.h = h
        self.ninst = sum(s.mat.batch for s in self.solvers)

    def __del__(self):
        if getattr(self, 'h', None) and LB._lib is not None:
            LB._lib.ocmp_group_destroy(self.h)
            self.h = None

    def solve(self, bs, xs, stream=None, raise_on_fail=True):
        """bs, xs: one device tensor per member (its instances one after another); returns the
        SolveInfo of every instance in member order."""
        if len(bs) != len(self.solvers) or len(xs) != len(self.solvers):
            raise ValueError('one right-hand side and one solution per member')
        pb = (C.c_void_p * len(bs))(*[_ptr(b) for b in bs])
        px = (C.c_void_p * len(xs))(*[_ptr(x) for x in xs])
        infos = (LB.SolveInfo * self.ninst)()
        st = LB.load().ocmp_group_solve(self.h, pb, px, _stream(stream), infos)
        if raise_on_fail:
            LB.check(st)
        return list(infos)


_EDGES = {2: [(0, 1), (0, 2), (1, 2)], 3: [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]}


def interpolate_p2_arrays(coords, sorted_conn, dofs, ndof, fn):
    """P2 Lagrange interpolant of fn in the hierarchical basis (vertex values; edge bubble
    lam_a lam_b with coefficient 4 (f(mid) - (f(a) + f(b)) / 2)). Host-side, numpy."""
    D = coords.shape[1]
    u = np.zeros(ndof, np.float64)
    nv = coords.shape[0]
    u[:nv] = fn(coords)
    for k, (a, b) in enumerate(_EDGES[D]):
        va, vb = sorted_conn[:, a], sorted_conn[:, b]
        mid = 0.5 * (coords[va] + coords[vb])
        u[dofs[:, D + 1 + k]] = 4.0 * (fn(mid) - 0.5 * (u[va] + u[vb]))
    return u


def interpolate_p2(space: 'Space', fn):
    """Interpolant of fn in an H1 order-2 space (initial conditions of the benchmarks)."""
    if space.kind != LB.H1 or space.order != 2:
        raise ValueError('interpolate_p2 needs an H1 order-2 space')
    m = space.mesh
    return interpolate_p2_arrays(m.coords, np.sort(m.elements, axis=1), space.dofs(), space.ndof, fn)


class TaylorHood:
    """Taylor-Hood velocity/pressure system on triangles (``ocmp_th_*``): velocity H1 order k per
    component, pressure H1 order k-1, compound vector [u_x | u_y | p]; ``dirichlet`` names the
    velocity Dirichlet labels."""

    def __init__(self, mesh: Mesh, k: int = 2, dirichlet: Sequence[str] | str = (), gmesh: Optional[GPUMesh] = None):
        self.mesh = mesh
        self.gmesh = gmesh or GPUMesh(mesh)
        self.k = k
        self.dirichlet_mask = mesh.label_mask(dirichlet)
        h = C.c_void_p()
        LB.call('ocmp_th_create', self.gmesh.h, k, self.dirichlet_mask, C.byref(h))
        self.h = h
        v, p, c = C.c_void_p(), C.c_void_p(), C.c_void_p()
        LB.call('ocmp_th_spaces', self.h, C.byref(v), C.byref(p), C.byref(c))
        self.V = _SpaceView(mesh, self.gmesh, v, 'H1', k)
        self.Q = _SpaceView(mesh, self.gmesh, p, 'H1', k - 1)
        self.C = _SpaceView(mesh, self.gmesh, c, 'compound', k)
        self.nu, self.np = self.V.ndof, self.Q.ndof
        self.ndof, self.nnz = self.C.ndof, self.C.nnz
        self.nq = LB.load().ocmp_th_nq(self.h)

    def __del__(self):
        if getattr(self, 'h', None) and LB._lib is not None:
            LB._lib.ocmp_th_destroy(self.h)
            self.h = None

    def quad_points(self) -> np.ndarray:
        x = np.empty((self.mesh.ne, self.nq, 2), np.float64)
        LB.call('ocmp_th_quad_points', self.h, _ptr(x))
        return x

    def matrix(self) -> 'Matrix':
        return Matrix(self.C)

    def assemble(self, mat: 'Matrix', mass=0.0, nu=1.0, dt=1.0, eps_p=1e-10, wind: Optional[torch.Tensor] = None,
                 tcoef: Optional[float] = None, stream=None):
        """tcoef: factor of the divergence / pressure terms (default dt)."""
        f = LB.THForm(mass, nu, dt, eps_p, wind.data_ptr() if wind is not None else None,
                      dt if tcoef is None else tcoef)
        LB.call('ocmp_th_assemble', self.h, mat.h, C.byref(f), _stream(stream))

    def assemble_rhs(self, b: torch.Tensor, dt=1.0, src=(0.0, 0.0), src_qp: Optional[torch.Tensor] = None, mass=0.0,
                     uprev: Optional[torch.Tensor] = None, imex: Optional[torch.Tensor] = None, imex_coef=1.0,
                     accumulate=False, stream=None):
        r = LB.THRhs()
        r.dt, r.mass = dt, mass
        r.imex_coef, r.accumulate = imex_coef, int(accumulate)
        r.src[0], r.src[1] = src
        r.src_qp = src_qp.data_ptr() if src_qp is not None else None
        r.uprev = uprev.data_ptr() if uprev is not None else None
        r.imex = imex.data_ptr() if imex is not None else None
        LB.call('ocmp_th_assemble_rhs', self.h, C.byref(r), _ptr(b), _stream(stream))

    def block_diag(self, mat: 'Matrix', out: torch.Tensor, stream=None):
        LB.call('ocmp_th_block_diag', self.h, mat.h, _ptr(out), _stream(stream))

    def errors(self, u: torch.Tensor, ref_qp: Optional[torch.Tensor] = None, stream=None):
        l2, dv = C.c_double(0), C.c_double(0)
        LB.call('ocmp_th_errors', self.h, _ptr(u), _ptr(ref_qp) if ref_qp is not None else None, C.byref(l2),
                C.byref(dv), _stream(stream))
        return l2.value, dv.value

    def component(self, u: torch.Tensor, c: int) -> torch.Tensor:
        """View of velocity component c (0, 1) or the pressure (2) of a compound vector."""
        if c < 2:
            return u[c * self.nu:(c + 1) * self.nu]
        return u[2 * self.nu:]


class _SpaceView(Space):
    """A space owned by another object (the Taylor-Hood system): same queries, no destroy."""

    def __init__(self, mesh, gmesh, h, kind, order):
        self.mesh, self.gmesh, self.h, self.order = mesh, gmesh, h, order
        self.kind = {'H1': LB.H1, 'L2': LB.L2}.get(kind, LB.COMPOUND)
        self.dirichlet_mask = 0
        info = LB.SpaceInfo()
        LB.call('ocmp_space_info', self.h, C.byref(info))
        self.info = info
        self.ndof, self.nnz, self.nloc, self.nq = info.ndof, info.nnz, info.nloc, info.nq
        self._free = None

    def __del__(self):
        pass
