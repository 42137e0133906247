"""The allocation-free CG entry point (ocmp_solve_cg_noalloc), called through the C ABI.

It exists for callers that cannot call cudaMalloc when they solve: a host whose device memory
belongs to another allocator's fixed pool, or a loop that cannot take cudaFree's device-wide
synchronisation. Its workspace is a static device array shared by all calls, so the checks run it
on two calls in a row, then on a smaller system (different size, reduction grid and rows per
thread), then on the first system again, and compare every result with the allocating solve
(ocmp_solve, CG + Jacobi, FP64) at the solution tolerance the other GPU tests use (1e-8 relative).
They also check that the call leaves the device's free memory unchanged, and that an oversized
system, a batched matrix and a stream under capture are refused with a clear error.
This file sorts last so a run that stops at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from opencmp_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _noalloc(lib, mat, b, x, tol, maxit, stream=None):
    import torch
    info = lib.SolveInfo()
    s = stream if stream is not None else torch.cuda.current_stream()
    st = lib.load().ocmp_solve_cg_noalloc(mat.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), tol, maxit,
                                          C.c_void_p(s.cuda_stream), C.byref(info))
    return st, info


def _system(m, order):
    import torch
    from opencmp_gb300 import fem
    g = fem.Space(m, 'H1', order, m.bc_names)
    A = fem.Matrix(g)
    f = fem.make_form(mass=1.0, diff=0.05, dt=1.0)
    A.assemble(f)
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    fem.assemble_rhs(g, f, fem.make_rhs(src_const=1.0), b)
    return g, A, b


def _reference(A, b, tol):
    import torch
    from opencmp_gb300 import fem
    x = torch.zeros_like(b)
    info = fem.KrylovSolver(A, method='CG', precond='jacobi', precision='fp64', tol=tol, maxit=5000).solve(b, x)
    assert info.status == 0
    return x.cpu().numpy()


def _check(lib, A, b, xr, tol):
    import torch
    x = torch.zeros_like(b)
    st, info = _noalloc(lib, A, b, x, tol, 5000)
    assert st == lib.OK, lib.last_error()
    assert info.status == 0 and info.relres <= tol
    xn = x.cpu().numpy()
    assert np.linalg.norm(xn - xr) <= 1e-8 * np.linalg.norm(xr)


def test_noalloc_cg_matches_allocating_solve_twice(gpu_lib):
    import torch
    lib = gpu_lib
    tol = 1e-12
    _, A, b = _system(M.unit_square(40), 2)
    xr = _reference(A, b, tol)
    _check(lib, A, b, xr, tol)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _check(lib, A, b, xr, tol)               # second call in a row: the workspace keeps the first's contents
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)    # nothing was allocated on the device
    # a smaller system (other n, reduction grid and rows per thread), then the first one again
    _, A2, b2 = _system(M.unit_square(8), 1)
    xr2 = _reference(A2, b2, tol)
    _check(lib, A2, b2, xr2, tol)
    _check(lib, A, b, xr, tol)


def test_noalloc_cg_rejects_oversized_system(gpu_lib):
    import torch
    from opencmp_gb300 import fem
    lib = gpu_lib
    m = M.unit_square(1025)                 # P1: 1,052,676 dofs > 1,048,576
    g = fem.Space(m, 'H1', 1, m.bc_names)
    assert g.ndof > 1048576
    A = fem.Matrix(g)
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    x = torch.zeros_like(b)
    st, _ = _noalloc(lib, A, b, x, 1e-8, 10)
    assert st == lib.ERR_ARG
    assert 'limit' in lib.last_error()


def test_noalloc_cg_rejects_batched_matrix(gpu_lib):
    import torch
    from opencmp_gb300 import fem
    lib = gpu_lib
    m = M.unit_square(4)
    g = fem.Space(m, 'H1', 1, m.bc_names)
    A = fem.Matrix(g, batch=2)
    b = torch.zeros(2 * g.ndof, dtype=torch.float64, device='cuda')
    x = torch.zeros_like(b)
    st, _ = _noalloc(lib, A, b, x, 1e-8, 10)
    assert st == lib.ERR_UNSUPPORTED
    assert 'batched' in lib.last_error()


def test_noalloc_cg_refuses_a_capturing_stream(gpu_lib):
    import torch
    lib = gpu_lib
    _, A, b = _system(M.unit_square(8), 1)
    x = torch.zeros_like(b)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s, capture_error_mode='thread_local'):
        y = b * 2.0                          # keeps the captured graph non-empty
        st, _ = _noalloc(lib, A, b, x, 1e-8, 10, stream=s)
    assert st == lib.ERR_UNSUPPORTED
    assert 'captured' in lib.last_error()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, b * 2.0)
