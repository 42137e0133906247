"""The allocation-free CG entry point (ocmp_solve_cg_noalloc), called through the C ABI.

It exists for callers that cannot call cudaMalloc when they solve (a stream under global-mode
graph capture, a device memory budget owned by another allocator, a loop that cannot take
cudaFree's device-wide synchronisation). Its workspace is a static device array shared by all
calls, so the check runs it twice in a row and compares both results with the allocating solve
(ocmp_solve, CG + Jacobi, FP64) at the solution tolerance the other GPU tests use (1e-8 relative),
and checks that an oversized system is refused with a clear error instead of overrunning it.
This file sorts last so a run that stops at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from opencmp_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _noalloc(lib, mat, b, x, tol, maxit):
    import torch
    info = lib.SolveInfo()
    st = lib.load().ocmp_solve_cg_noalloc(mat.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), tol, maxit,
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream), C.byref(info))
    return st, info


def test_noalloc_cg_matches_allocating_solve_twice(gpu_lib):
    import torch
    from opencmp_gb300 import fem
    lib = gpu_lib
    m = M.unit_square(40)
    g = fem.Space(m, 'H1', 2, m.bc_names)
    A = fem.Matrix(g)
    f = fem.make_form(mass=1.0, diff=0.05, dt=1.0)
    A.assemble(f)
    b = torch.zeros(g.ndof, dtype=torch.float64, device='cuda')
    fem.assemble_rhs(g, f, fem.make_rhs(src_const=1.0), b)
    tol = 1e-12
    x_ref = torch.zeros_like(b)
    ref = fem.KrylovSolver(A, method='CG', precond='jacobi', precision='fp64', tol=tol, maxit=5000).solve(b, x_ref)
    assert ref.status == 0
    xr = x_ref.cpu().numpy()
    for call in range(2):
        x = torch.zeros_like(b)
        st, info = _noalloc(lib, A, b, x, tol, 5000)
        assert st == lib.OK, lib.last_error()
        assert info.status == 0 and info.relres <= tol
        xn = x.cpu().numpy()
        assert np.linalg.norm(xn - xr) <= 1e-8 * np.linalg.norm(xr), call


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
