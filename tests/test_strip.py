"""Dense products of the strip factorisation (ocmp_dense_gemm_nt) and the strip direct
preconditioner with each product backend.

The products are checked against a plain PyTorch reference of the same operation (computed in FP64
from the same FP32 inputs): the FP32 SIMT kernel to FP32 rounding, the tensor-core kernel (tcgen05
kind::tf32 with the 3xTF32 split, operands staged by TMA) to the split scheme's error bound, about
2^-21 of sum_k |a_ik b_jk| per entry.
"""
import ctypes as C

import numpy as np
import pytest

from opencmp_gb300 import mesh as M

pytestmark = pytest.mark.gpu

EPS_CD = 1e-3


def _gemm(lib, kind, A, B, Cm, alpha, beta):
    import torch
    M_, K = A.shape
    N = B.shape[0]
    st = lib.load().ocmp_dense_gemm_nt(kind, M_, N, K, C.c_void_p(A.data_ptr()), A.stride(0), C.c_void_p(B.data_ptr()),
                                       B.stride(0), C.c_void_p(Cm.data_ptr()), Cm.stride(0), alpha, beta,
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == lib.OK, lib.last_error()
    torch.cuda.synchronize()


@pytest.mark.parametrize('kind', [0, 1])
@pytest.mark.parametrize('shape', [(128, 128, 32), (256, 384, 128), (384, 256, 1536), (1024, 640, 128)])
@pytest.mark.parametrize('ab', [(1.0, 0.0), (-1.0, 1.0)])
def test_dense_product_matches_torch(gpu_lib, kind, shape, ab):
    import torch
    M_, N, K = shape
    alpha, beta = ab
    g = torch.Generator(device='cuda').manual_seed(M_ * 7 + N * 3 + K + kind)
    A = torch.randn(M_, K, device='cuda', generator=g, dtype=torch.float32)
    B = torch.randn(N, K, device='cuda', generator=g, dtype=torch.float32)
    C0 = torch.randn(M_, N, device='cuda', generator=g, dtype=torch.float32)
    Cm = C0.clone()
    _gemm(gpu_lib, kind, A, B, Cm, alpha, beta)
    ref = alpha * (A.double() @ B.double().T) + beta * C0.double()
    scale = (A.double().abs() @ B.double().abs().T) + abs(beta) * C0.double().abs()
    err = ((Cm.double() - ref).abs() / scale).max().item()
    bound = 2e-6 if kind == 0 else 2e-5
    assert err <= bound, (kind, shape, err)


def test_dense_product_strided_operands(gpu_lib):
    """Leading dimensions larger than the rows: sub-blocks of bigger row-major arrays, as the
    factorisation passes them."""
    import torch
    g = torch.Generator(device='cuda').manual_seed(5)
    big_a = torch.randn(256, 512, device='cuda', generator=g)
    big_b = torch.randn(384, 256, device='cuda', generator=g)
    big_c = torch.randn(256, 768, device='cuda', generator=g)
    A, B = big_a[:, 128:256], big_b[:, :128]
    for kind in (0, 1):
        Cm = big_c.clone()
        view = Cm[:, 256:640]
        _gemm(gpu_lib, kind, A, B, view, -1.0, 1.0)
        ref = big_c.double().clone()
        ref[:, 256:640] -= A.double() @ B.double().T
        scale = (A.double().abs() @ B.double().abs().T).max().item()
        assert (Cm.double() - ref).abs().max().item() <= 2e-5 * scale
        assert torch.equal(Cm[:, :256], big_c[:, :256]) and torch.equal(Cm[:, 640:], big_c[:, 640:])


def _cd_system(n):
    import torch
    from opencmp_gb300 import fem
    m = M.unit_square(n)
    sp = fem.Space(m, 'L2', 2)
    X = m.coords
    W = torch.as_tensor(np.ascontiguousarray(np.stack([-(X[:, 1] - 0.5), X[:, 0] - 0.5], 1)), device='cuda')
    allb = m.label_mask(m.bc_names)
    f = fem.make_form(diff=EPS_CD, dt=1.0, wind_vtx=W, dg=True, ipc=10.0, nitsche_mask=allb)
    A = fem.Matrix(sp)
    A.assemble(f)
    Xq = sp.quad_points()
    r2 = (Xq[..., 0] - 0.3) ** 2 + (Xq[..., 1] - 0.5) ** 2
    fq = torch.as_tensor(np.exp(-r2 / (2 * 0.05 ** 2)), device='cuda')
    b = torch.zeros(sp.ndof, dtype=torch.float64, device='cuda')
    fem.assemble_rhs(sp, f, fem.make_rhs(src_qp=fq, gval={k: 0.0 for k in range(len(m.bc_names))}), b)
    return sp, A, b


def test_strip_factorisation_tensor_and_simt_agree(gpu_lib):
    """The strip preconditioner built with tensor-core products and with FP32 SIMT products:
    both GMRES solves reach 1e-10 in a few iterations and agree to what that residual allows."""
    import torch
    from opencmp_gb300 import fem
    sp, A, b = _cd_system(48)
    sols, iters = {}, {}
    for kind in ('simt', 'tensor'):
        sv = fem.KrylovSolver(A, method='GMRES', restart=50, precond='strip', precision='fp64', tol=1e-10, maxit=200)
        sv.strip_gemm(kind)
        sv.update()
        x = torch.zeros_like(b)
        info = sv.solve(b, x)
        assert info.status == 0 and info.relres <= 1e-10
        st = sv.strip_stats()
        assert st['gemm_kind'] == (1 if kind == 'tensor' else 0) and st['singular_tiles'] == 0
        sols[kind], iters[kind] = x.cpu().numpy(), info.iterations
    d = np.linalg.norm(sols['tensor'] - sols['simt']) / np.linalg.norm(sols['simt'])
    assert d <= 1e-8, d
    assert abs(iters['tensor'] - iters['simt']) <= 3, iters


def test_strip_preconditioner_refuses_cg_and_unbanded(gpu_lib):
    from opencmp_gb300 import fem, _lib
    sp, A, b = _cd_system(8)
    with pytest.raises(_lib.OcmpError) as e:
        fem.KrylovSolver(A, method='CG', precond='strip')
    assert e.value.status in (_lib.ERR_UNSUPPORTED, _lib.ERR_ARG)


def test_strip_preconditioner_built_before_assembly(gpu_lib):
    """OpenCMP's order (base_model.py:365-383, base_solver.py:368-377): the preconditioner is built on
    a matrix that is not assembled yet and updated after every assembly. Building it does not
    factorise; a solve before the first update is refused; after assembly and update the solve
    converges."""
    import torch
    from opencmp_gb300 import fem, _lib
    sp, A, b = _cd_system(16)
    A0 = fem.Matrix(sp)
    sv = fem.KrylovSolver(A0, method='GMRES', restart=50, precond='strip', precision='fp64', tol=1e-10, maxit=200)
    x = torch.zeros_like(b)
    with pytest.raises(_lib.OcmpError) as e:
        sv.solve(b, x)
    assert e.value.status == _lib.ERR_ARG
    A0.device_values()[0].copy_(A.device_values()[0])
    sv.update()
    info = sv.solve(b, x)
    assert info.status == 0 and info.relres <= 1e-10 and info.iterations <= 20


@pytest.mark.parametrize('kind', ['simt', 'tensor'])
def test_strip_newton_schulz_matches_gauss_jordan(gpu_lib, kind):
    """At 96 x 96 every strip is one row of DG elements: its non-interface dofs (the elements that
    do not touch the previous row) are independent 6-dof groups, and the interface inverse comes
    from Newton-Schulz started at the previous strip's. The factorisation with that path and the
    block Gauss-Jordan one precondition GMRES to the same solution in as many iterations, give or
    take two."""
    import torch
    from opencmp_gb300 import fem
    sp, A, b = _cd_system(96)
    sols, iters, stats = {}, {}, {}
    for on in (False, True):
        sv = fem.KrylovSolver(A, method='GMRES', restart=50, precond='strip', precision='fp64', tol=1e-10, maxit=200)
        sv.strip_gemm(kind)
        sv.strip_schulz(on)
        sv.update()
        x = torch.zeros_like(b)
        info = sv.solve(b, x)
        assert info.status == 0 and info.relres <= 1e-10
        stats[on] = sv.strip_stats()
        assert stats[on]['singular_tiles'] == 0
        sols[on], iters[on] = x.cpu().numpy(), info.iterations
    st = stats[True]
    assert stats[False]['fast_strips'] == 0 and stats[False]['schulz_strips'] == 0
    assert st['fast_strips'] >= st['nstrips'] - 2, st
    assert st['schulz_strips'] >= st['fast_strips'] - 2 and st['schulz_fallbacks'] <= 2, st
    assert st['schulz_iterations'] <= 6 * st['schulz_strips'], st
    d = np.linalg.norm(sols[True] - sols[False]) / np.linalg.norm(sols[False])
    assert d <= 1e-8, d
    assert abs(iters[True] - iters[False]) <= 2, iters
