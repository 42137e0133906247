"""ctypes binding of libopencmp_gpu.so (include/opencmp_gpu.h).

The library is the only compute path: if it is missing or fails to load, every entry point raises;
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libopencmp_gpu.so')

OK, ERR_ARG, ERR_CUDA, ERR_NONFINITE, NOT_CONVERGED, BREAKDOWN, TIMEOUT, ERR_UNSUPPORTED, ERR_NOMEM = range(9)
STATUS_NAMES = ['OK', 'ERR_ARG', 'ERR_CUDA', 'ERR_NONFINITE', 'NOT_CONVERGED', 'BREAKDOWN', 'TIMEOUT',
                'ERR_UNSUPPORTED', 'ERR_NOMEM']
H1, L2, COMPOUND = 0, 1, 2
WIND_NONE, WIND_CONST, WIND_VERTEX = 0, 1, 2
SRC_NONE, SRC_CONST, SRC_QP = 0, 1, 2
CG, GMRES = 0, 1
PRE_NONE, PRE_JACOBI, PRE_BLOCK_JACOBI, PRE_USER, PRE_STRIP, PRE_CAHOUET_CHABARD = 0, 1, 2, 3, 4, 5
FP64, MIXED = 0, 1


class OcmpError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__('{} ({}): {}'.format(STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else status,
                                              status, msg))
        self.status = status


class Form(C.Structure):
    _fields_ = [('mass', C.c_double), ('diff', C.c_double), ('dt', C.c_double), ('wind_kind', C.c_int32),
                ('wind', C.c_double * 3), ('wind_vtx', C.c_void_p), ('ipc', C.c_double), ('dg', C.c_int32),
                ('outflow_mask', C.c_uint32), ('wn_mask', C.c_uint32), ('nitsche_mask', C.c_uint32),
                ('skeleton_own_dt', C.c_int32), ('skeleton_dt', C.c_double),
                ('robin_mask', C.c_uint32), ('robin', C.c_double * 32)]


class Rhs(C.Structure):
    _fields_ = [('dt', C.c_double), ('src_kind', C.c_int32), ('src_const', C.c_double), ('src_qp', C.c_void_p),
                ('mass', C.c_double), ('uprev', C.c_void_p), ('bval', C.c_double * 32), ('bval_mask', C.c_uint32),
                ('gval', C.c_double * 32), ('bval_fq', C.c_void_p), ('gval_fq', C.c_void_p),
                ('accumulate', C.c_int32), ('dfloat', C.c_int32)]


class THForm(C.Structure):
    _fields_ = [('mass', C.c_double), ('nu', C.c_double), ('dt', C.c_double), ('eps_p', C.c_double),
                ('wind', C.c_void_p), ('tcoef', C.c_double)]


class THRhs(C.Structure):
    _fields_ = [('dt', C.c_double), ('src', C.c_double * 2), ('src_qp', C.c_void_p), ('mass', C.c_double),
                ('uprev', C.c_void_p), ('imex', C.c_void_p), ('imex_coef', C.c_double), ('accumulate', C.c_int32)]


class SpaceInfo(C.Structure):
    _fields_ = [('ndof', C.c_int64), ('nnz', C.c_int64), ('ne', C.c_int64), ('nv', C.c_int64),
                ('nloc', C.c_int32), ('nq', C.c_int32), ('dim', C.c_int32), ('order', C.c_int32),
                ('kind', C.c_int32), ('n_interior_facets', C.c_int64), ('n_boundary_facets', C.c_int64),
                ('n_contrib', C.c_int64), ('nfq', C.c_int32)]


class SolveParams(C.Structure):
    _fields_ = [('method', C.c_int32), ('restart', C.c_int32), ('precond', C.c_int32), ('precision', C.c_int32),
                ('tol', C.c_double), ('maxit', C.c_int32), ('inner_tol', C.c_double), ('check_every', C.c_int32)]


class SolveInfo(C.Structure):
    _fields_ = [('status', C.c_int32), ('iterations', C.c_int32), ('outer_iterations', C.c_int32),
                ('relres0', C.c_double), ('relres', C.c_double)]


class StripStats(C.Structure):
    _fields_ = [('nstrips', C.c_int64), ('max_strip', C.c_int64), ('bytes', C.c_int64), ('factor_ms', C.c_double),
                ('gemm_ms', C.c_double), ('gemm_flops', C.c_double), ('singular_tiles', C.c_int32),
                ('gemm_kind', C.c_int32), ('tile_ms', C.c_double), ('panel_ms', C.c_double),
                ('fast_strips', C.c_int32), ('schulz_strips', C.c_int32), ('schulz_iterations', C.c_int32),
                ('schulz_fallbacks', C.c_int32), ('gemm_bytes', C.c_double)]


P = C.c_void_p
I32, I64, U32, D = C.c_int32, C.c_int64, C.c_uint32, C.c_double

# name -> argtypes (all return int status unless listed in _RESTYPE)
SIGNATURES = {
    'ocmp_abi_version': [],
    'ocmp_last_error': [C.c_char_p, C.c_int],
    'ocmp_device_sync': [P],
    'ocmp_mesh_create': [P, I64, I32, P, I64, P, P, I64, C.POINTER(P)],
    'ocmp_mesh_destroy': [P],
    'ocmp_space_create': [P, I32, I32, U32, C.POINTER(P)],
    'ocmp_space_destroy': [P],
    'ocmp_space_info': [P, C.POINTER(SpaceInfo)],
    'ocmp_space_get_dofs': [P, P],
    'ocmp_space_get_pattern': [P, P, P],
    'ocmp_space_get_free': [P, P],
    'ocmp_space_quad_points': [P, P],
    'ocmp_set_boundary': [P, U32, P, P, P],
    'ocmp_l2_error': [P, P, P, D, P, P],
    'ocmp_space_facet_quad_points': [P, P],
    'ocmp_space_boundary_facets': [P, P],
    'ocmp_boundary_points': [P, U32, P, P],
    'ocmp_set_boundary_values': [P, U32, P, P, P],
    'ocmp_matrix_create': [P, I32, C.POINTER(P)],
    'ocmp_matrix_create_batch': [P, I32, I32, C.POINTER(P)],
    'ocmp_assemble_matrix_batch': [P, P, P],
    'ocmp_solve_batch': [P, P, P, P, P],
    'ocmp_group_create': [C.POINTER(P), I32, C.POINTER(P)],
    'ocmp_group_solve': [P, C.POINTER(P), C.POINTER(P), P, P],
    'ocmp_group_destroy': [P],
    'ocmp_solver_set_graph': [P, I32],
    'ocmp_matrix_destroy': [P],
    'ocmp_matrix_values': [P, C.POINTER(P), C.POINTER(P)],
    'ocmp_matrix_scaled_values': [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)],
    'ocmp_assemble_matrix': [P, C.POINTER(Form), P],
    'ocmp_assemble_rhs': [P, C.POINTER(Form), C.POINTER(Rhs), P, P],
    'ocmp_spmv': [P, P, P, P],
    'ocmp_spmv_axpby': [P, D, P, D, P, P],
    'ocmp_solver_set_diag': [P, P, P],
    'ocmp_launch_count': [],
    'ocmp_solver_spmv_timing': [P, I32],
    'ocmp_solver_spmv_stats': [P, P, P],
    'ocmp_th_create': [P, I32, U32, P],
    'ocmp_th_destroy': [P],
    'ocmp_th_spaces': [P, P, P, P],
    'ocmp_th_nq': [P],
    'ocmp_th_quad_points': [P, P],
    'ocmp_th_assemble': [P, P, P, P],
    'ocmp_th_assemble_rhs': [P, P, P, P],
    'ocmp_th_block_diag': [P, P, P, P],
    'ocmp_th_errors': [P, P, P, P, P, P],
    'ocmp_matrix_autotune': [P, P, P, P, P, P, P],
    'ocmp_solver_create': [P, C.POINTER(SolveParams), C.POINTER(P)],
    'ocmp_solver_destroy': [P],
    'ocmp_solver_update': [P, P],
    'ocmp_solve': [P, P, P, P, C.POINTER(SolveInfo)],
    'ocmp_solve_cg_noalloc': [P, P, P, D, I32, P, C.POINTER(SolveInfo)],
    'ocmp_solver_strip_stats': [P, C.POINTER(StripStats)],
    'ocmp_solver_strip_timing': [P, I32],
    'ocmp_solver_set_cahouet_chabard': [P, P, P, P, I64, D, D, D, I32, P],
    'ocmp_solver_strip_gemm': [P, I32],
    'ocmp_solver_strip_schulz': [P, I32],
    'ocmp_dense_gemm_nt': [I32, I32, I32, I32, P, I64, P, I64, P, I64, C.c_float, C.c_float, P],
    'ocmp_guess_create': [I32, C.c_uint64, C.POINTER(P)],
    'ocmp_guess_destroy': [P],
    'ocmp_guess_nparams': [P],
    'ocmp_guess_params': [P, P, I32],
    'ocmp_guess_forward': [P, P, I64, P, P],
    'ocmp_guess_loss_grad': [P, P, P, I64, P, P, P],
    'ocmp_guess_adam_step': [P, C.c_float, P],
    'ocmp_guess_backward': [P, P, P, I64, P, P],
    'ocmp_guess_push': [I64, I32, I32, P, P, P],
    'ocmp_guess_features': [P, I64, I32, P, P, P, P, P],
    'ocmp_guess_predict': [P, I64, I32, P, P, P, I32, P, P],
    'ocmp_guess_target': [I64, I32, P, P, P, I32, P, P, P],
    'ocmp_guess_residual_loss': [P, P, P, P, P, P, D, P, P, P],
    'ocmp_spmv_transpose': [P, P, P, P],
}

_lib = None


def load():
    """Load the in-tree library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OcmpError(ERR_ARG, 'libopencmp_gpu.so is not built; run opencmp_gb300.build.build() '
                                 '(or __graft_entry__.build())')
    L = C.CDLL(LIB_PATH)
    for name, argt in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = argt
        fn.restype = C.c_int
    L.ocmp_launch_count.restype = C.c_uint64
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().ocmp_last_error(buf, 1024)
    return buf.value.decode(errors='replace')


def check(status: int, allow=()):
    if status != OK and status not in allow:
        raise OcmpError(status, last_error())
    return status


def call(name, *args, allow=()):
    return check(getattr(load(), name)(*args), allow=allow)
