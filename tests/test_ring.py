"""The pipelined element-ring assembly against the two-pass assembly and the oracle.

Element-only forms on H1 spaces assembled in double-float with OCMP_MAT_RING run through the
element ring (element matrices of consecutive chunks in a ring of slots held in L2, summed into the
CSR entries once every element a row needs is written). Its sums are the two-pass
assembly's, term for term and in the same order, so every output must agree bit for bit with the
two-pass assembly (the default): FP64 values, FP32 copy, Jacobi-scaled values in CSR and
SELL-32 order, and the inverse diagonal. The meshes are large enough for many chunks and for the
ring to wrap around (unit cube 24^3 x 6: 82,944 tetrahedra in 2,048-element chunks). Against the
oracle the tolerance is the parity suite's: 1e-12 relative to the largest entry.
"""
import numpy as np
import pytest

from opencmp_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _t(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device='cuda')


def _forms(fem, m):
    D = m.dim
    X = m.coords
    wv = np.stack([-(X[:, 1] - 0.5), X[:, 0] - 0.5] + ([0.3 + 0 * X[:, 0]] if D == 3 else []), 1)
    return [
        ('mass+diffusion', fem.make_form(mass=1.0, diff=0.7, dt=0.3)),
        ('implicit-euler-const-wind', fem.make_form(mass=1.0, diff=1e-2, dt=1e-3, wind=(1.0, 0.5, 0.25)[:D])),
        ('vertex-wind', fem.make_form(mass=0.0, diff=1e-3, dt=1.0, wind_vtx=_t(wv))),
    ]


def _outputs(A):
    import torch
    torch.cuda.synchronize()
    v64, v32 = A.device_values()
    s64, s32, d = A.scaled_values()
    return [v64.cpu().numpy(), None if v32 is None else v32.cpu().numpy(), s64, s32, d]


def _same(a, b):
    for x, y in zip(a, b):
        assert (x is None) == (y is None)
        if x is not None:
            assert x.dtype == y.dtype and np.array_equal(x.view(np.uint8), y.view(np.uint8))


MESHES = [
    ('tet-p2-24', lambda: M.unit_cube(24), 2),
    ('tet-p1-16', lambda: M.unit_cube(16), 1),
    ('tri-p1-96', lambda: M.unit_square(96), 1),
    ('tri-p2-64', lambda: M.unit_square(64), 2),
    ('tri-p3-48', lambda: M.unit_square(48), 3),
]


@pytest.mark.parametrize('name,mk,order', MESHES, ids=[c[0] for c in MESHES])
def test_ring_matches_two_pass_bit_for_bit(gpu_lib, name, mk, order):
    from opencmp_gb300 import fem
    m = mk()
    sp = fem.Space(m, 'H1', order, m.bc_names)
    layouts = [dict(jacobi32=True, sell=True), dict(fp32=True, jacobi64=True, jacobi32=True)]
    for lay in layouts:
        ring = fem.Matrix(sp, dfloat=True, ring=True, **lay)
        two = fem.Matrix(sp, dfloat=True, **lay)
        # several forms in a row: the ring, its counters and the diagonal are reused every time
        for _, f in _forms(fem, m):
            ring.assemble(f)
            two.assemble(f)
            _same(_outputs(ring), _outputs(two))


def test_ring_with_scattered_numbering(gpu_lib):
    """Elements in random order: every row's elements spread over the whole element range. The
    assembly must still produce the two-pass values (the ring is planned only where the numbering
    keeps each row's elements within a window it can hold; otherwise the two-pass assembly runs)."""
    from opencmp_gb300 import fem
    m = M.unit_cube(14)
    perm = np.random.default_rng(3).permutation(m.ne)
    mp = M.Mesh(m.coords, np.ascontiguousarray(m.elements[perm]), m.bfacets, m.blabels, list(m.bc_names))
    sp = fem.Space(mp, 'H1', 2, mp.bc_names)
    ring = fem.Matrix(sp, dfloat=True, jacobi32=True, sell=True, ring=True)
    two = fem.Matrix(sp, dfloat=True, jacobi32=True, sell=True)
    f = _forms(fem, mp)[1][1]
    ring.assemble(f)
    two.assemble(f)
    _same(_outputs(ring), _outputs(two))


def test_ring_matches_oracle(gpu_lib, oracle):
    """The benchmark's form (implicit Euler, constant wind, P2 tetrahedra) through the ring against
    the oracle's FP64 assembly, and the Jacobi-scaled FP32 copy against the oracle's scaling."""
    from opencmp_gb300 import fem
    m = M.unit_cube(12)
    sp = fem.Space(m, 'H1', 2, m.bc_names)
    o = oracle.Space(m, oracle.H1, 2, m.label_mask(m.bc_names))
    kw = dict(mass=1.0, diff=1e-2, dt=1e-3, wind=(1.0, 0.5, 0.25))
    A = fem.Matrix(sp, dfloat=True, fp32=True, jacobi32=True, ring=True)
    A.assemble(fem.make_form(**kw))
    ao = o.assemble(oracle.make_form(**kw))
    v = A.values()
    assert np.abs(v - ao).max() <= 1e-12 * np.abs(ao).max()
    _, s32, d = A.scaled_values()
    rp, col = o.pattern()
    rows = np.repeat(np.arange(o.ndof), np.diff(rp))
    diag = np.zeros(o.ndof)
    diag[rows[rows == col]] = ao[rows == col]
    free = o.freedofs().astype(bool)
    dinv = np.where(free & (diag != 0), 1.0 / np.where(diag != 0, diag, 1.0), 0.0)
    assert np.allclose(d, dinv, rtol=1e-12, atol=0)
    assert np.allclose(s32, (ao * dinv[col]).astype(np.float32), rtol=1e-6, atol=1e-30)
