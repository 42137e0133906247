"""Simplicial meshes for the GPU finite-element path.

A :class:`Mesh` holds what the GPU library needs and nothing else: vertex coordinates (nv x D,
float64), element connectivity (ne x (D+1), int32), boundary facets (nbf x D, int32) with a
boundary label per facet, and the label names.  It stands in for the netgen mesh OpenCMP loads in
``opencmp/helpers/io.py:69-110`` (``load_mesh``): ``.vol`` (Netgen ASCII) and ``.msh`` (Gmsh 2.2)
files are read here, and the structured meshes of the benchmark configurations are generated here.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import List

import numpy as np


@dataclass
class Mesh:
    coords: np.ndarray            # (nv, D) float64
    elements: np.ndarray          # (ne, D+1) int32
    bfacets: np.ndarray           # (nbf, D) int32
    blabels: np.ndarray           # (nbf,) int32, index into bc_names
    bc_names: List[str] = field(default_factory=list)

    @property
    def dim(self) -> int:
        return int(self.coords.shape[1])

    @property
    def nv(self) -> int:
        return int(self.coords.shape[0])

    @property
    def ne(self) -> int:
        return int(self.elements.shape[0])

    def GetBoundaries(self) -> List[str]:
        """Boundary names, like netgen's ``Mesh.GetBoundaries``."""
        return list(self.bc_names)

    def Refine(self) -> 'Mesh':
        """Uniform refinement in place, as netgen's ``Mesh.Refine()`` that OpenCMP's h-convergence test
        calls (``opencmp/post_processing/error_analysis.py:84``): every triangle into four, every
        tetrahedron into eight (:func:`refine_uniform`)."""
        r = refine_uniform(self)
        self.coords, self.elements, self.bfacets, self.blabels = r.coords, r.elements, r.bfacets, r.blabels
        return self

    def label_mask(self, names) -> int:
        """Bit mask of the labels named in ``names`` (a list or a '|'-separated string)."""
        if isinstance(names, str):
            names = [n for n in names.split('|') if n]
        m = 0
        for n in names:
            if n in self.bc_names:
                m |= 1 << self.bc_names.index(n)
        return m


def _midpoints(coords: np.ndarray, pairs: np.ndarray):
    """Unique edges of the (k, 2) vertex pairs and, per pair, the index of its midpoint vertex
    (appended after the existing vertices, edges in ascending (lower, upper) order)."""
    lo = np.minimum(pairs[:, 0], pairs[:, 1]).astype(np.int64)
    hi = np.maximum(pairs[:, 0], pairs[:, 1]).astype(np.int64)
    nv = coords.shape[0]
    key = lo * nv + hi
    uniq, inv = np.unique(key, return_inverse=True)
    ea, eb = uniq // nv, uniq % nv
    mid = 0.5 * (coords[ea] + coords[eb])
    return np.concatenate([coords, mid]), (nv + inv).astype(np.int64)


def refine_uniform(mesh: Mesh) -> Mesh:
    """One level of uniform (red) refinement of a straight-sided simplicial mesh.

    Triangles: the three corner triangles and the middle one of the edge midpoints. Tetrahedra: the
    four corner tetrahedra and the inner octahedron cut into four along its shortest diagonal
    (the diagonal choice keeps the element shapes from degrading over repeated refinements).
    Boundary facets are split the same way (edges into two, triangles into four) and keep their
    labels. Midpoint vertices are numbered after the old vertices in ascending edge order."""
    X, E = mesh.coords, mesh.elements.astype(np.int64)
    D = mesh.dim
    ne = E.shape[0]
    if D == 2:
        loc = [(0, 1), (1, 2), (0, 2)]
    else:
        loc = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    pairs = np.concatenate([E[:, [a, b]] for a, b in loc])
    Xn, mids = _midpoints(X, pairs)
    M = mids.reshape(len(loc), ne).T                     # M[e, k] = midpoint of local edge k
    if D == 2:
        v0, v1, v2 = E[:, 0], E[:, 1], E[:, 2]
        m01, m12, m02 = M[:, 0], M[:, 1], M[:, 2]
        kids = [(v0, m01, m02), (v1, m12, m01), (v2, m02, m12), (m01, m12, m02)]
    else:
        v0, v1, v2, v3 = E.T
        m = {k: M[:, i] for i, k in enumerate(loc)}
        kids = [(v0, m[0, 1], m[0, 2], m[0, 3]), (v1, m[0, 1], m[1, 2], m[1, 3]),
                (v2, m[0, 2], m[1, 2], m[2, 3]), (v3, m[0, 3], m[1, 3], m[2, 3])]
        # octahedron of the six midpoints: its three diagonals join midpoints of opposite edges;
        # the four faces around a diagonal run through the other four midpoints in the cycle in
        # which neighbours share an element vertex
        diag = [((0, 1), (2, 3), [(0, 2), (1, 2), (1, 3), (0, 3)]),
                ((0, 2), (1, 3), [(0, 1), (1, 2), (2, 3), (0, 3)]),
                ((0, 3), (1, 2), [(0, 1), (1, 3), (2, 3), (0, 2)])]
        length = np.stack([np.linalg.norm(Xn[m[a]] - Xn[m[b]], axis=1) for a, b, _ in diag], 1)
        pick = np.argmin(length, axis=1)
        inner = np.zeros((ne, 4, 4), np.int64)
        for d, (a, b, cyc) in enumerate(diag):
            sel = pick == d
            for q in range(4):
                c0, c1 = cyc[q], cyc[(q + 1) % 4]
                inner[sel, q] = np.stack([m[a][sel], m[b][sel], m[c0][sel], m[c1][sel]], 1)
        kids += [tuple(inner[:, q, i] for i in range(4)) for q in range(4)]
    En = np.sort(np.concatenate([np.stack(k, 1) for k in kids]), axis=1).astype(np.int32)
    # boundary facets: their edge midpoints are midpoints of element edges (same vertex pairs)
    F = mesh.bfacets.astype(np.int64)
    nv = X.shape[0]
    lo = np.minimum(pairs[:, 0], pairs[:, 1])
    hi = np.maximum(pairs[:, 0], pairs[:, 1])
    keys = lo * nv + hi
    order = np.argsort(keys, kind='stable')
    ks = keys[order]

    def mid_of(a, b):
        k = np.minimum(a, b) * nv + np.maximum(a, b)
        pos = np.searchsorted(ks, k)
        if np.any(pos >= ks.size) or np.any(ks[np.minimum(pos, ks.size - 1)] != k):
            raise ValueError('refine_uniform: a boundary facet is not a face of an element')
        return mids[order[pos]]
    if D == 2:
        a, b = F[:, 0], F[:, 1]
        mab = mid_of(a, b)
        Fn = np.concatenate([np.stack([a, mab], 1), np.stack([mab, b], 1)])
        Ln = np.concatenate([mesh.blabels, mesh.blabels])
    else:
        a, b, c = F[:, 0], F[:, 1], F[:, 2]
        mab, mbc, mac = mid_of(a, b), mid_of(b, c), mid_of(a, c)
        Fn = np.concatenate([np.stack([a, mab, mac], 1), np.stack([b, mbc, mab], 1),
                             np.stack([c, mac, mbc], 1), np.stack([mab, mbc, mac], 1)])
        Ln = np.concatenate([mesh.blabels] * 4)
    return Mesh(np.ascontiguousarray(Xn), np.ascontiguousarray(En), np.ascontiguousarray(Fn.astype(np.int32)),
                np.ascontiguousarray(Ln.astype(np.int32)), list(mesh.bc_names))


def unit_square(n: int) -> Mesh:
    """Unit square, n x n quads each split into two triangles along the (i,j)-(i+1,j+1) diagonal.

    Boundary labels follow the reference's coarse square mesh: bottom, right, top, left.
    """
    g = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(g, g, indexing='xy')
    coords = np.stack([X.ravel(), Y.ravel()], axis=1).astype(np.float64)
    vid = lambda i, j: j * (n + 1) + i  # noqa: E731
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing='xy')
    i = i.ravel(); j = j.ravel()
    v00, v10, v01, v11 = vid(i, j), vid(i + 1, j), vid(i, j + 1), vid(i + 1, j + 1)
    t1 = np.stack([v00, v10, v11], 1)
    t2 = np.stack([v00, v11, v01], 1)
    elements = np.empty((2 * n * n, 3), np.int32)
    elements[0::2] = t1
    elements[1::2] = t2
    k = np.arange(n)
    bottom = np.stack([vid(k, 0), vid(k + 1, 0)], 1)
    right = np.stack([vid(n, k), vid(n, k + 1)], 1)
    top = np.stack([vid(k + 1, n), vid(k, n)], 1)
    left = np.stack([vid(0, k + 1), vid(0, k)], 1)
    bf = np.concatenate([bottom, right, top, left]).astype(np.int32)
    bl = np.repeat(np.arange(4, dtype=np.int32), n)
    return Mesh(coords, elements, bf, bl, ['bottom', 'right', 'top', 'left'])


# The six tetrahedra of the Kuhn split of the unit cube: paths 000 -> 111 through the cube's
# vertices, one per permutation of the axes.  Cube vertex index = x + 2 y + 4 z.
_KUHN = [(0, 1, 3, 7), (0, 1, 5, 7), (0, 2, 3, 7), (0, 2, 6, 7), (0, 4, 5, 7), (0, 4, 6, 7)]


def unit_cube(n: int) -> Mesh:
    """Unit cube, n^3 cubes each split into six tetrahedra (Kuhn split, conforming).

    Boundary labels: left (x=0), right (x=1), front (y=0), back (y=1), bottom (z=0), top (z=1).
    """
    m = n + 1
    g = np.linspace(0.0, 1.0, m)
    Z, Y, X = np.meshgrid(g, g, g, indexing='ij')
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1).astype(np.float64)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing='ij')
    i = i.ravel(); j = j.ravel(); k = k.ravel()
    corner = np.stack([((k + ((c >> 2) & 1)) * m + (j + ((c >> 1) & 1))) * m + (i + (c & 1)) for c in range(8)], 1)
    elements = np.concatenate([corner[:, list(t)] for t in _KUHN], axis=0).astype(np.int32)
    # order element-major by cube so that neighbouring elements are close in memory
    order = np.arange(elements.shape[0]).reshape(6, -1).T.ravel()
    elements = np.ascontiguousarray(elements[order])
    # boundary: each cube face split along the diagonal through the cube's 000-111 path
    faces, labels = [], []
    a, b = np.meshgrid(np.arange(n), np.arange(n), indexing='ij')
    a = a.ravel(); b = b.ravel()

    def vid(x, y, z):
        return (z * m + y) * m + x

    for lab, (axis, val) in enumerate([(0, 0), (0, n), (1, 0), (1, n), (2, 0), (2, n)]):
        # face quad in the plane axis = val with the two other axes (u, w) in increasing order
        def P(du, dw):
            u = a + du
            w = b + dw
            if axis == 0:
                return vid(np.full_like(u, val), u, w)
            if axis == 1:
                return vid(u, np.full_like(u, val), w)
            return vid(u, w, np.full_like(u, val))
        p00, p10, p01, p11 = P(0, 0), P(1, 0), P(0, 1), P(1, 1)
        faces.append(np.stack([p00, p10, p11], 1))
        faces.append(np.stack([p00, p11, p01], 1))
        labels.append(np.full(2 * a.size, lab, np.int32))
    bf = np.concatenate(faces).astype(np.int32)
    bl = np.concatenate(labels)
    return Mesh(coords, elements, bf, bl, ['left', 'right', 'front', 'back', 'bottom', 'top'])


def _read_vol(path: str) -> Mesh:
    """Netgen ASCII ``.vol`` reader for 2D meshes (triangles with edge segments) and 3D tet meshes."""
    with open(path) as fh:
        lines = [ln.strip() for ln in fh]
    dim = 3
    tris, tets, segs, pts, names = [], [], [], [], {}
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln == 'dimension':
            dim = int(lines[i + 1]); i += 2; continue
        if ln == 'surfaceelements':
            cnt = int(lines[i + 1])
            for r in range(cnt):
                v = lines[i + 2 + r].split()
                npnt = int(v[4])
                tris.append((int(v[1]), [int(t) - 1 for t in v[5:5 + npnt]]))
            i += 2 + cnt; continue
        if ln == 'volumeelements':
            cnt = int(lines[i + 1])
            for r in range(cnt):
                v = lines[i + 2 + r].split()
                npnt = int(v[1])
                tets.append([int(t) - 1 for t in v[2:2 + npnt]])
            i += 2 + cnt; continue
        if ln in ('edgesegmentsgi2', 'edgesegmentsgi', 'edgesegments'):
            cnt = int(lines[i + 1])
            for r in range(cnt):
                v = lines[i + 2 + r].split()
                segs.append((int(v[0]), int(v[2]) - 1, int(v[3]) - 1))
            i += 2 + cnt; continue
        if ln == 'points':
            cnt = int(lines[i + 1])
            for r in range(cnt):
                pts.append([float(t) for t in lines[i + 2 + r].split()])
            i += 2 + cnt; continue
        if ln == 'bcnames':
            cnt = int(lines[i + 1])
            for r in range(cnt):
                v = lines[i + 2 + r].split()
                names[int(v[0])] = v[1]
            i += 2 + cnt; continue
        i += 1
    coords = np.asarray(pts, np.float64)[:, :dim]
    if dim == 2:
        elements = np.asarray([t for _, t in tris], np.int32)
        bnr = sorted({s[0] for s in segs} | set(names))
        bc_names = [names.get(b, 'default') for b in bnr]
        bf = np.asarray([[s[1], s[2]] for s in segs], np.int32)
        bl = np.asarray([bnr.index(s[0]) for s in segs], np.int32)
    else:
        elements = np.asarray(tets, np.int32)
        bnr = sorted({b for b, _ in tris} | set(names))
        bc_names = [names.get(b, 'default') for b in bnr]
        bf = np.asarray([t for _, t in tris], np.int32)
        bl = np.asarray([bnr.index(b) for b, _ in tris], np.int32)
    return Mesh(np.ascontiguousarray(coords), elements, bf, bl, bc_names)


def _read_msh(path: str) -> Mesh:
    """Gmsh 2.2 ASCII reader: 2-node lines / 3-node triangles (2D) or triangles / tets (3D)."""
    with open(path) as fh:
        lines = [ln.strip() for ln in fh]
    names, nodes, elems = {}, {}, []
    i = 0
    while i < len(lines):
        if lines[i] == '$PhysicalNames':
            cnt = int(lines[i + 1])
            for r in range(cnt):
                v = lines[i + 2 + r].split()
                names[(int(v[0]), int(v[1]))] = v[2].strip('"')
            i += 2 + cnt; continue
        if lines[i] == '$Nodes':
            cnt = int(lines[i + 1])
            for r in range(cnt):
                v = lines[i + 2 + r].split()
                nodes[int(v[0])] = [float(t) for t in v[1:4]]
            i += 2 + cnt; continue
        if lines[i] == '$Elements':
            cnt = int(lines[i + 1])
            for r in range(cnt):
                v = [int(t) for t in lines[i + 2 + r].split()]
                etype, ntags = v[1], v[2]
                phys = v[3] if ntags > 0 else 0
                elems.append((etype, phys, v[3 + ntags:]))
            i += 2 + cnt; continue
        i += 1
    dim = 3 if any(e[0] == 4 for e in elems) else 2
    ids = sorted(nodes)
    remap = {k: n for n, k in enumerate(ids)}
    coords = np.asarray([nodes[k] for k in ids], np.float64)[:, :dim]
    vol_t, bnd_t = (2, 1) if dim == 2 else (4, 2)
    elements = np.asarray([[remap[k] for k in e[2]] for e in elems if e[0] == vol_t], np.int32)
    bnd = [e for e in elems if e[0] == bnd_t]
    phys = sorted({e[1] for e in bnd})
    bc_names = [names.get((dim - 1, p), str(p)) for p in phys]
    bf = np.asarray([[remap[k] for k in e[2]] for e in bnd], np.int32).reshape(-1, dim)
    bl = np.asarray([phys.index(e[1]) for e in bnd], np.int32)
    return Mesh(np.ascontiguousarray(coords), elements, bf, bl, bc_names)


def load_mesh(filename: str) -> Mesh:
    """Load a ``.vol`` or ``.msh`` mesh, like ``opencmp/helpers/io.py:69-110``."""
    ext = os.path.splitext(filename)[1]
    if ext == '.vol':
        return _read_vol(filename)
    if ext == '.msh':
        return _read_msh(filename)
    if ext == '.npz':
        d = np.load(filename, allow_pickle=False)
        return Mesh(d['coords'], d['elements'].astype(np.int32), d['bfacets'].astype(np.int32),
                    d['blabels'].astype(np.int32), [str(s) for s in d['bc_names']])
    raise TypeError('Only .vol and .msh meshes are supported, got {}'.format(filename))
