"""Mesh readers of the drop-in layer (``load_mesh``, after ``opencmp/helpers/io.py:69-110``): Netgen
ASCII ``.vol`` and Gmsh 2.2 ``.msh`` files written here by hand for a unit square of two triangles
with four boundary labels, and one tetrahedron; ``.npz`` round trip; unknown extensions refused."""
import os

import numpy as np
import pytest

from opencmp_gb300.mesh import Mesh, load_mesh, unit_square

VOL_2D = """mesh3d
dimension
2
geomtype
0

# surfnr    bcnr   domin  domout      np      p1      p2      p3
surfaceelements
2
1 1 0 0 3 1 2 3
1 1 0 0 3 1 3 4

volumeelements
0

edgesegmentsgi2
4
1 0 1 2 -1 -1 1 0 0 0.0 0 1.0
2 0 2 3 -1 -1 1 0 0 0.0 0 1.0
3 0 3 4 -1 -1 1 0 0 0.0 0 1.0
4 0 4 1 -1 -1 1 0 0 0.0 0 1.0

points
4
0.0 0.0 0.0
1.0 0.0 0.0
1.0 1.0 0.0
0.0 1.0 0.0

bcnames
4
1 bottom
2 right
3 top
4 left

endmesh
"""

MSH_2D = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
5
1 1 "bottom"
1 2 "right"
1 3 "top"
1 4 "left"
2 5 "domain"
$EndPhysicalNames
$Nodes
4
1 0 0 0
2 1 0 0
3 1 1 0
4 0 1 0
$EndNodes
$Elements
6
1 1 2 1 1 1 2
2 1 2 2 2 2 3
3 1 2 3 3 3 4
4 1 2 4 4 4 1
5 2 2 5 1 1 2 3
6 2 2 5 1 1 3 4
$EndElements
"""

MSH_3D = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
2
2 1 "wall"
2 2 "outlet"
$EndPhysicalNames
$Nodes
4
10 0 0 0
20 1 0 0
30 0 1 0
40 0 0 1
$EndNodes
$Elements
5
1 2 2 1 1 10 30 20
2 2 2 1 1 10 20 40
3 2 2 1 1 10 40 30
4 2 2 2 2 20 30 40
5 4 2 7 1 10 20 30 40
$EndElements
"""


def _write(tmp_path, name, text):
    p = os.path.join(str(tmp_path), name)
    with open(p, 'w') as fh:
        fh.write(text)
    return p


def _check_square(m: Mesh):
    np.testing.assert_array_equal(m.coords, [[0, 0], [1, 0], [1, 1], [0, 1]])
    np.testing.assert_array_equal(m.elements, [[0, 1, 2], [0, 2, 3]])
    assert m.bc_names == ['bottom', 'right', 'top', 'left']
    np.testing.assert_array_equal(m.bfacets, [[0, 1], [1, 2], [2, 3], [3, 0]])
    np.testing.assert_array_equal(m.blabels, [0, 1, 2, 3])
    assert m.label_mask(['top']) == 1 << 2


def test_read_netgen_vol_2d(tmp_path):
    _check_square(load_mesh(_write(tmp_path, 'sq.vol', VOL_2D)))


def test_read_gmsh_2d(tmp_path):
    _check_square(load_mesh(_write(tmp_path, 'sq.msh', MSH_2D)))


def test_read_gmsh_3d_renumbers_nodes(tmp_path):
    m = load_mesh(_write(tmp_path, 'tet.msh', MSH_3D))
    assert m.coords.shape == (4, 3)
    np.testing.assert_array_equal(m.elements, [[0, 1, 2, 3]])
    assert m.bc_names == ['wall', 'outlet']
    np.testing.assert_array_equal(m.blabels, [0, 0, 0, 1])
    np.testing.assert_array_equal(m.bfacets[3], [1, 2, 3])


def test_npz_round_trip_and_unknown_extension(tmp_path):
    m = unit_square(3)
    p = os.path.join(str(tmp_path), 'sq.npz')
    np.savez(p, coords=m.coords, elements=m.elements, bfacets=m.bfacets, blabels=m.blabels,
             bc_names=np.asarray(m.bc_names))
    r = load_mesh(p)
    np.testing.assert_array_equal(r.coords, m.coords)
    np.testing.assert_array_equal(r.elements, m.elements)
    np.testing.assert_array_equal(r.bfacets, m.bfacets)
    np.testing.assert_array_equal(r.blabels, m.blabels)
    assert r.bc_names == m.bc_names
    with pytest.raises(TypeError):
        load_mesh(os.path.join(str(tmp_path), 'sq.stl'))
