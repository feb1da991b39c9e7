"""Mesh writers (seismicmesh_gb300.io) against known-answer files built here
from the published formats, not from the writers' own readers:

* legacy VTK, binary: ASCII header lines, then big-endian float64 point
  triples, big-endian int32 cell records (vertex count, then the 0-based
  vertex ids) and big-endian int32 cell types (5 triangle, 10 tetrahedron),
  each block starting on a new line;
* gmsh 2.2 ASCII: $MeshFormat "2.2 0 8", $Nodes with 1-based tags and three
  coordinates, $Elements with "tag type ntags tags... nodes..." (type 2
  triangle, 4 tetrahedron; two tags, physical and elementary, both 0).
"""
import struct

import numpy as np
import pytest

from seismicmesh_gb300.io import read_gmsh22, write_gmsh22, write_mesh, write_vtk

P2 = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 0.5]])
T2 = np.array([[0, 1, 2], [0, 2, 3]])


def _vtk_bytes(points3, cells, ctype):
    out = b"# vtk DataFile Version 3.0\nseismicmesh_gb300 mesh\nBINARY\nDATASET UNSTRUCTURED_GRID\n"
    out += b"POINTS %d double\n" % len(points3)
    for x in points3:
        out += struct.pack(">ddd", *x)
    k = len(cells[0])
    out += b"\nCELLS %d %d\n" % (len(cells), len(cells) * (k + 1))
    for c in cells:
        out += struct.pack(">%di" % (k + 1), k, *c)
    out += b"\nCELL_TYPES %d\n" % len(cells)
    out += struct.pack(">%di" % len(cells), *([ctype] * len(cells)))
    return out


def test_vtk_triangles_known_answer(tmp_path):
    f = tmp_path / "t.vtk"
    write_vtk(str(f), P2, T2)
    p3 = [(x, y, 0.0) for x, y in P2]
    assert f.read_bytes() == _vtk_bytes(p3, T2.tolist(), 5)


def test_vtk_tetrahedron_with_cell_data_known_answer(tmp_path):
    p = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    t = np.array([[0, 1, 2, 3]])
    f = tmp_path / "k.vtk"
    write_vtk(str(f), p, t, cell_data={"quality": [0.75]})
    want = _vtk_bytes(p.tolist(), t.tolist(), 10)
    want += b"\nCELL_DATA 1\nSCALARS quality double 1\nLOOKUP_TABLE default\n"
    want += struct.pack(">d", 0.75) + b"\n"
    assert f.read_bytes() == want


def test_gmsh22_known_answer(tmp_path):
    f = tmp_path / "t.msh"
    write_gmsh22(str(f), P2, T2)
    want = (
        "$MeshFormat\n2.2 0 8\n$EndMeshFormat\n"
        "$Nodes\n4\n1 0 0 0\n2 1 0 0\n3 1 1 0\n4 0 0.5 0\n$EndNodes\n"
        "$Elements\n2\n1 2 2 0 0 1 2 3\n2 2 2 0 0 1 3 4\n$EndElements\n"
    )
    assert f.read_text() == want


def test_gmsh22_reader_on_a_file_written_by_hand(tmp_path):
    """a tetrahedron with three tags per element and a trailing blank line,
    as other writers produce it"""
    f = tmp_path / "h.msh"
    f.write_text(
        "$MeshFormat\n2.2 0 8\n$EndMeshFormat\n"
        "$Nodes\n4\n1 0 0 0\n2 2.5 0 0\n3 0 1 0\n4 0 0 -1\n$EndNodes\n"
        "$Elements\n1\n1 4 3 7 1 0 1 2 4 3\n$EndElements\n\n"
    )
    p, t = read_gmsh22(str(f))
    np.testing.assert_array_equal(p, [[0, 0, 0], [2.5, 0, 0], [0, 1, 0], [0, 0, -1]])
    np.testing.assert_array_equal(t, [[0, 1, 3, 2]])


def test_write_mesh_dispatches_on_the_extension(tmp_path):
    write_mesh(str(tmp_path / "a.vtk"), P2, T2)
    write_mesh(str(tmp_path / "a.msh"), P2, T2)
    assert (tmp_path / "a.vtk").read_bytes() == _vtk_bytes([(x, y, 0.0) for x, y in P2], T2.tolist(), 5)
    assert (tmp_path / "a.msh").read_text().startswith("$MeshFormat\n2.2 0 8\n")
    with pytest.raises(ValueError, match="unknown mesh format"):
        write_mesh(str(tmp_path / "a.obj"), P2, T2)
