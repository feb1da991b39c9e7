"""Mesh output: legacy VTK unstructured grids (binary), so meshes made on the
GPU can be inspected offline (the reference writes through meshio in its
tests and examples).  Triangles (VTK type 5) and tetrahedra (type 10)."""
import numpy as np

_TYPES = {3: 5, 4: 10}


def write_vtk(filename, points, cells, cell_data=None):
    """Write points (n, 2|3) and cells (m, 3|4) as a binary legacy VTK file;
    cell_data: optional {name: (m,) float array}."""
    p = np.asarray(points, dtype=np.float64)
    t = np.asarray(cells, dtype=np.int64)
    if p.ndim != 2 or p.shape[1] not in (2, 3) or t.ndim != 2 or t.shape[1] not in _TYPES:
        raise ValueError("points must be (n, 2|3) and cells (m, 3|4)")
    if p.shape[1] == 2:
        p = np.column_stack([p, np.zeros(len(p))])
    p = p.astype(">f8")  # legacy VTK binary data is big-endian
    nv = t.shape[1]
    with open(filename, "wb") as fh:
        fh.write(b"# vtk DataFile Version 3.0\nseismicmesh_gb300 mesh\nBINARY\nDATASET UNSTRUCTURED_GRID\n")
        fh.write(f"POINTS {len(p)} double\n".encode())
        fh.write(np.ascontiguousarray(p).tobytes())
        fh.write(f"\nCELLS {len(t)} {len(t) * (nv + 1)}\n".encode())
        conn = np.column_stack([np.full(len(t), nv, dtype=np.int64), t]).astype(">i4")
        fh.write(np.ascontiguousarray(conn).tobytes())
        fh.write(f"\nCELL_TYPES {len(t)}\n".encode())
        fh.write(np.full(len(t), _TYPES[nv], dtype=">i4").tobytes())
        if cell_data:
            fh.write(f"\nCELL_DATA {len(t)}\n".encode())
            for name, vals in cell_data.items():
                v = np.asarray(vals, dtype=">f8").reshape(-1)
                fh.write(f"SCALARS {name} double 1\nLOOKUP_TABLE default\n".encode())
                fh.write(v.tobytes())
                fh.write(b"\n")


def read_vtk(filename):
    """Read back a file written by write_vtk: (points (n, 3), cells (m, k))."""
    data = open(filename, "rb").read()

    def header(tag, start):
        i = data.index(tag, start)
        j = data.index(b"\n", i)
        return data[i:j].split(), j + 1

    h, pos = header(b"POINTS", 0)
    n = int(h[1])
    pts = np.frombuffer(data[pos:pos + 24 * n], dtype=">f8").reshape(n, 3).astype(float)
    h, pos = header(b"CELLS", pos + 24 * n)
    m, size = int(h[1]), int(h[2])
    conn = np.frombuffer(data[pos:pos + 4 * size], dtype=">i4").reshape(m, -1)
    return pts, conn[:, 1:].astype(np.int64)


_GMSH_TYPES = {3: 2, 4: 4}  # triangle, tetrahedron


def write_gmsh22(filename, points, cells):
    """Write an ASCII gmsh 2.2 mesh (the README's file_format="gmsh22");
    node and element tags are 1-based."""
    p = np.asarray(points, dtype=np.float64)
    t = np.asarray(cells, dtype=np.int64)
    if t.ndim != 2 or t.shape[1] not in _GMSH_TYPES:
        raise ValueError("cells must be (m, 3|4)")
    if p.shape[1] == 2:
        p = np.column_stack([p, np.zeros(len(p))])
    et = _GMSH_TYPES[t.shape[1]]
    with open(filename, "w") as fh:
        fh.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(p))
        np.savetxt(fh, np.column_stack([np.arange(1, len(p) + 1), p]), fmt=["%d", "%.17g", "%.17g", "%.17g"])
        fh.write("$EndNodes\n$Elements\n%d\n" % len(t))
        rows = np.column_stack([np.arange(1, len(t) + 1), np.full(len(t), et), np.full(len(t), 2),
                                np.zeros(len(t), dtype=np.int64), np.zeros(len(t), dtype=np.int64), t + 1])
        np.savetxt(fh, rows, fmt="%d")
        fh.write("$EndElements\n")


def read_gmsh22(filename):
    """Read back a file written by write_gmsh22: (points (n, 3), cells (m, k))."""
    lines = open(filename).read().split("\n")
    i = lines.index("$Nodes")
    n = int(lines[i + 1])
    pts = np.array([ln.split()[1:] for ln in lines[i + 2:i + 2 + n]], dtype=float)
    j = lines.index("$Elements")
    m = int(lines[j + 1])
    el = [ln.split() for ln in lines[j + 2:j + 2 + m]]
    cells = np.array([[int(v) - 1 for v in e[3 + int(e[2]):]] for e in el], dtype=np.int64)
    return pts, cells


def write_mesh(filename, points, cells, cell_data=None):
    """Write by extension: .vtk (binary legacy VTK) or .msh (gmsh 2.2)."""
    if filename.endswith(".vtk"):
        write_vtk(filename, points, cells, cell_data)
    elif filename.endswith(".msh"):
        write_gmsh22(filename, points, cells)
    else:
        raise ValueError("unknown mesh format (use .vtk or .msh): " + filename)
