"""Delaunay oracle (test infrastructure).

The reference triangulates with CGAL (generation/cpp/delaunay_class.cpp,
delaunay_class3.cpp), which is not buildable here.  For points in general
position the Delaunay triangulation is unique, so Qhull (scipy.spatial.Delaunay,
an independent implementation) is the connectivity oracle; cells are
compared after canonical ordering (sorted vertices, sorted rows).
"""
import numpy as np
from scipy.spatial import Delaunay


def canonical(cells):
    c = np.sort(np.asarray(cells, dtype=np.int64), axis=1)
    if len(c) == 0:
        return c
    order = np.lexsort(c.T[::-1])
    return c[order]


def qhull_cells(p):
    # Qt: triangulated output; Qbb/Qc/Qz as scipy's defaults for d>=3
    return Delaunay(np.asarray(p, dtype=np.float64)).simplices


def assert_same_triangulation(p, cells):
    a = canonical(cells)
    b = canonical(qhull_cells(p))
    if a.shape != b.shape or not np.array_equal(a, b):
        sa = {tuple(r) for r in a}
        sb = {tuple(r) for r in b}
        raise AssertionError(
            f"triangulations differ: gpu {len(a)} cells, oracle {len(b)} cells, "
            f"{len(sa - sb)} only on gpu, {len(sb - sa)} only in oracle"
        )
