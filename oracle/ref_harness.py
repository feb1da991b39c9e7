"""Runs the reference SeismicMesh Python package in this container.

TEST INFRASTRUCTURE ONLY (fixture generation and oracle validation); it
needs the reference sources and cannot run on a machine without them.

The reference imports modules that cannot be installed here:
  * mpi4py                  -> a size-1 communicator (serial path)
  * matplotlib              -> empty modules (plotting only)
  * pyamg                   -> ruge_stuben_solver(A).solve(b) by a direct sparse solve
  * _delaunay_class(3)      -> CGAL triangulations; stood in for by Qhull
                               (scipy.spatial.Delaunay), duplicates merged;
                               in 3D optionally by the oracle's exact-predicate
                               C++ Delaunay (use_cpp_triangulator)
  * _delaunay, _cpputils    -> CGAL helpers off the serial hot path
  * _fast_geometry, _FastHJ -> built from the reference's own C++ sources
                               (oracle/Makefile -> oracle/_ref/)
and geometry/utils.py:157 uses np.character, removed in numpy 2, so
unique_rows is replaced by the equivalent np.unique(axis=0) call.
"""
import os
import subprocess
import sys
import types

import numpy as np
import scipy.sparse.linalg as spla
from scipy.spatial import Delaunay

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: $SEISMICMESH_REF, else `reference` beside this repository
REF = os.environ.get("SEISMICMESH_REF",
                     os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
REF_BUILD = os.path.join(HERE, "_ref")


def build_ref():
    subprocess.run(["make", "-s", "-C", HERE, f"REF={REF}"], check=True)


class _Comm:
    rank = 0
    size = 1

    def bcast(self, x, root=0):
        return x

    def allreduce(self, x, op=None):
        return x

    def Barrier(self):
        pass


def _install_stubs():
    mpi4py = types.ModuleType("mpi4py")
    MPI = types.ModuleType("mpi4py.MPI")
    MPI.COMM_WORLD = _Comm()
    MPI.Intracomm = _Comm
    MPI.MIN = "min"
    MPI.SUM = "sum"
    mpi4py.MPI = MPI
    sys.modules["mpi4py"] = mpi4py
    sys.modules["mpi4py.MPI"] = MPI

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt

    pyamg = types.ModuleType("pyamg")

    class _Solver:
        def __init__(self, A):
            self.A = A.tocsc()

        def solve(self, b):
            return spla.spsolve(self.A, b)

    pyamg.ruge_stuben_solver = lambda A: _Solver(A)
    sys.modules["pyamg"] = pyamg

    class _DT:
        dim = 2

        def __init__(self):
            self.p = np.zeros((0, self.dim))

        def insert(self, flat):
            q = np.asarray(flat, dtype=float).reshape(-1, self.dim)
            self.p = np.vstack((self.p, q))
            # CGAL keeps one vertex per location (the first)
            self.p = self.p[_first_occurrences(self.p)]

        def move(self, ids, flat):
            q = np.asarray(flat, dtype=float).reshape(-1, self.dim)
            self.p[np.asarray(ids, dtype=int)] = q

        def remove(self, ids):
            self.p = np.delete(self.p, np.asarray(ids, dtype=int), axis=0)

        def number_of_vertices(self):
            return len(self.p)

        def get_finite_vertices(self):
            return self.p.copy()

        def get_finite_cells(self):
            if self.dim == 3 and _tri3 is not None:
                return _tri3(self.p).astype(np.int32)
            return Delaunay(self.p).simplices.astype(np.int32)

    class DT2(_DT):
        dim = 2

    class DT3(_DT):
        dim = 3

    m2 = types.ModuleType("_delaunay_class")
    m2.DelaunayTriangulation = DT2
    m3 = types.ModuleType("_delaunay_class3")
    m3.DelaunayTriangulation3 = DT3
    sys.modules["_delaunay_class"] = m2
    sys.modules["_delaunay_class3"] = m3

    md = types.ModuleType("_delaunay")

    def _circumballs(p, dim):
        p = np.asarray(p, dtype=float).reshape(-1, dim + 1, dim)
        A = 2 * (p[:, 1:] - p[:, :1])
        b = (p[:, 1:] ** 2).sum(-1) - (p[:, :1] ** 2).sum(-1)
        c = np.linalg.solve(A, b[..., None])[..., 0]
        r2 = ((p[:, 0] - c) ** 2).sum(-1)
        return np.column_stack((c, r2))

    md._circumballs2 = lambda p: _circumballs(p, 2)
    md._circumballs3 = lambda p: _circumballs(p, 3)
    md._delaunay2 = lambda x, y: Delaunay(np.column_stack((x, y))).simplices
    md._delaunay3 = lambda x, y, z: Delaunay(np.column_stack((x, y, z))).simplices
    sys.modules["_delaunay"] = md
    sys.modules["_cpputils"] = types.ModuleType("_cpputils")


_loaded = None
_tri3 = None  # 3D triangulation stub: None for Qhull, else points -> tetrahedra


def use_cpp_triangulator(on=True):
    """Triangulate 3D sets with the oracle's exact-predicate C++ Delaunay
    (oracle/cdt3.cpp) in CGAL's place instead of Qhull."""
    global _tri3
    if on:
        from . import cdt

        _tri3 = cdt.delaunay
    else:
        _tri3 = None


def _first_occurrences(p):
    """mask of the rows of p that equal no earlier row (what CGAL keeps)"""
    if len(p) < 2:
        return np.ones(len(p), dtype=bool)
    order = np.lexsort(p.T[::-1])  # stable: equal rows keep their input order
    s = p[order]
    later = np.zeros(len(p), dtype=bool)
    later[order[1:]] = np.all(s[1:] == s[:-1], axis=1)
    return ~later


def load():
    """Import and return the reference SeismicMesh package."""
    global _loaded
    if _loaded is not None:
        return _loaded
    build_ref()
    _install_stubs()
    sys.path.insert(0, REF_BUILD)
    sys.path.insert(0, REF)
    import SeismicMesh  # noqa: E402
    from SeismicMesh.geometry import utils as gu

    def unique_rows(A, return_index=False, return_inverse=False):
        A = np.require(A, requirements="C")
        B, I, J = np.unique(A, axis=0, return_index=True, return_inverse=True)
        J = np.asarray(J).reshape(-1)
        if return_index and return_inverse:
            return B, I, J
        if return_index:
            return B, I
        if return_inverse:
            return B, J
        return B

    gu.unique_rows = unique_rows
    _loaded = SeismicMesh
    return SeismicMesh
