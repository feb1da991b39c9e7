"""The exact-predicate C++ Delaunay tetrahedralisation (oracle/cdt3.cpp)
through ctypes.

TEST INFRASTRUCTURE ONLY: the second triangulation stub of the oracle's
reference loop (the CPU baseline of bench.py), in place of the CGAL rebuild
of the reference (generation/mesh_generator.py:465-469), beside Qhull; and
its tests.  Built by oracle/build.py (g++, no GPU).
"""
import ctypes

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_cdt()
        if path is None:
            raise RuntimeError("the C++ triangulator (oracle/cdt3.cpp) could not be built")
        L = ctypes.CDLL(path)
        P = ctypes.POINTER(ctypes.c_double)
        L.cdt3_delaunay.restype = ctypes.c_int64
        L.cdt3_delaunay.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64]
        L.cdt3_orient4.restype = ctypes.c_int
        L.cdt3_orient4.argtypes = [P] * 4
        L.cdt3_insphere.restype = ctypes.c_int
        L.cdt3_insphere.argtypes = [P] * 5
        L.cdt3_insphere_sos.restype = ctypes.c_int
        L.cdt3_insphere_sos.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib = L
    return _lib


def available():
    try:
        lib()
        return True
    except (RuntimeError, OSError):
        return False


def delaunay(p):
    """tetrahedra (m, 4) int64 of the points p (n, 3); exact duplicates of an
    earlier point (in insertion order) are left out, as Qhull leaves them"""
    p = np.ascontiguousarray(p, dtype=np.float64)
    if p.ndim != 2 or p.shape[1] != 3:
        raise ValueError("points must be (n, 3)")
    cap = 7 * len(p) + 64
    while True:
        out = np.empty((cap, 4), dtype=np.int32)
        m = lib().cdt3_delaunay(p.ctypes.data, len(p), out.ctypes.data, cap)
        if m >= 0:
            return out[:m].astype(np.int64)
        if m <= -(1 << 41):
            raise RuntimeError(f"cdt3_delaunay failed (code {m})")
        cap = -m


def _ptr(x):
    return np.ascontiguousarray(x, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def orient4(a, b, c, d):
    """sign of det[[x y z 1]] over the rows a, b, c, d (exact)"""
    arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c, d)]
    return lib().cdt3_orient4(*[_ptr(v) for v in arrs])


def insphere(a, b, c, d, e):
    """sign of det[[x - e, |x - e|^2]] over the rows x = a, b, c, d (exact):
    for orient4(a, b, c, d) > 0, positive iff e lies inside the sphere"""
    arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c, d, e)]
    return lib().cdt3_insphere(*[_ptr(v) for v in arrs])


def insphere_sos(xyz, v, ie):
    """insphere of the points xyz[v] and xyz[ie] with the lifted coordinate
    perturbed by point index (never 0 unless all five are coplanar)"""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.int32)
    return lib().cdt3_insphere_sos(xyz.ctypes.data, v.ctypes.data, int(ie))
