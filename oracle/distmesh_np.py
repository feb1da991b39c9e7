"""CPU restatement of the reference DistMesh path in float64 numpy.

TEST INFRASTRUCTURE ONLY: the parity checker of tests/, smoke() and the
timed CPU baseline of bench.py.  Connectivity comes from Qhull
(scipy.spatial.Delaunay) in place of CGAL, which cannot be built here; for
points in general position both give the unique Delaunay triangulation.

Each function names the reference code it restates (paths inside the
SeismicMesh project).
"""
import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
from scipy.spatial import Delaunay

EPS = np.finfo(float).eps


# ---------------------------------------------------------------------------
# initial points: generation/utils.py:15-25, generation/mesh_generator.py:808-852
def staggered_grid(h0, dim, bbox):
    g = np.mgrid[tuple(slice(lo, hi + h0, h0) for lo, hi in bbox)].astype(float)
    odd0 = np.arange(g[0].shape[0]) % 2 == 1
    odd1 = np.arange(g[1].shape[0]) % 2 == 1
    g[1][odd0] += h0 / 2
    if dim == 3:
        g[2][odd1] += h0 / 2
    return g.reshape(dim, -1).T


def initial_points(fd, fh, h0, bbox, geps, dim, pfix=None, seed=0, r0m_is_h0=False):
    p = staggered_grid(h0, dim, np.asarray(bbox).reshape(-1, 2))
    p = p[fd(p) < geps]
    r0 = fh(p)
    if r0m_is_h0:
        r0m = 1.1 * h0 if 1.1 * h0 < r0.min() else h0
    else:
        r0m = r0.min()
    np.random.seed(seed)
    keep = np.random.rand(p.shape[0]) < r0m**dim / r0**dim
    pf = np.empty((0, dim)) if pfix is None else np.asarray(pfix, dtype=float)
    return np.vstack((pf, p[keep]))


# ---------------------------------------------------------------------------
# connectivity: Qhull stands in for the CGAL rebuild
# (generation/mesh_generator.py:465-469)
def delaunay(p):
    return Delaunay(p).simplices.astype(np.int64)


def unique_edges(t):
    """_get_edges + unique_edges (mesh_generator.py:680-688,
    fast_geometry.cpp:30-77): sorted unique (min, max) pairs.  Each pair is
    one int64 key min * n + max, whose order is the lexicographic order of
    the pairs, so one integer sort does what the reference's std::sort of
    pairs does (a row-wise np.unique took ten times the reference's time).
    Sorting, then dropping repeats, is one tenth of np.unique's time on the
    18.7 M keys of the h = 0.02 ball."""
    dim = t.shape[1] - 1
    pairs = [(0, 1), (1, 2), (2, 0)] + ([(0, 3), (1, 3), (2, 3)] if dim == 3 else [])
    t = np.asarray(t, dtype=np.int64)
    if len(t) == 0:
        return np.zeros((0, 2), dtype=np.int64)
    n = int(t.max()) + 1
    i = np.concatenate([t[:, a] for a, _ in pairs])
    j = np.concatenate([t[:, b] for _, b in pairs])
    key = np.sort(np.minimum(i, j) * n + np.maximum(i, j))
    key = key[np.concatenate([[True], key[1:] != key[:-1]])]  # np.unique is slow here
    return np.stack([key // n, key % n], axis=1)


def remove_outside(p, t, fd, geps):
    """_remove_triangles_outside (mesh_generator.py:734-738)"""
    cen = p[t].sum(1) / (p.shape[1] + 1)
    return t[fd(cen) < -geps]


def bar_forces(p, t, fh, L0mult):
    """_compute_forces + dense scatter (mesh_generator.py:691-712,
    generation/utils.py:48-68)"""
    dim = p.shape[1]
    e = unique_edges(t)
    bar = p[e[:, 0]] - p[e[:, 1]]
    L = np.sqrt((bar**2).sum(1))
    L[L == 0] = EPS
    h = fh(p[e].sum(1) / 2)
    L0 = h * L0mult * ((L**dim).sum() / (h**dim).sum()) ** (1.0 / dim)
    F = np.maximum(L0 - L, 0.0)
    Fv = (F / L)[:, None] * bar
    Ftot = np.zeros_like(p)
    for k in range(dim):
        Ftot[:, k] += np.bincount(e[:, 0], weights=Fv[:, k], minlength=len(p))
        Ftot[:, k] -= np.bincount(e[:, 1], weights=Fv[:, k], minlength=len(p))
    return Ftot


def project_back(p, fd, deps, hmin, level):
    """_project_points_back_newton (mesh_generator.py:762-784): one Newton
    step with a one-sided finite-difference gradient"""
    dim = p.shape[1]
    d = fd(p)
    ix = d > 0.0 if level == 0 else np.logical_and(d > 0.0, d < hmin / 1.5)
    if ix.any():
        q = p[ix]
        g = np.empty((q.shape[0], dim))
        for k in range(dim):
            s = q.copy()
            s[:, k] += deps
            g[:, k] = (fd(s) - d[ix]) / deps
        g2 = (g**2).sum(1)
        g2 = np.where(g2 < deps, deps, g2)
        p[ix] = q - (d[ix] / g2)[:, None] * g
    return p


def one_iteration(p, fd, fh, h0, levels=None, nfix=0, delta_t=0.30, geps_mult=0.1, tri=None):
    """triangulate, filter, forces, update, project: the body of the
    generate_mesh loop (mesh_generator.py:460-527) for a fixed point order;
    tri: the triangulation stub (default Qhull; oracle.cdt.delaunay is the
    exact-predicate C++ one)"""
    dim = p.shape[1]
    L0mult = 1 + 0.4 / 2 ** (dim - 1)
    geps = geps_mult * h0
    deps = np.sqrt(EPS) * h0
    t = remove_outside(p, (tri or delaunay)(p), fd, geps)
    F = bar_forces(p, t, fh, L0mult)
    F[:nfix] = 0
    p = p + delta_t * F
    for i, lv in enumerate(levels or [fd]):
        p = project_back(p, lv, deps, h0, i)
    return p, t, F


# ---------------------------------------------------------------------------
# mesh utilities: geometry/utils.py
def simp_vol(p, t):
    """signed simplex volumes (geometry/utils.py:175-201)"""
    d = p[t[:, 1:]] - p[t[:, :1]]
    if p.shape[1] == 2:
        return (d[:, 0, 0] * d[:, 1, 1] - d[:, 0, 1] * d[:, 1, 0]) / 2
    return np.einsum("ij,ij->i", np.cross(d[:, 0], d[:, 1]), d[:, 2]) / 6


def simp_qual(p, t):
    """2 r / R of the triangle of the first three vertices (252-274)"""
    a = np.linalg.norm(p[t[:, 1]] - p[t[:, 0]], axis=1)
    b = np.linalg.norm(p[t[:, 2]] - p[t[:, 0]], axis=1)
    c = np.linalg.norm(p[t[:, 2]] - p[t[:, 1]], axis=1)
    r = 0.5 * np.sqrt((b + c - a) * (c + a - b) * (a + b - c) / (a + b + c))
    R = a * b * c / np.sqrt((a + b + c) * (b + c - a) * (c + a - b) * (a + b - c))
    return 2 * r / R


def boundary_facets(t):
    """facets of exactly one cell (310-326, 421-437)"""
    dim = t.shape[1] - 1
    f = np.concatenate([np.delete(t, k, axis=1) for k in range(dim + 1)])
    f = np.sort(f, axis=1)
    u, c = np.unique(f, axis=0, return_counts=True)
    return u[c == 1]


def boundary_vertices(t):
    return np.unique(boundary_facets(t).reshape(-1))


def fix_mesh(p, t, ptol=2e-13, delete_unused=False):
    """fix_mesh (204-249): merge near-duplicate vertices, drop duplicate
    cells, optionally unused vertices, orient positively"""
    snap = (p.max(0) - p.min(0)).max() * ptol
    _, ix, jx = np.unique(np.round(p / snap) * snap, axis=0, return_index=True, return_inverse=True)
    p = p[ix]
    t = np.asarray(jx).reshape(-1)[t]
    t = np.unique(np.sort(t, axis=1), axis=0)
    if delete_unused:
        used, inv = np.unique(t, return_inverse=True)
        t = inv.reshape(t.shape)
        p = p[used]
    flip = simp_vol(p, t) < 0
    t[flip, :2] = t[flip, 1::-1]
    return p, t


def delete_boundary_entities(p, t, min_qual):
    """cells touching a boundary vertex with quality < min_qual (440-469)"""
    q = simp_qual(p, t)
    bv = np.zeros(len(p), bool)
    bv[boundary_vertices(t)] = True
    kill = bv[t].any(1) & (q < min_qual)
    return fix_mesh(p, t[~kill], delete_unused=True)


def laplacian_fixed_point(p, t):
    """laplacian2_fixed_point (494-547) with a direct solve in place of AMG"""
    n = len(p)
    e = unique_edges(t)
    A = sp.coo_matrix(
        (np.ones(2 * len(e)), (np.r_[e[:, 0], e[:, 1]], np.r_[e[:, 1], e[:, 0]])), shape=(n, n)
    ).tocsr()
    deg = np.asarray(A.sum(1)).reshape(-1)
    L = (sp.diags(deg) - A).tolil()
    b = np.zeros((n, 2))
    bnd = boundary_vertices(t)
    for v in bnd:
        L.rows[v] = [v]
        L.data[v] = [1.0]
    b[bnd] = p[bnd]
    L = L.tocsc()
    return np.column_stack([spla.spsolve(L, b[:, 0]), spla.spsolve(L, b[:, 1])])


def improve_level_set(p, t, fd, deps):
    """_improve_level_set_newton (mesh_generator.py:741-759)"""
    dim = p.shape[1]
    bid = boundary_vertices(t)
    alpha = 1.0
    for it in range(5):
        q = p[bid]
        d = fd(q)
        g = np.empty((len(bid), dim))
        for k in range(dim):
            s = q.copy()
            s[:, k] += deps
            g[:, k] = (fd(s) - d) / deps
        g2 = (g**2).sum(1)
        g2 = np.where(g2 < deps, deps, g2)
        p[bid] = q - alpha * (d / g2)[:, None] * g
        alpha /= it + 1
    return p


def generate_mesh(fd, fh, h0, bbox, max_iter=50, seed=0, pfix=None, delta_t=0.30,
                  geps_mult=0.1, mesh_improvement=True, subdomains=None, points=None,
                  r0m_is_h0=False):
    """generate_mesh (mesh_generator.py:291-529), serial, Qhull connectivity.
    fd, fh: numpy callables.  Returns (p, t)."""
    dim = len(bbox) // 2
    geps = geps_mult * h0
    deps = np.sqrt(EPS) * h0
    nfix = 0 if pfix is None else len(pfix)
    if points is None:
        p = initial_points(fd, fh, h0, bbox, geps, dim, pfix, seed, r0m_is_h0)
    else:
        p = np.asarray(points, dtype=float)
    levels = [fd] + list(subdomains or [])
    L0mult = 1 + 0.4 / 2 ** (dim - 1)
    count = 0
    while True:
        t = remove_outside(p, delaunay(p), fd, geps)
        if count == max_iter - 1:
            break
        F = bar_forces(p, t, fh, L0mult)
        F[:nfix] = 0
        p = p + delta_t * F
        for i, lv in enumerate(levels):
            p = project_back(p, lv, deps, h0, i)
        assert delta_t * np.sqrt((F**2).sum(1)).max() < 1000 * h0
        count += 1
    if dim == 2:
        p, t = fix_mesh(p, t, delete_unused=True)
        p, t = delete_boundary_entities(p, t, 0.15)
        if subdomains is None and mesh_improvement:
            p = laplacian_fixed_point(p, t)
    p, t = fix_mesh(p, t, delete_unused=True)
    p = improve_level_set(p, t, fd, deps)
    t = remove_outside(p, t, fd, h0 * 0.001)
    return p, t


# ---------------------------------------------------------------------------
# sliver kernels: geometry/cpp/fast_geometry.cpp:351-418, 580-666
_DH_EDGES = ((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1))


def dihedral_angles(p, t):
    out = np.empty((len(t), 6))
    for i in range(6):
        e0, e1 = _DH_EDGES[i]
        o0, o1 = _DH_EDGES[5 - i]
        p0 = p[t[:, e0]]
        v1 = p[t[:, e1]] - p0
        v2 = p[t[:, o0]] - p0
        v3 = p[t[:, o1]] - p0
        v1 /= np.linalg.norm(v1, axis=1)[:, None]
        v2 /= np.linalg.norm(v2, axis=1)[:, None]
        v3 /= np.linalg.norm(v3, axis=1)[:, None]
        c12 = np.cross(v1, v2)
        c13 = np.cross(v1, v3)
        num = (v2 * v3).sum(1) - (v1 * v2).sum(1) * (v1 * v3).sum(1)
        out[:, i] = np.arccos(num / (np.linalg.norm(c12, axis=1) * np.linalg.norm(c13, axis=1)))
    return out.reshape(-1, 1)


def circumsphere_grad(p0, p1, p2, p3):
    """gradient of the squared circumradius w.r.t. p0, as the closed form
    derivative of |c|^2 with c the circumcentre of (p0, p1, p2) - p3"""
    x = np.stack([p0 - p3, p1 - p3, p2 - p3], axis=1)
    s = (x**2).sum(-1)
    a = np.linalg.det(x)
    # circumcentre numerator D = adj-based: c = D / (2 a)
    D = (s[:, 0, None] * np.cross(x[:, 1], x[:, 2]) + s[:, 1, None] * np.cross(x[:, 2], x[:, 0])
         + s[:, 2, None] * np.cross(x[:, 0], x[:, 1]))
    # d/dx0 of |D|^2 / (4 a^2): D depends on x0 through s0 and the two cross
    # products containing x0
    g = np.empty_like(p0)
    for k in range(3):
        dx0 = np.zeros_like(x[:, 0])
        dx0[:, k] = 1.0
        dD = (2 * x[:, 0, k, None] * np.cross(x[:, 1], x[:, 2]) + s[:, 2, None] * np.cross(dx0, x[:, 1])
              + s[:, 1, None] * np.cross(x[:, 2], dx0))
        da = np.einsum("ij,ij->i", dx0, np.cross(x[:, 1], x[:, 2]))
        g[:, k] = (D * dD).sum(1) / (2 * a**2) - da * (D**2).sum(1) / (2 * a**3)
    return g


def sliver_removal(p, fd, h0, max_iter=50, min_dh=10.0, max_dh=180.0, gamma=1.0, geps_mult=0.1):
    """sliver_removal (mesh_generator.py:59-288), Qhull connectivity"""
    geps = geps_mult * h0
    lo, hi = min_dh * math.pi / 180, max_dh * math.pi / 180
    step, old = 0.10, np.inf
    p = np.asarray(p, dtype=float).copy()
    for count in range(max_iter):
        t = remove_outside(p, delaunay(p), fd, geps)
        dh = dihedral_angles(p, t)[:, 0]
        bad = np.unique(np.nonzero((dh < lo) | (dh > hi))[0] // 6)
        if count == max_iter - 1:
            break
        if len(bad) == 0:
            return fix_mesh(p, t, delete_unused=True)
        g = circumsphere_grad(*(p[t[bad, k]] for k in range(4)))
        g[np.isinf(g)] = 1.0
        g /= np.sqrt((g**2).sum(1))[:, None]
        nb = len(bad)
        step = step / gamma if nb < old else (step * gamma if nb > old else step / 0.8)
        p[t[bad, 0]] += step * h0 * g
        old = nb
    return fix_mesh(p, t, delete_unused=True)


def jittered_ball_points(h, seed=0):
    """The reference's initial points of the unit ball at constant size h
    (initial_points: lattice, rejection, decimation) moved by a seeded
    U(-1e-3 h, 1e-3 h) per coordinate and rounded to float32: a generic
    start, where every Delaunay triangulation of the run is unique."""
    from . import sdf_np as S

    fd = S.ball(0.0, 0.0, 0.0, 1.0)
    p0 = initial_points(fd, lambda x: np.full(len(x), h), h, (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0),
                        0.1 * h, 3)
    rng = np.random.default_rng(seed)
    return (p0 + rng.uniform(-1e-3 * h, 1e-3 * h, p0.shape)).astype(np.float32).astype(np.float64)
