"""Mesh quality and linting checks in plain Python/numpy (test
infrastructure, small meshes only).

Restates geometry/utils.py of the reference: calc_re_ratios (17-54),
vertex_to_entities (97-130), vertex_in_entity2 (657-679), vertex_in_entity3
(682-726) with calc_4x4determinant (geometry/cpp/fast_geometry.cpp:482-495),
get_centroids (729-742) and do_any_overlap (745-817).  Python floats are
IEEE doubles and every expression keeps the reference's operation order, so
the overlap decisions are the reference's bit for bit.
"""
import numpy as np


def circumradius(x):
    """circumradius of the simplex with vertex rows x[dim + 1, dim]"""
    a = x[1:] - x[0]
    rhs = 0.5 * (a * a).sum(1)
    return float(np.linalg.norm(np.linalg.solve(a, rhs)))


def calc_re_ratios(p, t, dim=2):
    """circumradius / shortest edge of every cell"""
    out = np.empty(len(t))
    for i, c in enumerate(t):
        x = p[c]
        e = min(np.linalg.norm(x[a] - x[b]) for a in range(dim + 1) for b in range(a + 1, dim + 1))
        out[i] = circumradius(x) / e
    return out


def det4x4(m):
    """the 24-term expansion, products and sums left to right"""
    terms = (
        (12, 9, 6, 3, 1), (8, 13, 6, 3, -1), (12, 5, 10, 3, -1), (4, 13, 10, 3, 1),
        (8, 5, 14, 3, 1), (4, 9, 14, 3, -1), (12, 9, 2, 7, -1), (8, 13, 2, 7, 1),
        (12, 1, 10, 7, 1), (0, 13, 10, 7, -1), (8, 1, 14, 7, -1), (0, 9, 14, 7, 1),
        (12, 5, 2, 11, 1), (4, 13, 2, 11, -1), (12, 1, 6, 11, -1), (0, 13, 6, 11, 1),
        (4, 1, 14, 11, 1), (0, 5, 14, 11, -1), (8, 5, 2, 15, -1), (4, 9, 2, 15, 1),
        (8, 1, 6, 15, 1), (0, 9, 6, 15, -1), (4, 1, 10, 15, -1), (0, 5, 10, 15, 1),
    )
    s = 0.0
    for k, (a, b, c, d, sg) in enumerate(terms):
        v = m[a] * m[b] * m[c] * m[d]
        s = v if k == 0 else (s + v if sg > 0 else s - v)
    return s


def _sign(v):
    return 1 if v > 0 else (-1 if v < 0 else 0)


def inside2(q, x):
    (x_, y_), (x1, y1), (x2, y2), (x3, y3) = q, x[0], x[1], x[2]
    den = (y2 - y3) * (x1 - x3) + (x3 - x2) * (y1 - y3)
    with np.errstate(all="ignore"):
        a = np.float64((y2 - y3) * (x_ - x3) + (x3 - x2) * (y_ - y3)) / den
        b = np.float64((y3 - y1) * (x_ - x3) + (x1 - x3) * (y_ - y3)) / den
    c = 1 - a - b
    return bool(0 <= a <= 1 and 0 <= b <= 1 and 0 <= c <= 1)


def inside3(q, x):
    rows = [[float(v) for v in r] + [1.0] for r in x]
    s0 = _sign(det4x4([v for r in rows for v in r]))
    prev = s0
    for r in range(4):
        m = [list(row) for row in rows]
        m[r] = [float(v) for v in q] + [1.0]
        s = _sign(det4x4([v for row in m for v in row]))
        if s != prev:
            return False
        prev = s
    return s0 != 0


def do_any_overlap(p, t, dim=2):
    """(ie, ele) once per shared vertex, ordered by ie, vertex slot, ele"""
    p = np.asarray(p, dtype=np.float64)
    rows = [[] for _ in range(len(p))]
    for ie, c in enumerate(t):
        for v in c:
            rows[v].append(ie)
    cent = p[t].sum(1) / (dim + 1)
    inside = inside2 if dim == 2 else inside3
    out = []
    for ie, c in enumerate(t):
        for v in c:
            for ele in rows[v]:
                if ele != ie and inside(cent[ie], p[t[ele]]):
                    out.append((ie, ele))
    return out


def cell_quality(p, t):
    """dim * inradius / circumradius and (3D) min sin dihedral / (2 sqrt(2) / 3),
    per cell, from the textbook formulas (meshplex, the package the reference
    benchmark reports use, is not vendored in the reference)"""
    p = np.asarray(p, dtype=np.float64)
    dim = p.shape[1]
    q = np.empty(len(t))
    s = np.empty(len(t)) if dim == 3 else None
    for c, cell in enumerate(t):
        x = p[cell]
        R = circumradius(x)
        if dim == 2:
            l = [np.linalg.norm(x[(k + 1) % 3] - x[(k + 2) % 3]) for k in range(3)]
            u, w = x[1] - x[0], x[2] - x[0]
            area = 0.5 * abs(u[0] * w[1] - u[1] * w[0])
            q[c] = 2 * (2 * area / sum(l)) / R
        else:
            A = [0.5 * np.linalg.norm(np.cross(*(x[[j for j in range(4) if j != k][1:]]
                                                  - x[[j for j in range(4) if j != k][0]])))
                 for k in range(4)]
            V = abs(np.linalg.det(x[1:] - x[0])) / 6
            q[c] = 3 * (3 * V / sum(A)) / R
            sines = []
            for i in range(4):
                for j in range(i + 1, 4):
                    k, l2 = [m for m in range(4) if m not in (i, j)]
                    sines.append(3 * V * np.linalg.norm(x[i] - x[j]) / (2 * A[k] * A[l2]))
            s[c] = min(sines) / (2 * np.sqrt(2) / 3)
    return q, s


def cell_quality_vec(p, t):
    """Vectorised cell_quality for large meshes: the same textbook measures,
    dim * inradius / circumradius and (3D) the minimum sine of the dihedral
    angles normalised to the regular tetrahedron, in float64."""
    p = np.asarray(p, dtype=np.float64)
    t = np.asarray(t, dtype=np.int64)
    dim = p.shape[1]
    x = p[t]                                     # [m, dim+1, dim]
    a = x[:, 1:] - x[:, :1]
    rhs = 0.5 * (a * a).sum(-1)
    R = np.linalg.norm(np.linalg.solve(a, rhs[..., None])[..., 0], axis=1)
    if dim == 2:
        l = [np.linalg.norm(x[:, (k + 1) % 3] - x[:, (k + 2) % 3], axis=1) for k in range(3)]
        area = 0.5 * np.abs(a[:, 0, 0] * a[:, 1, 1] - a[:, 0, 1] * a[:, 1, 0])
        return 2 * (2 * area / sum(l)) / R, None
    faces = [[j for j in range(4) if j != k] for k in range(4)]
    A = [0.5 * np.linalg.norm(np.cross(x[:, f[1]] - x[:, f[0]], x[:, f[2]] - x[:, f[0]]), axis=1)
         for f in faces]
    V = np.abs(np.linalg.det(a)) / 6
    q = 3 * (3 * V / sum(A)) / R
    s = np.full(len(t), np.inf)
    for i in range(4):
        for j in range(i + 1, 4):
            k, l2 = [m for m in range(4) if m not in (i, j)]
            s = np.minimum(s, 3 * V * np.linalg.norm(x[:, i] - x[:, j], axis=1) / (2 * A[k] * A[l2]))
    return q, s / (2 * np.sqrt(2) / 3)
