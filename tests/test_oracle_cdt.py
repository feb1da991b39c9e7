"""The oracle's exact-predicate C++ triangulator (oracle/cdt3.cpp), the second
triangulation stub of the reference loop's CPU baseline:

* on points in general position it returns Qhull's tetrahedra exactly;
* on degenerate lattices (DistMesh's initial points, cubic grids) it returns
  a Delaunay tiling: every tetrahedron has positive volume, the volumes add
  up to the convex hull's, and no point lies strictly inside a circumsphere
  (checked with its exact in-sphere predicate, itself checked against
  rational arithmetic);
* exact duplicates are left out;
* degenerate inputs (too few, coplanar, collinear, coincident points) give
  no tetrahedra, and points far from the origin, where Qhull's floating
  point fails, still give an exact tiling.
"""
from fractions import Fraction

import numpy as np
import pytest
from scipy.spatial import ConvexHull, Delaunay, cKDTree

from oracle import cdt
from oracle import distmesh_np as O
from oracle import sdf_np as S

pytestmark = pytest.mark.skipif(not cdt.available(), reason="no C++ compiler for oracle/cdt3.cpp")


def _canon(t):
    t = np.sort(np.asarray(t), axis=1)
    return t[np.lexsort(t.T[::-1])]


@pytest.mark.parametrize("kind", ["cube", "gauss", "ball"])
def test_equals_qhull_on_generic_points(kind):
    rng = np.random.default_rng({"cube": 1, "gauss": 2, "ball": 3}[kind])
    if kind == "cube":
        p = rng.random((3000, 3))
    elif kind == "gauss":
        p = np.concatenate([rng.normal(c, 0.05, size=(600, 3)) for c in rng.random((5, 3))])
    else:
        x = rng.normal(size=(2500, 3))
        p = x / np.linalg.norm(x, axis=1)[:, None] * rng.random((2500, 1)) ** (1 / 3)
    np.testing.assert_array_equal(_canon(cdt.delaunay(p)), _canon(Delaunay(p).simplices))


def _det(rows):
    """exact determinant of a small matrix of Fractions (Laplace expansion)"""
    n = len(rows)
    if n == 1:
        return rows[0][0]
    return sum((-1) ** j * rows[0][j] * _det([r[:j] + r[j + 1:] for r in rows[1:]]) for j in range(n))


def _orient4_q(a, b, c, d):
    return _det([[Fraction(x) for x in v] + [Fraction(1)] for v in (a, b, c, d)])


def _insphere_q(a, b, c, d, e):
    E = [Fraction(x) for x in e]
    rows = []
    for v in (a, b, c, d):
        r = [Fraction(x) - y for x, y in zip(v, E)]
        rows.append(r + [sum(t * t for t in r)])
    return _det(rows)


def _sign(x):
    return (x > 0) - (x < 0)


def test_predicates_match_rational_arithmetic():
    rng = np.random.default_rng(4)
    cases = []
    # generic, large-offset and 1-ulp-perturbed near-degenerate configurations
    for _ in range(60):
        cases.append(rng.random((5, 3)))
        cases.append(rng.random((5, 3)) * 1e-3 + 1e3)
    cube = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1],
                     [0, 1, 1], [1, 1, 1]], dtype=float)
    for _ in range(60):
        q = cube[rng.permutation(8)[:5]] * 0.1 + 0.3  # cospherical / coplanar subsets
        cases.append(q)
        q2 = q.copy()
        i, k = rng.integers(5), rng.integers(3)
        q2[i, k] = np.nextafter(q2[i, k], np.inf)
        cases.append(q2)
    zeros = 0
    for q in cases:
        a, b, c, d, e = q
        so = cdt.orient4(a, b, c, d)
        assert so == _sign(_orient4_q(a, b, c, d))
        si = cdt.insphere(a, b, c, d, e)
        assert si == _sign(_insphere_q(a, b, c, d, e))
        zeros += si == 0
    assert zeros > 10  # the degenerate cases were exercised


def _check_tiling(p, t):
    """positive volumes, volumes adding up to the hull, empty circumspheres"""
    vol = 0.0
    tree = cKDTree(p)
    for tet in t:
        s = cdt.orient4(*p[tet])
        assert s != 0
        if s < 0:
            tet = tet[[1, 0, 2, 3]]
        X = p[tet]
        vol += abs(np.linalg.det(X[1:] - X[0])) / 6
        A = 2 * (X[1:] - X[0])
        rhs = (X[1:] ** 2).sum(1) - (X[0] ** 2).sum()
        cen = np.linalg.solve(A, rhs)
        r = np.sqrt(((X[0] - cen) ** 2).sum())
        for j in tree.query_ball_point(cen, r * (1 + 1e-6) + 1e-12):
            if j in tet:
                continue
            assert cdt.insphere(*X, p[j]) <= 0, (tet, j)
    hv = ConvexHull(p).volume
    assert abs(vol - hv) <= 1e-9 * hv, (vol, hv)


def test_delaunay_tiling_of_degenerate_lattices():
    # a cubic grid: every cell's corners are cospherical
    g = np.stack(np.meshgrid(*[np.arange(5.0)] * 3, indexing="ij"), -1).reshape(-1, 3) * 0.25
    t = cdt.delaunay(g)
    _check_tiling(g, t)
    assert set(np.unique(t)) == set(range(len(g)))
    # DistMesh's staggered initial lattice of the unit ball
    h = 0.2
    fd = S.ball(0.0, 0.0, 0.0, 1.0)
    p = O.initial_points(fd, lambda x: np.full(len(x), h), h, (-1, 1, -1, 1, -1, 1), 0.1 * h, 3)
    t = cdt.delaunay(p)
    _check_tiling(p, t)
    assert set(np.unique(t)) == set(range(len(p)))


def test_perturbed_insphere_decides_cospherical_ties():
    """the five corners of a cube face plus one are cospherical: the plain
    predicate is 0, the perturbed one is not, and it depends only on the
    indices (the same configuration under other labels gives a consistent
    sign)"""
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], dtype=float)
    v = [0, 1, 2, 3]
    if cdt.orient4(*xyz[v]) < 0:
        v = [1, 0, 2, 3]
    assert cdt.insphere(*xyz[v], xyz[4]) == 0
    s = cdt.insphere_sos(xyz, v, 4)
    assert s in (-1, 1)
    assert cdt.insphere_sos(xyz, [v[1], v[0], v[2], v[3]], 4) == -s  # odd permutation


def test_duplicates_are_left_out():
    rng = np.random.default_rng(6)
    p = rng.random((400, 3))
    q = np.concatenate([p, p[:50]])  # points 400..449 repeat 0..49
    t = cdt.delaunay(q)
    assert t.max() < 400
    np.testing.assert_array_equal(_canon(t), _canon(cdt.delaunay(p)))


def test_oracle_iteration_with_the_cpp_stub():
    """the oracle's loop body runs with either stub; from a generic point
    set both give the same next positions"""
    h = 0.1
    fd = S.ball(0.0, 0.0, 0.0, 1.0)
    fh = lambda x: np.full(len(x), h)  # noqa: E731
    rng = np.random.default_rng(7)
    x = rng.normal(size=(3000, 3))
    p = x / np.linalg.norm(x, axis=1)[:, None] * rng.random((3000, 1)) ** (1 / 3)
    a, _, _ = O.one_iteration(p.copy(), fd, fh, h)
    b, _, _ = O.one_iteration(p.copy(), fd, fh, h, tri=cdt.delaunay)
    np.testing.assert_array_equal(a, b)


def test_degenerate_and_far_inputs():
    """fewer than four points, coplanar, collinear and coincident sets give
    no tetrahedra (and no error); points a million units from the origin
    with unit spread, where Qhull's floating point breaks down, still give an
    exact Delaunay tiling"""
    rng = np.random.default_rng(3)
    for n in range(4):
        assert len(cdt.delaunay(rng.random((n, 3)))) == 0
    assert len(cdt.delaunay(np.c_[rng.random((50, 2)), np.zeros(50)])) == 0
    assert len(cdt.delaunay(np.c_[np.linspace(0, 1, 20), np.zeros((20, 2))])) == 0
    assert len(cdt.delaunay(np.zeros((10, 3)))) == 0
    q = rng.random((600, 3))
    p = q + 1e6
    t = cdt.delaunay(p)
    local = p - 1e6  # exact (Sterbenz): geometry measured without cancellation
    tree = cKDTree(local)
    vol = 0.0
    for tet in t:
        s = cdt.orient4(*p[tet])
        assert s != 0
        v = tet if s > 0 else tet[[1, 0, 2, 3]]
        X = local[v]
        vol += abs(np.linalg.det(X[1:] - X[0])) / 6
        A = 2 * (X[1:] - X[0])
        cen = np.linalg.solve(A, (X[1:] ** 2).sum(1) - (X[0] ** 2).sum())
        r = np.sqrt(((X[0] - cen) ** 2).sum())
        for j in tree.query_ball_point(cen, r * (1 + 1e-6) + 1e-12):
            if j not in v:
                assert cdt.insphere(*p[v], p[j]) <= 0, (v, j)  # exact, on the far points
    hv = ConvexHull(local).volume
    assert abs(vol - hv) <= 1e-9 * hv
