"""Parity at the headline workload: the 3D unit ball at h = 0.02 (526,727
initial vertices, max_iter 50, seed 0, then sliver_removal with a 10 degree
bound).

* End metrics against the reference's own runs (tests/golden/ball_h002*.json,
  made by tests/golden/make_golden_ball_h002.py through the reference package
  with Qhull, or the oracle's exact-predicate C++ Delaunay, standing in for
  CGAL): vertex count, cell count, mean quality and mean minimum dihedral
  angle within 1 % (2 % against the Qhull run from the degenerate lattice),
  minimum dihedral angle >= 10 degrees.
* Connectivity at full size: the production point set after 5 iterations
  (float32 positions on the run's position grid, so every predicate takes
  the fixed-point path) triangulated by dm_delaunay and by Qhull, compared
  cell for cell after canonical ordering.
"""
import json
import os

import numpy as np
import pytest

import seismicmesh_gb300 as sm
from conftest import GOLDEN
from oracle import delaunay_check as dc
from oracle import mesh_qa_np as QA

pytestmark = pytest.mark.gpu

H = 0.02
REL = 0.01


def _metrics(p, t):
    dh = np.degrees(sm.geometry.calc_dihedral_angles(p, t)).reshape(-1, 6).min(1)
    q, s = QA.cell_quality_vec(p, t)
    return {
        "n_points": len(p), "n_cells": len(t),
        "min_dihedral_deg": float(dh.min()), "mean_min_dihedral_deg": float(dh.mean()),
        "min_quality": float(q.min()), "mean_quality": float(q.mean()),
        "volume": float(np.abs(sm.geometry.simp_vol(p, t)).sum()),
    }


def _compare(g, got, keys, rel):
    for stage in ("generate_mesh", "sliver_removal"):
        for k in keys:
            a, b = got[stage][k], g[stage][k]
            print(f"{stage} {k}: gpu {a} reference {b} rel {(a - b) / b:+.3e}")
            assert abs(a - b) <= rel * abs(b), (stage, k, a, b)


def _run(**kw):
    ball = sm.Ball([0.0, 0.0, 0.0], 1.0)
    p, t = sm.generate_mesh(ball, H, verbose=0, **kw)
    ps, ts = sm.sliver_removal(p, ball, H, min_dh_angle_bound=10, verbose=0)
    return {"generate_mesh": _metrics(p, t), "sliver_removal": _metrics(ps, ts)}


def test_ball_h002_end_metrics_match_reference_from_a_generic_start(cuda):
    """From the reference's initial points moved by a seeded jitter of 1e-3 h
    (a generic start: every triangulation of the run is unique, so the
    reference's Qhull stand-in and dm_delaunay agree on each), vertex count,
    cell count, mean quality, mean minimum dihedral angle and volume are
    within 1 % of the reference's."""
    from oracle import distmesh_np as O

    with open(os.path.join(GOLDEN, "ball_h002_jitter.json")) as f:
        g = json.load(f)
    got = _run(points=O.jittered_ball_points(H))
    _compare(g, got, ("n_points", "n_cells", "mean_quality", "mean_min_dihedral_deg", "volume"), REL)
    assert got["sliver_removal"]["min_dihedral_deg"] >= 10.0 - 1e-6


def test_ball_h002_end_metrics_from_the_lattice(cuda):
    """The plain call, from the exact initial lattice: there the Delaunay
    triangulation is not unique (cospherical lattice points) and the first
    iterations depend on how ties are broken.  dm_delaunay breaks them by
    symbolic perturbation in lexicographic point order (the scheme published
    for CGAL, the reference's triangulator).  Two reference runs bracket it:

    * with Qhull standing in for CGAL (ball_h002.json), which breaks ties its
      own way: vertex count identical, cell count and volume within 1 %, mean
      quality and mean minimum dihedral angle within 2 % (measured: -1.2 %
      quality after sliver removal);
    * with the oracle's exact-predicate C++ Delaunay standing in for CGAL
      (ball_h002_cpp.json), ties broken by another symbolic perturbation:
      every metric within 1 % (measured: +0.9 % mean quality after
      generate_mesh, +0.6 % after sliver removal).  That run's mean minimum
      dihedral after generate_mesh is NaN (the reference's FP64 dihedral
      routine on an extremely flat sliver, quality 2e-8) and is not compared.

    The GPU's metrics lie between the two reference runs, and the
    generic-start test above shows that the differences come from the
    tie-breaking alone."""
    with open(os.path.join(GOLDEN, "ball_h002.json")) as f:
        g = json.load(f)
    with open(os.path.join(GOLDEN, "ball_h002_cpp.json")) as f:
        gx = json.load(f)
    got = _run()
    _compare(g, got, ("n_points", "n_cells", "volume"), REL)
    _compare(g, got, ("mean_quality", "mean_min_dihedral_deg"), 0.02)
    for stage, keys in (("generate_mesh", ("n_points", "n_cells", "volume", "mean_quality")),
                        ("sliver_removal", ("n_points", "n_cells", "volume", "mean_quality",
                                            "mean_min_dihedral_deg"))):
        for k in keys:
            a, b = got[stage][k], gx[stage][k]
            print(f"{stage} {k}: gpu {a} reference (exact stub) {b} rel {(a - b) / b:+.3e}")
            assert abs(a - b) <= REL * abs(b), (stage, k, a, b)
    assert got["sliver_removal"]["min_dihedral_deg"] >= 10.0 - 1e-6


def _production_points(k=5):
    """the engine's point set after k DistMesh iterations of the h = 0.02 ball
    (float32 positions on the run's position grid) and the grid exponent"""
    from seismicmesh_gb300 import _native as N
    from seismicmesh_gb300.generation import mesh_generator as MG

    ball = sm.Ball([0.0, 0.0, 0.0], 1.0)
    fd = MG._Domain(ball)
    sizing = MG._Sizing(H, 3)
    opts = {"points": None, "r0m_is_h0": False, "seed": 0}
    p0 = MG._initialize_points(3, 0.1 * H, np.array([[-1.0, 1.0]] * 3), sizing, fd, H, opts,
                               np.empty((0, 3)))
    assert len(p0) == 526727
    eng = MG._Engine(3, p0, 0)
    deps = float(np.sqrt(np.finfo(float).eps) * H)
    for _ in range(k):
        eng.triangulate()
        eng.filter(fd, 0.1 * H)
        eng.build_adjacency()
        eng.step(sizing, [fd], 1 + 0.4 / 2**2, 0.30, H, deps)
    assert int(eng.counters_host()[N.CNT_FLAGS]) == 0
    return eng.P[:, :3].double().cpu().numpy(), eng.grid_exp


def _triangulate(p, grid_exp):
    from seismicmesh_gb300.generation import mesh_generator as MG

    eng = MG._Engine(3, p, 0)
    assert eng.grid_exp == grid_exp
    nc = eng.triangulate()
    return eng.cells[:nc].cpu().numpy()


def test_ball_h002_delaunay_matches_qhull_at_full_size(cuda):
    """After 5 iterations the deep interior of the ball is still the exact
    initial lattice (its forces cancel by symmetry), where the Delaunay
    triangulation is not unique.  The production points are therefore moved
    by a seeded jitter of up to 64 grid units (staying on the position grid,
    so the fixed-point predicates still decide everything): the set is then
    in general position and its triangulation unique, and dm_delaunay must
    equal Qhull cell for cell at the full 526,727 points."""
    p, e = _production_points()
    rng = np.random.default_rng(11)
    q = p + rng.integers(-64, 65, size=p.shape) * 2.0**e
    scaled = q * 2.0 ** (-e)
    assert np.array_equal(scaled, np.rint(scaled))
    a = dc.canonical(_triangulate(q, e))
    b = dc.canonical(dc.qhull_cells(q))
    print(f"dm_delaunay {len(a)} cells, Qhull {len(b)} cells on {len(q)} points")
    assert a.shape == b.shape
    assert np.array_equal(a, b)


def test_ball_h002_delaunay_is_valid_on_the_production_points(cuda):
    """The unjittered production points (exact lattice inside): the cells tile
    the convex hull (volumes sum to the hull volume, every interior face is
    shared by two cells) and no point lies inside a cell's circumsphere."""
    from scipy.spatial import ConvexHull, cKDTree

    p, e = _production_points()
    t = _triangulate(p, e).astype(np.int64)
    x = p[t]
    a = x[:, 1:] - x[:, :1]
    vol = np.linalg.det(a) / 6
    assert (vol > 0).all() or (vol < 0).all()
    hull = ConvexHull(p)
    assert abs(np.abs(vol).sum() - hull.volume) <= 1e-9 * hull.volume
    faces = np.sort(np.concatenate([t[:, [1, 2, 3]], t[:, [0, 2, 3]], t[:, [0, 1, 3]], t[:, [0, 1, 2]]]), 1)
    _, cnt = np.unique(faces, axis=0, return_counts=True)
    assert cnt.max() == 2
    # empty circumspheres on a sample of cells: no point deeper inside than
    # the float64 evaluation error (1e-7 of the radius)
    rng = np.random.default_rng(3)
    sel = rng.choice(len(t), size=min(len(t), 300000), replace=False)
    xs, as_ = x[sel], a[sel]
    rhs = 0.5 * (as_ * as_).sum(-1)
    c = np.linalg.solve(as_, rhs[..., None])[..., 0]
    r = np.linalg.norm(c, axis=1)
    centre = xs[:, 0] + c
    tree = cKDTree(p)
    near = tree.query_ball_point(centre, r * (1 - 1e-7))
    bad = [i for i, lst in enumerate(near) if set(lst) - set(t[sel[i]])]
    print(f"{len(t)} cells; {len(sel)} circumspheres checked; {len(bad)} with an interior point")
    assert not bad
