"""dm_delaunay on clipped lattices with cavities: the initial points of 3D
CSG differences (a union of balls and axis-aligned cubes minus smaller
ones) are exact staggered lattices, cospherical everywhere and with empty
cavities inside.
The seed search must find a cell of the perturbed triangulation for every
star, and the result must be a valid Delaunay triangulation: no device
flags, the cells tile the convex hull (volumes sum to its volume, every
face shared by at most two cells) and no point lies inside a sampled
circumsphere (beyond 1e-7 of its radius)."""
import numpy as np
import pytest

from seismicmesh_gb300 import _native as N
from seismicmesh_gb300 import synthetic
from seismicmesh_gb300.generation import mesh_generator as MG

pytestmark = pytest.mark.gpu

OPTS = {"verbose": 0, "max_iter": 50, "seed": 0, "perform_checks": False, "pfix": None,
        "axis": 1, "points": None, "delta_t": 0.30, "geps_mult": 0.1, "subdomains": None,
        "mesh_improvement": True, "r0m_is_h0": False}


@pytest.mark.parametrize("index", [245, 246, 253])
def test_clipped_lattice_with_cavities(cuda, index):
    from scipy.spatial import ConvexHull, cKDTree

    dom, h = synthetic.batch_domains(256, rotate_cubes=False)[index]
    run = MG._Run(dom, h, dict(OPTS))
    eng = run.eng
    nc = eng.triangulate()
    assert int(eng.counters_host()[N.CNT_FLAGS]) == 0
    p = eng.P[:, :3].double().cpu().numpy()
    t = eng.cells[:nc].cpu().numpy().astype(np.int64)
    x = p[t]
    a = x[:, 1:] - x[:, :1]
    vol = np.abs(np.linalg.det(a)) / 6
    hull = ConvexHull(p)
    assert abs(vol.sum() - hull.volume) <= 1e-9 * hull.volume
    faces = np.sort(np.concatenate([t[:, [1, 2, 3]], t[:, [0, 2, 3]], t[:, [0, 1, 3]], t[:, [0, 1, 2]]]), 1)
    _, cnt = np.unique(faces, axis=0, return_counts=True)
    assert cnt.max() == 2
    rng = np.random.default_rng(0)
    sel = rng.choice(len(t), size=min(len(t), 50000), replace=False)
    rhs = 0.5 * (a[sel] ** 2).sum(-1)
    c = np.linalg.solve(a[sel], rhs[..., None])[..., 0]
    r = np.linalg.norm(c, axis=1)
    near = cKDTree(p).query_ball_point(x[sel, 0] + c, r * (1 - 1e-7))
    bad = [i for i, lst in enumerate(near) if set(lst) - set(t[sel[i]])]
    assert not bad, len(bad)
