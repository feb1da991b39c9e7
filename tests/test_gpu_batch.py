"""generate_meshes (many problems stepped together, graph-captured
iterations on tuned streams) against generate_mesh on each problem alone:
the same points (to 1e-6 of the domain's extent: the only arithmetic that
may differ is the order of the 2D Laplacian smoother's reductions) and the
same cells as sets, for problems of the batched workload's kind (CSG
unions/differences of disks and rectangles, balls and cubes)."""
import numpy as np
import pytest

import seismicmesh_gb300 as sm
from seismicmesh_gb300 import synthetic
from seismicmesh_gb300.generation.batch import generate_meshes

pytestmark = pytest.mark.gpu


def _cells(t):
    return np.unique(np.sort(np.asarray(t), axis=1), axis=0)


def test_batched_meshes_equal_sequential(cuda):
    problems = synthetic.batch_domains(n=8, seed=100, lo=1e3, hi=8e3)
    stats = {}
    got = generate_meshes(problems, candidates=(2, 4), checked=3, stats=stats, max_iter=20)
    print(stats["points"], stats["tuning"], stats["redone"])
    assert stats["captured_problems"] == len(problems)
    for (dom, h), (p, t) in zip(problems, got):
        p0, t0 = sm.generate_mesh(dom, h, max_iter=20, verbose=0)
        ext = np.ptp(np.asarray(dom.bbox).reshape(-1, 2), axis=1).max()
        assert p.shape == p0.shape
        assert np.abs(p - p0).max() <= 1e-6 * ext
        assert np.array_equal(_cells(t), _cells(t0))
