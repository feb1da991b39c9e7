"""Drop-in geometry functions on inputs the fixtures do not cover: unrounded
FP64 points (the reference computes in FP64, so do these entry points) and
unique_edges with hub vertices whose buckets take the block merge sort.

Tolerances: FP64 results within 1e-12 relative (dihedral angles: or 1e-9 rad
absolute) or 1e-10 relative (volumes, qualities) of the oracle's FP64 numpy
restatement (pinned to the reference's outputs in test_oracle.py); integer
pairs exact."""
import numpy as np
import pytest

import seismicmesh_gb300 as sm
from oracle import distmesh_np as O

pytestmark = pytest.mark.gpu


def _generic_tets(seed=5, n=3000):
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    p = rng.normal(size=(n, 3)) * np.array([1.0, 0.7, 1.3]) + 1e3 * np.pi
    t = Delaunay(p).simplices.astype(np.int32)
    return p, t


def test_dihedral_angles_are_fp64_on_unrounded_points(cuda):
    p, t = _generic_tets()
    assert not np.array_equal(p, p.astype(np.float32).astype(np.float64))
    got = sm.geometry.calc_dihedral_angles(p, t)
    ref = O.dihedral_angles(p, t)
    # acos is ill-conditioned near 0 and pi (flat hull tetrahedra of the
    # random set): 1e-12 relative, and 1e-9 rad absolute there
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-9)


def test_simp_vol_and_qual_are_fp64_on_unrounded_points(cuda):
    p, t = _generic_tets(seed=6)
    np.testing.assert_allclose(sm.geometry.simp_vol(p, t), O.simp_vol(p, t), rtol=1e-10)
    # 2D: the reference's simp_qual on generic float64 points
    rng = np.random.default_rng(7)
    from scipy.spatial import Delaunay

    q = rng.normal(size=(2000, 2)) + 123.456789
    tq = Delaunay(q).simplices.astype(np.int32)
    np.testing.assert_allclose(sm.geometry.simp_qual(q, tq), O.simp_qual(q, tq), rtol=1e-10)
    np.testing.assert_allclose(sm.geometry.simp_vol(q, tq), O.simp_vol(q, tq), rtol=1e-10)


@pytest.mark.parametrize("hub_degree", [33, 700, 5000, 40000])
def test_unique_edges_with_hub_vertices(cuda, hub_degree):
    """buckets above 32 entries go through the block merge sort; with
    duplicates and both orientations of every pair"""
    rng = np.random.default_rng(hub_degree)
    n = 60000
    hub = rng.integers(1, n, size=hub_degree)
    e_hub = np.stack([np.zeros_like(hub), hub], 1)
    e_rand = rng.integers(0, n, size=(50000, 2))
    e_hub2 = np.stack([rng.integers(0, 100, size=hub_degree), np.full(hub_degree, 7)], 1)
    e = np.concatenate([e_hub, e_hub[:, ::-1], e_rand, e_hub2]).astype(np.int32)
    e = e[rng.permutation(len(e))]
    got = sm.geometry.unique_edges(e)
    ref = np.unique(np.sort(e, axis=1), axis=0)
    np.testing.assert_array_equal(got, ref)


def test_unique_edges_above_four_million_vertices(cuda):
    """n = 5e6 vertex buckets: the bucket scan takes its two-level path"""
    rng = np.random.default_rng(9)
    n = 5_000_000
    e = rng.integers(0, n, size=(1_000_000, 2)).astype(np.int32)
    e[0] = (n - 1, 0)
    got = sm.geometry.unique_edges(e)
    ref = np.unique(np.sort(e, axis=1), axis=0)
    np.testing.assert_array_equal(got, ref)
