"""Mesh quality / linting kernels and the periodic Repeat domain on the GPU
against the reference's outputs (tests/golden/mesh_qa.npz, repeat.npz) and
the oracle restatement."""
import numpy as np
import pytest

import seismicmesh_gb300 as sm
from conftest import golden
from oracle import mesh_qa_np as Q

pytestmark = pytest.mark.gpu


def test_re_ratios_match_reference(cuda):
    g = golden("mesh_qa.npz")
    np.testing.assert_allclose(sm.geometry.calc_re_ratios(g["p2"], g["t2"], dim=2), g["re2"], rtol=1e-12)
    np.testing.assert_allclose(sm.geometry.calc_re_ratios(g["p3"], g["t3"], dim=3), g["re3"], rtol=1e-9)


def test_re_ratios_known_answer(cuda):
    """reference tests/test_geometry2.py:11-15"""
    points = np.array([[0, 0], [6, 0], [3, 3], [9, 3]], dtype=float)
    cells = np.array([[3, 2, 1], [2, 0, 1]], dtype=int)
    ce = sm.geometry.calc_re_ratios(points, cells, dim=2)
    assert np.allclose(ce, [0.70710678, 0.70710678])
    assert len(sm.geometry.do_any_overlap(points, cells, dim=2)) == 0
    assert len(sm.geometry.get_edges(cells)) == 6
    wedges = sm.geometry.get_winded_boundary_edges(cells)
    assert np.allclose(wedges, [[0, 1], [1, 3], [2, 3], [0, 2]])


@pytest.mark.parametrize("dim", [2, 3])
def test_overlap_pairs_match_reference(cuda, dim):
    """same pairs with the same multiplicity (bit-exact FP64 decisions); the
    reference lists the cells around a vertex in quicksort order, so the
    comparison is on the sorted lists"""
    g = golden("mesh_qa.npz")
    k = str(dim)
    ov = sm.geometry.do_any_overlap(g["f" + k], g["t" + k], dim=dim)
    assert len(ov) > 0
    assert sorted(ov) == sorted(map(tuple, g["ov" + k].tolist()))
    # the documented order: by cell, vertex slot, neighbour
    assert ov == Q.do_any_overlap(g["f" + k], g["t" + k], dim)
    assert sm.geometry.do_any_overlap(g["p" + k], g["t" + k], dim=dim) == []


def test_overlap_capacity_retry(cuda):
    """more pairs than the first buffer holds: a dense fold of a fine mesh"""
    p, t = sm.generate_mesh(domain=sm.Rectangle((0.0, 1.0, 0.0, 1.0)), edge_length=0.01, verbose=0)
    rng = np.random.default_rng(3)
    q = p + 0.03 * rng.normal(size=p.shape)
    ov = sm.geometry.do_any_overlap(q, t, dim=2)
    assert len(ov) > max(1024, len(t) // 8)
    sub = np.unique(np.array(ov)[:, 0])[:40]
    ref = [pr for pr in Q.do_any_overlap(q, t, 2) if pr[0] in set(sub.tolist())] if len(t) < 30000 else None
    if ref is not None:
        assert [pr for pr in ov if pr[0] in set(sub.tolist())] == ref


def test_linter_matches_reference(cuda):
    g = golden("mesh_qa.npz")
    p, t = sm.geometry.linter(g["f2"], g["t2"], dim=2)
    np.testing.assert_allclose(p, g["lint2_p"], rtol=0, atol=1e-12)
    assert np.array_equal(np.sort(t, axis=1)[np.lexsort(np.sort(t, axis=1).T[::-1])],
                          np.sort(g["lint2_t"], axis=1)[np.lexsort(np.sort(g["lint2_t"], axis=1).T[::-1])])


@pytest.mark.parametrize("name", ["ball", "ball_aniso", "union"])
def test_repeat_matches_reference(cuda, name):
    g = golden("repeat.npz")
    bbox = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    dom = {
        "ball": lambda: sm.Repeat(bbox, sm.Ball([0.0, 0.0, 0.0], 0.12), [0.4, 0.4, 0.4]),
        "ball_aniso": lambda: sm.Repeat(bbox, sm.Ball([0.0, 0.0, 0.0], 0.1), [0.3, 0.5, 0.45]),
        "union": lambda: sm.Repeat(
            bbox, sm.Union([sm.Ball([0.0, 0.0, 0.0], 0.1), sm.Cube((-0.05, 0.05, -0.2, 0.2, -0.05, 0.05))]),
            [0.5, 0.5, 0.5]),
    }[name]()
    d = dom.eval(g["x"])
    np.testing.assert_allclose(d, g[name], rtol=0, atol=1e-5 * (1 + np.abs(g[name]).max()))


def test_repeat_mesh(cuda):
    """README's periodic example on a smaller box: a periodic array of balls;
    every cell centroid inside the domain, volume of the 27 balls within 10%"""
    bbox = (0.0, 1.5, 0.0, 1.5, 0.0, 1.5)
    dom = sm.Repeat(bbox, sm.Ball([0.0, 0.0, 0.0], 0.2), [0.5, 0.5, 0.5])
    p, t = sm.generate_mesh(domain=dom, edge_length=0.05, verbose=0)
    assert len(t) > 1000
    c = p[t].mean(1)
    assert (dom.eval(c) < 0.01).all()
    vol = np.abs(sm.geometry.simp_vol(p, t)).sum()
    # balls centred on multiples of 0.5 inside [0, 1.5]^3: 4 per axis, halves
    # and quarters at the faces -> (0.5 + 1 + 1 + 0.5)^3 = 27 full balls
    expect = 27 * 4 / 3 * np.pi * 0.2**3
    assert abs(vol - expect) / expect < 0.1


@pytest.mark.parametrize("dim", [2, 3])
def test_cell_quality_matches_oracle(cuda, dim):
    g = golden("mesh_qa.npz")
    p, t = g["p" + str(dim)], g["t" + str(dim)]
    q, s = sm.geometry.cell_quality(p, t)
    rq, rs = Q.cell_quality(p, t)
    np.testing.assert_allclose(q, rq, rtol=1e-10)
    if dim == 3:
        np.testing.assert_allclose(s, rs, rtol=1e-10)
    # the known answers: regular simplices score 1
    tet = np.array([[1.0, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])
    q, s = sm.geometry.cell_quality(tet, np.array([[0, 1, 2, 3]]))
    np.testing.assert_allclose([q[0], s[0]], [1.0, 1.0], rtol=1e-14)
    st = sm.geometry.quality_stats(p, t)
    assert st["min_quality"] == pytest.approx(rq.min(), rel=1e-10)
    assert st["quality_hist"][0].sum() == len(t)
    if dim == 3:
        assert 0 < st["min_dihedral"] <= st["avg_dihedral"] <= st["max_dihedral"] <= 90.0
