"""The oracle's restatements against the reference's golden fixtures (CPU)."""
import json
import os

import numpy as np

from conftest import GOLDEN, golden
from oracle import distmesh_np as O
from oracle import sdf_np as S
from oracle import sizing_np as Z


def test_limgrad_restatement_matches_reference_bitwise():
    g = golden("limgrad.npz")
    for key in ("kat", "g2", "g3"):
        out = Z.limgrad(g[key + "_dims"], 12.5, 0.15, 10000, g[key + "_in"])
        np.testing.assert_array_equal(out, g[key + "_out"])


def test_kat_limgrad_is_manhattan_growth():
    out = Z.limgrad((3, 3, 1), 1.0, 0.1, 10000, [1.0] + [5.0] * 8)
    np.testing.assert_allclose(out, [1, 1.1, 1.2, 1.1, 1.2, 1.3, 1.2, 1.3, 1.4])


def _shape(name):
    table = {
        "disk": S.disk(0.1, -0.2, 0.9),
        "disk_rot": S.disk(0.1, -0.2, 0.9, rotate=(0.4, 0, 0), stretch=[2.0, 1.0], translate=[0.3, 0.1]),
        "rect": S.rectangle((-0.5, 1.0, -0.7, 0.4)),
        "rect_rot": S.rectangle((-0.5, 1.0, -0.7, 0.4), rotate=(0.3, 0, 0), translate=[0.1, 0.2]),
        "ball": S.ball(0.1, 0.0, -0.1, 0.8),
        "ball_xf": S.ball(0.1, 0.0, -0.1, 0.8, rotate=(0.2, 0.3, 0.4), stretch=[1.0, 2.0, 1.5], translate=[0.1, 0.2, 0.3]),
        "cube": S.cube((-0.5, 0.5, -0.6, 0.4, -0.2, 0.9)),
        "cube_rot": S.cube((-0.5, 0.5, -0.6, 0.4, -0.2, 0.9), rotate=(0.5, 0.0, 0.25)),
        "torus": S.torus(0.8, 0.3),
        "prism": S.prism(0.6, 0.4),
        "cylinder": S.cylinder(h=1.2, r=0.5),
        "cylinder_rot": S.cylinder(h=1.2, r=0.5, rotate=(0.3, 0.0, 0.6)),
        "union2": S.union([S.disk(0, 0, 0.5), S.rectangle((0.0, 1.0, -0.2, 0.3))]),
        "union2_smooth": S.union([S.disk(0, 0, 0.5), S.rectangle((0.0, 1.0, -0.2, 0.3))], k=0.1),
        "inter2": S.intersection([S.disk(0, 0, 0.8), S.rectangle((0.0, 1.0, -0.5, 0.5))]),
        "inter2_smooth": S.intersection([S.disk(0, 0, 0.8), S.rectangle((0.0, 1.0, -0.5, 0.5))], k=0.2),
        "diff2": S.difference([S.rectangle((-1.0, 1.0, -1.0, 1.0)), S.disk(0, 0, 0.4), S.disk(0.6, 0.6, 0.2)]),
        "diff3_smooth": S.difference([S.ball(0.0, 0.0, 0.5, 0.85), S.cube((-0.5, 0.5, -0.5, 0.5, -0.5, 0.5))], k=0.2),
        "union3": S.union([S.ball(0, 0, 0, 0.5), S.cube((0.0, 1.0, -0.2, 0.2, -0.2, 0.2))]),
    }
    return table[name]


SHAPES = ["disk", "disk_rot", "rect", "rect_rot", "ball", "ball_xf", "cube", "cube_rot", "torus",
          "prism", "cylinder", "cylinder_rot", "union2", "union2_smooth", "inter2", "inter2_smooth",
          "diff2", "diff3_smooth", "union3"]


def test_sdf_restatement_matches_reference():
    g = golden("sdf.npz")
    for name in SHAPES:
        ref = g[name]
        x = g["x2"] if ref.shape == g["x2"].shape[:1] and name in ("disk", "disk_rot", "rect", "rect_rot", "union2", "union2_smooth", "inter2", "inter2_smooth", "diff2") else g["x3"]
        np.testing.assert_allclose(_shape(name)(x), ref, rtol=1e-12, atol=1e-12, err_msg=name)


def test_fast_geometry_restatements():
    g = golden("fast_geometry.npz")
    e = g["edges"]
    u = np.unique(np.sort(e, axis=1), axis=0)
    np.testing.assert_array_equal(u, g["unique"])
    p, t = g["points"], g["cells"]
    np.testing.assert_allclose(O.dihedral_angles(p, t), g["dihedral"], rtol=1e-12, atol=1e-12)
    cg = O.circumsphere_grad(p[t[:, 0]], p[t[:, 1]], p[t[:, 2]], p[t[:, 3]])
    np.testing.assert_allclose(cg, g["cgrad"], rtol=1e-7, atol=1e-9 * np.abs(g["cgrad"]).max())


def test_one_iteration_restatement_matches_reference():
    for name, fd, h in (("iter_disk.npz", S.disk(0, 0, 1.0), 0.1), ("iter_ball.npz", S.ball(0, 0, 0, 1.0), 0.2),
                        ("iter_rect.npz", S.rectangle((0.0, 1.0, 0.0, 2.0)), 0.1),
                        ("iter_cube.npz", S.cube((0.0, 1.0, 0.0, 1.0, 0.0, 1.0)), 0.2)):
        g = golden(name)
        p1, t, F = O.one_iteration(g["p0"].copy(), fd, lambda x, h=h: np.full(len(x), h), h)
        np.testing.assert_array_equal(O.unique_edges(np.sort(t, 1)), O.unique_edges(np.sort(g["t"], 1)))
        np.testing.assert_allclose(F, g["F"], rtol=1e-10, atol=1e-12)
        # the projection's finite-difference gradient amplifies last-bit
        # differences of the distance formula by 1/deps (~1e8 / h)
        np.testing.assert_allclose(p1, g["p1"], rtol=1e-6, atol=1e-9)


def test_disk_generate_mesh_restatement_matches_reference():
    g = golden("disk_h01.npz")
    fd = S.disk(0.0, 0.0, 1.0)
    p, t = O.generate_mesh(fd, lambda x: np.full(len(x), 0.1), 0.1, (-1.0, 1.0, -1.0, 1.0))
    assert len(p) == len(g["p"]) and len(t) == len(g["t"])
    np.testing.assert_allclose(np.sort(O.simp_qual(p, t)), np.sort(g["qual"]), atol=1e-9)
    assert abs(O.simp_vol(p, t).sum() - float(g["area"])) < 1e-9


def test_sizing_restatement_matches_reference():
    g = golden("sizing.npz")
    for style in ("edge", "constant", "linear_ramp"):
        cell, bbox = Z.size_grid(g["vp2"], tuple(g["bbox2"]), hmin=75.0, wl=10, freq=2.0, grade=0.15,
                                 domain_pad=500.0, pad_style=style)
        np.testing.assert_allclose(bbox, g["bbox2_" + style])
        np.testing.assert_allclose(Z.interpolant(cell, bbox)(g["xq2"]), g["eval2_" + style], rtol=1e-12)
    cell, bbox = Z.size_grid(g["vp2"], tuple(g["bbox2"]), hmin=75.0, wl=10, freq=2.0, grade=0.15, dt=0.001, cr_max=0.5)
    np.testing.assert_allclose(Z.interpolant(cell, bbox)(g["xq2"]), g["eval2_courant"], rtol=1e-12)
    cell, bbox = Z.size_grid(g["vp3"], tuple(g["bbox3"]), hmin=50.0, wl=10, freq=2.0, grade=0.15)
    np.testing.assert_allclose(Z.interpolant(cell, bbox)(g["xq3"]), g["eval3"], rtol=1e-12)


def test_reference_test_goldens_recorded():
    with open(os.path.join(GOLDEN, "reference_tests.json")) as f:
        d = json.load(f)
    r = d["test_2dmesher_SDF"]
    assert np.allclose(r["ref_harness"], r["golden"], atol=r["atol"])
    assert min(d["test_2d_min_qual"]["ref_harness_min_quals"]) > 0.60


def test_mesh_qa_restatement_matches_reference():
    """re ratios, 1-ring overlaps (as multisets: the reference lists the cells
    around a vertex in quicksort order) against the reference's outputs"""
    from oracle import mesh_qa_np as Q

    g = golden("mesh_qa.npz")
    np.testing.assert_allclose(Q.calc_re_ratios(g["p2"], g["t2"], 2), g["re2"], rtol=1e-12)
    np.testing.assert_allclose(Q.calc_re_ratios(g["p3"], g["t3"][:400], 3), g["re3"][:400], rtol=1e-10)
    for key, dim in (("2", 2), ("3", 3)):
        ov = Q.do_any_overlap(g["f" + key], g["t" + key], dim)
        assert sorted(ov) == sorted(map(tuple, g["ov" + key].tolist()))
    assert Q.do_any_overlap(g["p2"], g["t2"], 2) == []


def test_kat_re_ratios_equilateral_pair():
    """reference tests/test_geometry2.py:11-15: two equilateral-ish triangles"""
    from oracle import mesh_qa_np as Q

    points = np.array([[0, 0], [6, 0], [3, 3], [9, 3]], dtype=float)
    cells = np.array([[3, 2, 1], [2, 0, 1]])
    np.testing.assert_allclose(Q.calc_re_ratios(points, cells, 2), [0.70710678, 0.70710678], rtol=1e-8)
    assert Q.do_any_overlap(points, cells, 2) == []


def test_kat_cell_quality_regular_and_right_triangle():
    from oracle import mesh_qa_np as Q

    tri = np.array([[0.0, 0.0], [1.0, 0.0], [0.5, np.sqrt(3) / 2]])
    q, _ = Q.cell_quality(tri, np.array([[0, 1, 2]]))
    np.testing.assert_allclose(q, [1.0], rtol=1e-14)
    q, _ = Q.cell_quality(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]), np.array([[0, 1, 2]]))
    np.testing.assert_allclose(q, [2 * (2 - np.sqrt(2)) / 2 / (np.sqrt(2) / 2)], rtol=1e-14)
    tet = np.array([[1.0, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])
    q, s = Q.cell_quality(tet, np.array([[0, 1, 2, 3]]))
    np.testing.assert_allclose(q, [1.0], rtol=1e-14)
    np.testing.assert_allclose(s, [1.0], rtol=1e-14)


def test_cell_quality_2d_is_the_reference_simp_qual():
    """in 2D the benchmark quality 2 r / R is the reference's simp_qual
    (geometry/utils.py:252-274): pinned to its outputs on the disk mesh"""
    from oracle import mesh_qa_np as Q

    g = golden("disk_h01.npz")
    q, _ = Q.cell_quality(g["p"], g["t"])
    np.testing.assert_allclose(q, g["qual"], rtol=1e-10)


def test_min_sin_dihedral_against_reference_dihedral_angles():
    """the 3D measure min sin(dihedral) / (2 sqrt(2) / 3) from the reference's
    own calc_dihedral_angles (fast_geometry.cpp:351-418) outputs"""
    from oracle import mesh_qa_np as Q

    g = golden("fast_geometry.npz")
    p, t = g["points"], g["cells"]
    vol = np.abs(np.einsum("ij,ij->i", p[t[:, 1]] - p[t[:, 0]],
                           np.cross(p[t[:, 2]] - p[t[:, 0]], p[t[:, 3]] - p[t[:, 0]])))
    ok = vol > 1e-12  # flat cells have no meaningful angles
    _, s = Q.cell_quality(p, t[ok])
    ref = np.sin(g["dihedral"].reshape(-1, 6)[ok]).min(1) / (2 * np.sqrt(2) / 3)
    np.testing.assert_allclose(s, ref, rtol=1e-8, atol=1e-12)


def test_kat_point_in_tetrahedron_from_the_reference_test():
    """tests/test_ptin.py of the reference: on its perfect tetrahedron the
    query (0.5, 0.5, 1.0) is inside and (0, 0, 1) outside; the oracle's
    restatement of vertex_in_entity3 (used by the overlap oracle) agrees, and
    so does the 2D one on a triangle"""
    from oracle import mesh_qa_np as QA

    tet = np.array([[0, 0, 0], [0, 1, 0], [np.sqrt(2), 0.5, 0], [0.5, 0.5, np.sqrt(2)]], dtype=float)
    assert QA.inside3((0.5, 0.5, 1.0), tet)
    assert not QA.inside3((0.0, 0.0, 1.0), tet)
    tri = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    assert QA.inside2((0.25, 0.25), tri)
    assert not QA.inside2((1.0, 1.0), tri)
