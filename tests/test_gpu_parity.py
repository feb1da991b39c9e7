"""GPU kernels against the reference's golden fixtures (through the C ABI).

Tolerances: integer / index results bit-exact; FP32 device results within
1e-5 relative of the reference's FP64 values (positions, forces, distances,
sizes) unless stated."""
import json
import os

import numpy as np
import pytest
import torch

import seismicmesh_gb300 as sm
from conftest import GOLDEN, golden
from oracle import delaunay_check as dc
from oracle import distmesh_np as O
from seismicmesh_gb300 import _native as N
from seismicmesh_gb300.generation import mesh_generator as MG

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _one_iteration(p0, domain, h, grid=False):
    dim = p0.shape[1]
    eng = MG._Engine(dim, p0, 0, grid=grid)
    eng.triangulate()
    fd = MG._Domain(domain)
    eng.filter(fd, 0.1 * h)
    nk = int(eng.counters[N.CNT_KEPT].item())
    t = eng.kept[:nk].cpu().numpy()
    eng.build_adjacency()
    sizing = MG._Sizing(h, dim)
    L0mult = 1 + 0.4 / 2 ** (dim - 1)
    eng.step(sizing, [fd], L0mult, 0.30, h, np.sqrt(np.finfo(float).eps) * h)
    return eng.P[:, :dim].double().cpu().numpy(), t


@pytest.mark.parametrize("name,shape", [
    ("iter_disk.npz", lambda: sm.Disk([0.0, 0.0], 1.0)),
    ("iter_ball.npz", lambda: sm.Ball([0.0, 0.0, 0.0], 1.0)),
    ("iter_rect.npz", lambda: sm.Rectangle((0.0, 1.0, 0.0, 2.0))),
    ("iter_cube.npz", lambda: sm.Cube((0.0, 1.0, 0.0, 1.0, 0.0, 1.0))),
])
@pytest.mark.parametrize("grid", [False, True], ids=["float32", "position-grid"])
def test_one_distmesh_iteration_matches_reference(cuda, name, shape, grid):
    """grid=True is the production path: the points are snapped to the run's
    position grid (a move of at most half a float32 ulp at the largest
    coordinate), the predicates run in fixed point and the update rounds
    back onto the grid; the same 1e-5 bound holds."""
    g = golden(name)
    h = float(g["h"])
    p1, t = _one_iteration(g["p0"], shape(), h, grid=grid)
    # connectivity of the kept cells: identical (generic points)
    np.testing.assert_array_equal(dc.canonical(t), dc.canonical(g["t"]))
    scale = np.abs(g["p1"]).max()
    assert np.abs(p1 - g["p1"]).max() <= RTOL * scale
    # displacement (forces) of points the projection did not touch
    moved = g["p1"] - g["p0"]
    free = np.abs(moved - 0.30 * g["F"]).max(1) < 1e-12
    dgpu = p1[free] - g["p0"][free]
    assert np.abs(dgpu - moved[free]).max() <= 1e-4 * np.abs(moved).max() + 1e-7 * scale


SDF_SHAPES = {
    "disk": lambda: sm.Disk([0.1, -0.2], 0.9),
    "disk_rot": lambda: sm.Disk([0.1, -0.2], 0.9, rotate=[0.4, 0, 0], stretch=[2.0, 1.0], translate=[0.3, 0.1]),
    "rect": lambda: sm.Rectangle((-0.5, 1.0, -0.7, 0.4)),
    "rect_rot": lambda: sm.Rectangle((-0.5, 1.0, -0.7, 0.4), rotate=[0.3, 0, 0], translate=[0.1, 0.2]),
    "ball": lambda: sm.Ball([0.1, 0.0, -0.1], 0.8),
    "ball_xf": lambda: sm.Ball([0.1, 0.0, -0.1], 0.8, rotate=[0.2, 0.3, 0.4], stretch=[1.0, 2.0, 1.5], translate=[0.1, 0.2, 0.3]),
    "cube": lambda: sm.Cube((-0.5, 0.5, -0.6, 0.4, -0.2, 0.9)),
    "cube_rot": lambda: sm.Cube((-0.5, 0.5, -0.6, 0.4, -0.2, 0.9), rotate=[0.5, 0.0, 0.25]),
    "torus": lambda: sm.Torus(0.8, 0.3),
    "prism": lambda: sm.Prism(0.6, 0.4),
    "cylinder": lambda: sm.Cylinder(h=1.2, r=0.5),
    "cylinder_rot": lambda: sm.Cylinder(h=1.2, r=0.5, rotate=[0.3, 0.0, 0.6]),
    "union2": lambda: sm.Union([sm.Disk([0.0, 0.0], 0.5), sm.Rectangle((0.0, 1.0, -0.2, 0.3))]),
    "union2_smooth": lambda: sm.Union([sm.Disk([0.0, 0.0], 0.5), sm.Rectangle((0.0, 1.0, -0.2, 0.3))], smoothness=0.1),
    "inter2": lambda: sm.Intersection([sm.Disk([0.0, 0.0], 0.8), sm.Rectangle((0.0, 1.0, -0.5, 0.5))]),
    "inter2_smooth": lambda: sm.Intersection([sm.Disk([0.0, 0.0], 0.8), sm.Rectangle((0.0, 1.0, -0.5, 0.5))], smoothness=0.2),
    "diff2": lambda: sm.Difference([sm.Rectangle((-1.0, 1.0, -1.0, 1.0)), sm.Disk([0.0, 0.0], 0.4), sm.Disk([0.6, 0.6], 0.2)]),
    "diff3_smooth": lambda: sm.Difference([sm.Ball((0.0, 0.0, 0.5), 0.85), sm.Cube((-0.5, 0.5, -0.5, 0.5, -0.5, 0.5))], smoothness=0.2),
    "union3": lambda: sm.Union([sm.Ball((0.0, 0.0, 0.0), 0.5), sm.Cube((0.0, 1.0, -0.2, 0.2, -0.2, 0.2))]),
}


@pytest.mark.parametrize("name", sorted(SDF_SHAPES))
def test_sdf_programs_match_reference(cuda, name):
    g = golden("sdf.npz")
    s = SDF_SHAPES[name]()
    x = g["x2"] if s.dim == 2 else g["x3"]
    d = s.eval(x)
    np.testing.assert_allclose(d, g[name], rtol=0, atol=RTOL * (1 + np.abs(g[name]).max()))
    np.testing.assert_allclose(s.bbox, g[name + "_bbox"], rtol=1e-12)
    if name + "_corners" in g:
        np.testing.assert_allclose(s.corners, g[name + "_corners"], rtol=1e-12)


def test_sdf_gradients_match_finite_differences(cuda):
    g = golden("sdf.npz")
    for name in ("ball_xf", "cube_rot", "torus", "cylinder_rot", "diff3_smooth", "disk_rot", "union2_smooth"):
        s = SDF_SHAPES[name]()
        x = (g["x2"] if s.dim == 2 else g["x3"])[:500]
        d, grad = s.eval(x, grad=True)
        ref = SDF_SHAPES[name]()
        eps = 1e-3
        fd = np.stack([(ref.eval(x + eps * np.eye(s.dim)[k]) - ref.eval(x - eps * np.eye(s.dim)[k])) / (2 * eps)
                       for k in range(s.dim)], 1)
        # away from kinks the analytic gradient equals the central difference
        ok = np.abs(fd - grad).max(1) < 1e-2
        assert ok.mean() > 0.97, name


def test_fast_geometry_kernels_match_reference(cuda):
    g = golden("fast_geometry.npz")
    np.testing.assert_array_equal(sm.geometry.unique_edges(g["edges"]), g["unique"])
    p, t = g["points"], g["cells"]
    np.testing.assert_allclose(sm.geometry.calc_dihedral_angles(p, t), g["dihedral"], rtol=1e-12, atol=1e-12)
    cg = sm.geometry.calc_circumsphere_grad(p[t[:, 0]], p[t[:, 1]], p[t[:, 2]], p[t[:, 3]])
    np.testing.assert_allclose(cg, g["cgrad"], rtol=1e-9, atol=1e-12 * np.abs(g["cgrad"]).max())


def test_limgrad_reaches_the_reference_fixed_point(cuda):
    from seismicmesh_gb300 import _device as D

    g = golden("limgrad.npz")
    for key in ("kat", "g2", "g3"):
        dims = g[key + "_dims"]
        f = torch.from_numpy(g[key + "_in"].copy()).cuda()
        N.call("dm_limgrad", (N.c_int * 3)(*map(int, dims)), 12.5, 0.15, 10000, D.ptr(f), D.stream_ptr())
        ref = g[key + "_out"]
        ftol = g[key + "_in"].min() * np.sqrt(np.finfo(float).eps)
        assert np.abs(f.cpu().numpy() - ref).max() <= 50 * ftol + 1e-12


@pytest.mark.parametrize("case", ["edge", "constant", "linear_ramp", "courant", "3d"])
def test_sizing_function_matches_reference(cuda, case):
    g = golden("sizing.npz")
    if case == "3d":
        ef = sm.get_sizing_function_from_segy(None, tuple(g["bbox3"]), velocity_data=g["vp3"].copy(),
                                              nz=21, nx=17, ny=15, hmin=50.0, wl=10, freq=2.0, grade=0.15)
        ref, x = g["eval3"], g["xq3"]
    elif case == "courant":
        ef = sm.get_sizing_function_from_segy(None, tuple(g["bbox2"]), velocity_data=g["vp2"].copy(),
                                              nz=60, nx=90, hmin=75.0, wl=10, freq=2.0, grade=0.15, dt=0.001, cr_max=0.5)
        ref, x = g["eval2_courant"], g["xq2"]
    else:
        ef = sm.get_sizing_function_from_segy(None, tuple(g["bbox2"]), velocity_data=g["vp2"].copy(),
                                              nz=60, nx=90, hmin=75.0, wl=10, freq=2.0, grade=0.15,
                                              domain_pad=500.0, pad_style=case)
        np.testing.assert_allclose(ef.bbox, g["bbox2_" + case])
        ref, x = g["eval2_" + case], g["xq2"]
    np.testing.assert_allclose(ef.eval(x), ref, rtol=RTOL)


def test_config1_disk_matches_reference(cuda):
    """2D unit disk, h = 0.1, max_iter 50, seed 0 (the reference's own run)"""
    g = golden("disk_h01.npz")
    p, t = sm.generate_mesh(sm.Disk([0.0, 0.0], 1.0), 0.1, verbose=0)
    assert len(p) == len(g["p"]) and len(t) == len(g["t"])
    q = sm.geometry.simp_qual(p, t)
    assert abs(q.min() - g["qual"].min()) < 1e-3 * g["qual"].min()
    assert abs(q.mean() - g["qual"].mean()) < 1e-3 * g["qual"].mean()
    assert abs(sm.geometry.simp_vol(p, t).sum() - float(g["area"])) < 1e-4


def test_reference_test_2dmesher_sdf(cuda):
    """test_2dmesher_SDF.py: counts [63, 93] +- 10 and area 3.14 +- 0.2"""
    hmin = 0.2
    disk = sm.Disk([0.0, 0.0], 1)
    p, t = sm.generate_mesh(bbox=(-1.0, 1.0, -1.0, 1.0), domain=disk, h0=hmin,
                            edge_length=lambda p: hmin - disk.eval(p) * 0.15, max_iter=100, verbose=0)
    assert np.allclose([len(p), len(t)], [63, 93], atol=10)
    assert np.allclose(sm.geometry.simp_vol(p, t).sum(), 3.14, atol=hmin)


def test_reference_test_2d_min_qual(cuda):
    """test_2d_min_qual.py: quarter annulus, min quality > 0.60 at 5 sizes"""
    for h in np.logspace(-1.0, -2.0, num=5):
        rect = sm.Rectangle((0.0, 1.0, 0.0, 1.0))
        disk0 = sm.Disk([0.0, 0.0], 0.25)
        quarter = sm.Intersection([sm.Difference([rect, disk0]), sm.Disk([0.0, 0.0], 1.0)])
        p, t = sm.generate_mesh(domain=quarter, edge_length=lambda x, h=h: h + 0.1 * np.abs(disk0.eval(x)),
                                h0=h, verbose=0)
        assert sm.geometry.simp_qual(p, t).min() > 0.60


def test_ball_against_oracle_end_metrics(cuda):
    """3D unit ball h = 0.1 + sliver removal: vertex count and mean quality
    within 1% of the oracle's (reference loop, Qhull connectivity)"""
    from oracle import sdf_np as S

    p, t = sm.generate_mesh(sm.Ball([0.0, 0.0, 0.0], 1.0), 0.1, verbose=0)
    fd = S.ball(0, 0, 0, 1.0)
    po, to = O.generate_mesh(fd, lambda x: np.full(len(x), 0.1), 0.1, (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0))
    assert abs(len(p) - len(po)) <= 0.01 * len(po)
    dh = np.degrees(O.dihedral_angles(p, t)).reshape(-1, 6).min(1)
    dho = np.degrees(O.dihedral_angles(po, to)).reshape(-1, 6).min(1)
    assert abs(np.mean(dh) - np.mean(dho)) < 0.01 * np.mean(dho)
    assert abs(O.simp_vol(p, t).sum() - O.simp_vol(po, to).sum()) < 0.01 * O.simp_vol(po, to).sum()
    ps, ts = sm.sliver_removal(p, sm.Ball([0.0, 0.0, 0.0], 1.0), 0.1, verbose=0)
    dhs = np.degrees(O.dihedral_angles(ps, ts)).reshape(-1, 6).min(1)
    assert dhs.min() >= 10.0 - 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_max_movement_is_written_where_it_is_read(cuda, dim):
    """dm_update_points writes the maximum of |F| to maxf[dm_bar_blocks(n)]
    in 2D and 3D, so the value read back never comes from stale memory."""
    import torch

    from seismicmesh_gb300.generation import mesh_generator as MG

    rng = np.random.default_rng(3)
    h = 0.05
    p = rng.uniform(-0.7, 0.7, (3000, dim))
    dom = sm.Disk([0.0, 0.0], 1.0) if dim == 2 else sm.Ball([0.0, 0.0, 0.0], 1.0)
    fd = MG._Domain(dom)
    sizing = MG._Sizing(h, dim)
    eng = MG._Engine(dim, p, 0)
    eng.triangulate()
    eng.filter(fd, 0.1 * h)
    eng.build_adjacency()
    eng.maxf.fill_(1e30)
    before = eng.P[:, :dim].cpu().numpy().astype(np.float64)
    eng.step(sizing, [fd], 1 + 0.4 / 2 ** (dim - 1), 0.3, h, float(np.sqrt(np.finfo(float).eps) * h))
    m = eng.max_movement(0.3)
    after = eng.P[:, :dim].cpu().numpy().astype(np.float64)
    torch.cuda.synchronize()
    # points well inside the domain are not projected: they move by dt |F|
    inner = (np.linalg.norm(before, axis=1) < 0.9) & (np.linalg.norm(after, axis=1) < 0.9)
    disp = np.linalg.norm(after - before, axis=1)[inner].max()
    assert np.isfinite(m) and m < 1e3, m
    assert m >= disp * (1 - 1e-5), (m, disp)
