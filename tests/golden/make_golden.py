"""Generates the golden fixtures in tests/golden/ by running the reference
SeismicMesh (through oracle/ref_harness.py) in the build container.

    python tests/golden/make_golden.py

Fixtures are small .npz/.json files; the GPU tests and the oracle tests read
them, the reference itself is not needed afterwards.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_harness  # noqa: E402

SM = ref_harness.load()
from SeismicMesh.generation import mesh_generator as MG  # noqa: E402
from SeismicMesh import geometry as G  # noqa: E402
from _fast_geometry import calc_circumsphere_grad, calc_dihedral_angles, unique_edges  # noqa: E402
from _FastHJ import limgrad  # noqa: E402


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name), **arrays)
    print("wrote", name, {k: getattr(v, "shape", v) for k, v in arrays.items()})


def perturbed_lattice(domain, h, dim, seed, jitter=0.2):
    """generic-position points inside a domain: a jittered lattice"""
    rng = np.random.default_rng(seed)
    bbox = np.array(domain.bbox).reshape(-1, 2)
    axes = [np.arange(lo - h, hi + h, h) for lo, hi in bbox]
    p = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, dim)
    p = p + jitter * h * rng.uniform(-1, 1, p.shape)
    p = p[domain.eval(p) < 0.1 * h]
    return f32(p)


def one_iteration(domain, h, dim, seed):
    """one DistMesh update with the reference's own functions
    (generation/mesh_generator.py:465-506) on generic points"""
    p = perturbed_lattice(domain, h, dim, seed)
    fd = domain.eval
    fh, _, hmin, _ = MG._unpack_sizing(h)
    L0mult = 1 + 0.4 / 2 ** (dim - 1)
    geps = 0.1 * h
    deps = np.sqrt(np.finfo(np.double).eps) * h
    DT = MG._select_cgal_dim(dim)
    dt = DT()
    dt.insert(p.ravel().tolist())
    q, t = MG._get_topology(dt)
    assert np.array_equal(q, p)
    t = MG._remove_triangles_outside(q, t, fd, geps)
    F = MG._compute_forces(q, t, fh, h, L0mult)
    p1 = q + 0.30 * F
    p1 = MG._project_points_back_newton(p1, fd, deps, h, 0)
    return dict(p0=q, t=t.astype(np.int32), F=F, p1=p1, h=np.float64(h))


def main():
    rng = np.random.default_rng(1234)
    # --- config 1: 2D unit disk, h = 0.1, max_iter 50, seed 0
    p, t = SM.generate_mesh(SM.Disk([0.0, 0.0], 1.0), 0.1, verbose=0)
    q = G.simp_qual(p, t)
    save("disk_h01.npz", p=p, t=t.astype(np.int32), qual=q, area=np.float64(G.simp_vol(p, t).sum()))

    # --- single iterations on generic points (2D disk, 3D ball, 2D box, 3D box)
    save("iter_disk.npz", **one_iteration(SM.Disk([0.0, 0.0], 1.0), 0.1, 2, 1))
    save("iter_ball.npz", **one_iteration(SM.Ball([0.0, 0.0, 0.0], 1.0), 0.2, 3, 2))
    save("iter_rect.npz", **one_iteration(SM.Rectangle((0.0, 1.0, 0.0, 2.0)), 0.1, 2, 3))
    save("iter_cube.npz", **one_iteration(SM.Cube((0.0, 1.0, 0.0, 1.0, 0.0, 1.0)), 0.2, 3, 4))

    # --- signed distance functions at random points
    x2 = f32(rng.uniform(-2, 2, (4000, 2)))
    x3 = f32(rng.uniform(-2, 2, (4000, 3)))
    shapes = {
        "disk": SM.Disk([0.1, -0.2], 0.9),
        "disk_rot": SM.Disk([0.1, -0.2], 0.9, rotate=[0.4, 0, 0], stretch=[2.0, 1.0], translate=[0.3, 0.1]),
        "rect": SM.Rectangle((-0.5, 1.0, -0.7, 0.4)),
        "rect_rot": SM.Rectangle((-0.5, 1.0, -0.7, 0.4), rotate=[0.3, 0, 0], translate=[0.1, 0.2]),
        "ball": SM.Ball([0.1, 0.0, -0.1], 0.8),
        "ball_xf": SM.Ball([0.1, 0.0, -0.1], 0.8, rotate=[0.2, 0.3, 0.4], stretch=[1.0, 2.0, 1.5], translate=[0.1, 0.2, 0.3]),
        "cube": SM.Cube((-0.5, 0.5, -0.6, 0.4, -0.2, 0.9)),
        "cube_rot": SM.Cube((-0.5, 0.5, -0.6, 0.4, -0.2, 0.9), rotate=[0.5, 0.0, 0.25]),
        "torus": SM.Torus(0.8, 0.3),
        "prism": SM.Prism(0.6, 0.4),
        "cylinder": SM.Cylinder(h=1.2, r=0.5),
        "cylinder_rot": SM.Cylinder(h=1.2, r=0.5, rotate=[0.3, 0.0, 0.6]),
        "union2": SM.Union([SM.Disk([0.0, 0.0], 0.5), SM.Rectangle((0.0, 1.0, -0.2, 0.3))]),
        "union2_smooth": SM.Union([SM.Disk([0.0, 0.0], 0.5), SM.Rectangle((0.0, 1.0, -0.2, 0.3))], smoothness=0.1),
        "inter2": SM.Intersection([SM.Disk([0.0, 0.0], 0.8), SM.Rectangle((0.0, 1.0, -0.5, 0.5))]),
        "inter2_smooth": SM.Intersection([SM.Disk([0.0, 0.0], 0.8), SM.Rectangle((0.0, 1.0, -0.5, 0.5))], smoothness=0.2),
        "diff2": SM.Difference([SM.Rectangle((-1.0, 1.0, -1.0, 1.0)), SM.Disk([0.0, 0.0], 0.4), SM.Disk([0.6, 0.6], 0.2)]),
        "diff3_smooth": SM.Difference([SM.Ball((0.0, 0.0, 0.5), 0.85), SM.Cube((-0.5, 0.5, -0.5, 0.5, -0.5, 0.5))], smoothness=0.2),
        "union3": SM.Union([SM.Ball((0.0, 0.0, 0.0), 0.5), SM.Cube((0.0, 1.0, -0.2, 0.2, -0.2, 0.2))]),
    }
    sdf = {}
    for name, s in shapes.items():
        x = x2 if s.dim == 2 else x3
        sdf[name] = s.eval(x)
        sdf[name + "_bbox"] = np.asarray(s.bbox, dtype=float)
        if s.corners is not None:
            sdf[name + "_corners"] = np.asarray(s.corners, dtype=float)
    save("sdf.npz", x2=x2, x3=x3, **sdf)

    # --- fast_geometry kernels
    e = rng.integers(0, 300, (5000, 2)).astype(np.int32)
    ue = unique_edges(e)
    pt = f32(rng.uniform(-1, 1, (60, 3)))
    tt = rng.integers(0, 60, (400, 4)).astype(np.int32)
    tt = tt[np.array([len(set(r)) == 4 for r in tt])]
    dh = calc_dihedral_angles(pt, tt)
    g = calc_circumsphere_grad(pt[tt[:, 0]], pt[tt[:, 1]], pt[tt[:, 2]], pt[tt[:, 3]])
    save("fast_geometry.npz", edges=e, unique=ue, points=pt, cells=tt, dihedral=dh, cgrad=g)

    # --- limgrad
    lg = {}
    for key, dims in (("kat", (3, 3, 1)), ("g2", (37, 41, 1)), ("g3", (13, 11, 9))):
        f = np.array([1.0, 5, 5, 5, 5, 5, 5, 5, 5]) if key == "kat" else rng.uniform(75, 300, int(np.prod(dims)))
        lg[key + "_in"] = f
        lg[key + "_out"] = np.asarray(limgrad(list(dims), 12.5, 0.15, 10000, f)).reshape(-1)
        lg[key + "_dims"] = np.array(dims)
    save("limgrad.npz", **lg)

    # --- sizing from a synthetic velocity model (2D and 3D, pad styles)
    sz = {}
    vp2 = np.zeros((60, 90))
    for i in range(60):
        vp2[i] = 1500 + 3000 * i / 59
    vp2 += rng.normal(0, 50, vp2.shape)
    vp2[:5] = 0.0  # water (vs) rows
    bbox2 = (-6000.0, 0.0, 0.0, 18000.0)
    xq2 = f32(np.column_stack([rng.uniform(-6500, 500, 3000), rng.uniform(-500, 18500, 3000)]))
    for style in ("edge", "constant", "linear_ramp"):
        ef = SM.get_sizing_function_from_segy(
            None, bbox2, velocity_data=vp2.copy(), nz=60, nx=90, hmin=75.0, wl=10, freq=2.0,
            grade=0.15, domain_pad=500.0, pad_style=style)
        sz["eval2_" + style] = ef.eval(xq2)
        sz["bbox2_" + style] = np.asarray(ef.bbox)
    ef = SM.get_sizing_function_from_segy(None, bbox2, velocity_data=vp2.copy(), nz=60, nx=90,
                                          hmin=75.0, wl=10, freq=2.0, grade=0.15, dt=0.001, cr_max=0.5)
    sz["eval2_courant"] = ef.eval(xq2)
    vp3 = 1500 + 2500 * np.linspace(0, 1, 21)[:, None, None] * np.ones((21, 17, 15))
    vp3 += rng.normal(0, 40, vp3.shape)
    bbox3 = (-4200.0, 0.0, 0.0, 3400.0, 0.0, 3000.0)
    xq3 = f32(np.column_stack([rng.uniform(-4300, 100, 3000), rng.uniform(-100, 3500, 3000), rng.uniform(-100, 3100, 3000)]))
    ef = SM.get_sizing_function_from_segy(None, bbox3, velocity_data=vp3.copy(), nz=21, nx=17, ny=15,
                                          hmin=50.0, wl=10, freq=2.0, grade=0.15)
    sz["eval3"] = ef.eval(xq3)
    save("sizing.npz", vp2=vp2, bbox2=np.asarray(bbox2), xq2=xq2, vp3=vp3, bbox3=np.asarray(bbox3), xq3=xq3, **sz)

    # --- reference test goldens, re-run here through the harness
    out = {}
    hmin = 0.2
    disk = SM.Disk([0.0, 0.0], 1)
    p, t = SM.generate_mesh(bbox=(-1.0, 1.0, -1.0, 1.0), domain=disk, h0=hmin,
                            edge_length=lambda p: hmin - disk.eval(p) * 0.15, max_iter=100, verbose=0)
    out["test_2dmesher_SDF"] = {"golden": [63, 93], "atol": 10, "area_golden": 3.14, "area_atol": 0.2,
                                "ref_harness": [int(len(p)), int(len(t))], "ref_area": float(G.simp_vol(p, t).sum())}
    quals = []
    for h in np.logspace(-1.0, -2.0, num=5):
        rect = SM.Rectangle((0.0, 1.0, 0.0, 1.0))
        d0 = SM.Disk([0.0, 0.0], 0.25)
        quarter = SM.Intersection([SM.Difference([rect, d0]), SM.Disk([0.0, 0.0], 1.0)])
        p, t = SM.generate_mesh(domain=quarter, edge_length=lambda x, h=h: h + 0.1 * np.abs(d0.eval(x)), h0=h, verbose=0)
        quals.append(float(G.simp_qual(p, t).min()))
    out["test_2d_min_qual"] = {"bound": 0.60, "ref_harness_min_quals": quals}
    with open(os.path.join(HERE, "reference_tests.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
