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


def gradient_goldens():
    """reference _gradient_sizing (sizing/mesh_size_function.py:428-448) and a
    sizing pipeline with grad > 0"""
    from SeismicMesh.sizing.mesh_size_function import _gradient_sizing

    rng = np.random.default_rng(99)
    out = {}
    cases = {
        "g2": ((15, 25), 10.0),
        "g2w": ((9, 14), (40, 3)),  # windows larger than the grid
        "g3": ((12, 9, 7), (3, 4, 5)),
    }
    for key, (shape, st) in cases.items():
        vp = 1500 + 3000 * rng.random(shape)
        vp[: shape[0] // 3] = 1500.0  # a flat layer: zero variance somewhere
        out[key + "_vp"] = vp
        out[key + "_stencil"] = np.atleast_1d(np.asarray(st, dtype=float))
        out[key + "_out"] = _gradient_sizing(vp.copy(), 50.0, st)
    vp2 = np.zeros((60, 90))
    for i in range(60):
        vp2[i] = 1500 + 3000 * i / 59
    vp2 += rng.normal(0, 50, vp2.shape)
    vp2[20:35, 30:60] = 4500.0  # a block of salt
    bbox2 = (-6000.0, 0.0, 0.0, 18000.0)
    xq2 = f32(np.column_stack([rng.uniform(-6000, 0, 3000), rng.uniform(0, 18000, 3000)]))
    ef = SM.get_sizing_function_from_segy(None, bbox2, velocity_data=vp2.copy(), nz=60, nx=90,
                                          hmin=75.0, wl=10, freq=2.0, grad=120.0, grade=0.15)
    out.update(vp2=vp2, bbox2=np.asarray(bbox2), xq2=xq2, eval2=ef.eval(xq2))
    save("gradient.npz", **out)


def reference_test_goldens():
    """the reference's mesh tests that read its own velocity fixtures and its
    remaining SDF tests, re-run through the harness; only decoded velocity
    arrays are stored (not the fixture files)"""
    from SeismicMesh.sizing.mesh_size_function import read_velocity_model

    tdir = os.path.join(ref_harness.REF, "tests")
    # segyio (the reference's SEG-Y reader) is not installed: decode the SEG-Y
    # rev 1 layout directly (3200-byte text and 400-byte binary headers,
    # 240-byte trace headers, IBM float samples), traces as columns, then
    # flipped like the reference's _read_segy
    raw = open(os.path.join(tdir, "testing.segy"), "rb").read()
    ns = int.from_bytes(raw[3220:3222], "big")
    assert int.from_bytes(raw[3224:3226], "big") == 1  # IBM float samples
    ntr = (len(raw) - 3600) // (240 + 4 * ns)
    words = np.frombuffer(raw[3600:], ">u4").reshape(ntr, 60 + ns)[:, 60:].astype(np.uint64)
    sign = 1.0 - 2.0 * ((words >> 31) & 1).astype(float)
    expo = ((words >> 24) & 0x7F).astype(int) - 64
    frac = (words & 0xFFFFFF).astype(float) / 2.0**24
    vp2 = np.flipud((sign * frac * 16.0 ** expo).T)
    nz2, nx2 = vp2.shape
    vp3, nz3, nx3, ny3 = read_velocity_model(os.path.join(tdir, "test3D.bin"), nz=20, nx=10, ny=10,
                                             byte_order="little", axes_order=(2, 0, 1),
                                             axes_order_sort="F", dtype="float32")
    save("velocity_fixtures.npz", segy_vp=np.asarray(vp2), bin_vp=np.asarray(vp3))
    res = {}

    def counts(p, t):
        return [int(len(p)), int(len(t))]

    # test_2dmesher_vs_water / test_2dmesher_r0m_values: water layer sizing
    bbox = (-10000.0, 0.0, 0.0, 10000.0)
    rect = SM.Rectangle(bbox)
    vs = np.zeros((200, 200))
    vs[0:150, :] = 1000
    for hmin, key in ((10, "vs_water"), (75, "r0m")):
        ef = SM.get_sizing_function_from_segy(None, bbox=bbox, grade=0.0, grad=0.0, wl=5, freq=2.0,
                                              hmin=hmin, hmax=10e6, velocity_data=vs.copy(), nz=200, nx=200)
        if key == "vs_water":
            ef.hmin = None
            p, t = SM.generate_mesh(rect, ef, h0=125, perform_checks=True, verbose=0)
            res["vs_water"] = {"golden": [5616, 10955], "atol": 100, "harness": counts(p, t)}
        else:
            runs = []
            for r0m, efh in ((False, 75), (True, 75), (True, 100)):
                ef.hmin = efh
                p, t = SM.generate_mesh(rect, ef, h0=125, perform_checks=True, r0m_is_h0=r0m, verbose=0)
                runs.append(counts(p, t))
            res["r0m"] = {"golden": [[15460, 30464], [10566, 20771], [8739, 17131]], "atol": 100,
                          "harness": runs}
    # test_2dmesher (testing.segy)
    ef = SM.get_sizing_function_from_segy(None, bbox=bbox, grade=0.005, grad=50.0, wl=5, freq=5.0,
                                          hmin=100, hmax=10e6, velocity_data=np.asarray(vp2).copy(),
                                          nz=nz2, nx=nx2)
    p, t = SM.generate_mesh(rect, ef, h0=100, perform_checks=True, verbose=0)
    res["segy2d"] = {"golden": [7690, 15045], "atol": 100, "harness": counts(p, t)}
    # test_2dmesher_domain_extension
    ext = {}
    for style, ans in (("linear_ramp", [9428, 18525]), ("edge", [9724, 19078]), ("constant", [9428, 18525])):
        ef = SM.get_sizing_function_from_segy(None, bbox=bbox, grade=0.005, grad=50.0, stencil_size=100,
                                              wl=5, freq=5.0, hmin=100, hmax=10e6, pad_style=style,
                                              domain_pad=1e3, velocity_data=np.asarray(vp2).copy(),
                                              nz=nz2, nx=nx2)
        p, t = SM.generate_mesh(rect, ef, h0=100, perform_checks=True, verbose=0)
        ext[style] = {"golden": ans, "harness": counts(p, t)}
    res["domain_extension_2d"] = ext
    # test_3dmesher (test3D.bin) and test_3dmesher_domain_extension
    bbox3 = (-2e3, 0.0, 0.0, 1e3, 0.0, 1e3)
    cube = SM.Cube(bbox3)
    ef = SM.get_sizing_function_from_segy(None, bbox3, grade=0.005, grad=50, freq=2, wl=10, hmin=50,
                                          nz=20, nx=10, ny=10, domain_pad=0.0,
                                          velocity_data=np.asarray(vp3).copy())
    p, t = SM.generate_mesh(domain=cube, edge_length=ef, h0=50, max_iter=25, perform_checks=False, verbose=0)
    p, t = SM.sliver_removal(points=p, edge_length=ef, domain=cube, h0=50, verbose=0)
    res["bin3d"] = {"golden": [16459, 89240], "atol": 100, "harness": counts(p, t)}
    ext3 = {}
    for style, ans in (("linear_ramp", [1388, 6592]), ("edge", [1383, 6545]), ("constant", [1406, 6622])):
        ef = SM.get_sizing_function_from_segy(None, bbox3, grade=0.005, grad=150, freq=2, wl=5, hmin=150,
                                              nz=20, nx=10, ny=10, domain_pad=200, pad_style=style,
                                              velocity_data=np.asarray(vp3).copy())
        p, t = SM.generate_mesh(domain=cube, edge_length=ef, h0=150, perform_checks=False, verbose=0)
        p, t = SM.sliver_removal(points=p, domain=cube, edge_length=ef, h0=150, verbose=0)
        ext3[style] = {"golden": ans, "harness": counts(p, t)}
    res["domain_extension_3d"] = ext3
    with open(os.path.join(HERE, "reference_tests2.json"), "w") as fh:
        json.dump(res, fh, indent=1)
    print(json.dumps(res, indent=1))


def repeat_goldens():
    """geometry.Repeat (signed_distance_functions.py:283-297) at random points"""
    from SeismicMesh.geometry.signed_distance_functions import Repeat

    rng = np.random.default_rng(41)
    x = f32(rng.uniform(-1.2, 1.2, (5000, 3)))
    bbox = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    cases = {
        "ball": Repeat(bbox, SM.Ball([0.0, 0.0, 0.0], 0.12), [0.4, 0.4, 0.4]),
        "ball_aniso": Repeat(bbox, SM.Ball([0.0, 0.0, 0.0], 0.1), [0.3, 0.5, 0.45]),
        "union": Repeat(bbox, SM.Union([SM.Ball([0.0, 0.0, 0.0], 0.1), SM.Cube((-0.05, 0.05, -0.2, 0.2, -0.05, 0.05))]),
                        [0.5, 0.5, 0.5]),
    }
    save("repeat.npz", x=x, **{k: v.eval(x) for k, v in cases.items()})


def folded(p, t, dim, h, seed, k=6, scale=0.8):
    """a mesh with overlapping cells: k interior vertices pushed by scale*h"""
    rng = np.random.default_rng(seed)
    p = p.copy()
    bnd = set(G.get_boundary_vertices(t, dim=dim).tolist())
    interior = np.array([v for v in range(len(p)) if v not in bnd])
    pick = rng.choice(interior, k, replace=False)
    d = rng.normal(size=(k, dim))
    p[pick] += scale * h * d / np.linalg.norm(d, axis=1, keepdims=True)
    return p


def qa_goldens():
    """mesh quality and linting: calc_re_ratios (geometry/utils.py:17-54),
    do_any_overlap (745-817) and linter (820-872) on small meshes"""
    import contextlib
    import io

    disk = np.load(os.path.join(HERE, "disk_h01.npz"))
    ball = np.load(os.path.join(HERE, "iter_ball.npz"))
    p2, t2 = disk["p"], disk["t"].astype(np.int64)
    p3, t3 = ball["p0"], ball["t"].astype(np.int64)
    out = dict(p2=p2, t2=t2, p3=p3, t3=t3)
    out["re2"] = G.calc_re_ratios(p2, t2, dim=2)
    out["re3"] = G.calc_re_ratios(p3, t3, dim=3)
    out["f2"] = folded(p2, t2, 2, 0.1, 7, k=12, scale=1.6)
    out["f3"] = folded(p3, t3, 3, 0.2, 8, scale=0.6)
    sink = io.StringIO()
    with contextlib.redirect_stdout(sink):
        out["ov2"] = np.array(G.do_any_overlap(out["f2"], t2, dim=2), dtype=np.int64).reshape(-1, 2)
        out["ov3"] = np.array(G.do_any_overlap(out["f3"], t3, dim=3), dtype=np.int64).reshape(-1, 2)
        out["ov2_clean"] = np.array(G.do_any_overlap(p2, t2, dim=2), dtype=np.int64).reshape(-1, 2)
        lp, lt = G.linter(out["f2"], t2, dim=2)
    out["lint2_p"], out["lint2_t"] = lp, lt.astype(np.int64)
    save("mesh_qa.npz", **out)


if __name__ == "__main__":
    parts = sys.argv[1:] or ["main"]
    for part in parts:
        {"main": main, "gradient": gradient_goldens, "reftests2": reference_test_goldens,
         "repeat": repeat_goldens, "qa": qa_goldens}[part]()
