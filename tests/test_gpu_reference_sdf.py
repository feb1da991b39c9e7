"""The reference's SDF-driven mesh tests (tests/test_3dmesher_SDF.py,
test_3d_sliver.py, test_immersion.py, test_pfix.py, test_smooth_sets.py,
test_rotations.py of SeismicMesh) run through this package on the GPU with
the assertions of the reference tests."""
import math

import numpy as np
import pytest

import seismicmesh_gb300 as sm

pytestmark = pytest.mark.gpu

MIN_DH = 10 * math.pi / 180
MAX_DH = 180 * math.pi / 180


def _bad_cells(points, cells):
    dh = sm.geometry.calc_dihedral_angles(points, cells)
    out = np.argwhere((dh[:, 0] < MIN_DH) | (dh[:, 0] > MAX_DH))
    return np.unique(np.floor(out / 6).astype(int))


def test_3dmesher_sdf_callable_cylinder(cuda):
    """host-callable domain and edge length (the slow path): unit cylinder
    volume 2 pi within h"""
    hmin = 0.10
    bbox = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)

    def cylinder(p):
        r, z = np.sqrt(p[:, 0] ** 2 + p[:, 1] ** 2), p[:, 2]
        d1, d2, d3 = r - 1.0, z - 1.0, -z - 1.0
        d4, d5 = np.sqrt(d1**2 + d2**2), np.sqrt(d1**2 + d3**2)
        d = np.maximum.reduce([d1, d2, d3])
        ix = (d1 > 0) * (d2 > 0)
        d[ix] = d4[ix]
        ix = (d1 > 0) * (d3 > 0)
        d[ix] = d5[ix]
        return d

    def ef(p):
        return np.array([hmin] * len(p))

    points, cells = sm.generate_mesh(bbox=bbox, domain=cylinder, h0=hmin, edge_length=ef, max_iter=100,
                                     verbose=0)
    points, cells = sm.sliver_removal(points=points, domain=cylinder, edge_length=ef, h0=hmin, bbox=bbox,
                                      verbose=0)
    assert np.allclose(np.sum(sm.geometry.simp_vol(points, cells)), 6.28, atol=hmin)


def _cylinder(h):
    dom = sm.Cylinder(h=1.0, r=1.0)
    p, c = sm.generate_mesh(domain=dom, edge_length=h, verbose=0)
    return sm.sliver_removal(points=p, domain=dom, edge_length=h, verbose=0)


def _l_shape(h):
    tol = h / 10
    dom = sm.Union([sm.Cube((-1.0, 1.0, -1.0, 1.0, -1.0, tol)), sm.Cube((-1.0, 1.0, 0.0, 1.0, -tol, 1.0)),
                    sm.Cube((-tol, 1.0, -1.0, 1.0, -tol, 1.0))])
    p, c = sm.generate_mesh(domain=dom, edge_length=h, verbose=0)
    return sm.sliver_removal(domain=dom, points=p, edge_length=h, verbose=0)


def _box_refined(h):
    cube = sm.Cube((-1.0, 1.0, -1.0, 1.0, -1.0, 1.0))

    def edge_length(x):
        return h + 0.1 * np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2 + x[:, 2] ** 2)

    p, c = sm.generate_mesh(domain=cube, h0=h, edge_length=edge_length, verbose=0)
    return sm.sliver_removal(domain=cube, points=p, h0=h, edge_length=edge_length, verbose=0)


@pytest.mark.parametrize("shape,hs", [
    ("cylinder", np.logspace(-1.0, -1.3, num=5)),
    ("l_shape", np.logspace(-1.0, -1.2, num=5)),
    ("box_refined", np.logspace(-1.0, -1.3, num=5)),
])
def test_3d_sliver(cuda, shape, hs):
    make = {"cylinder": _cylinder, "l_shape": _l_shape, "box_refined": _box_refined}[shape]
    for h in hs:
        points, cells = make(h)
        assert len(_bad_cells(points, cells)) == 0, (shape, h)


def test_immersion(cuda):
    hmin = 0.05
    for radius in (0.25, 0.30, 0.35):
        box0 = sm.Rectangle((0.0, 1.0, 0.0, 1.0))
        disk0 = sm.Disk([0.5, 0.5], radius)

        def fh(p):
            return 0.05 * np.abs(disk0.eval(p)) + hmin

        points, cells = sm.generate_mesh(domain=box0, edge_length=fh, h0=hmin, subdomains=[disk0], verbose=0)
        pmid = points[cells].sum(1) / 3
        sd = disk0.eval(pmid)
        vol = np.sum(sm.geometry.simp_vol(points, cells[sd < 0]))
        assert np.isclose(vol, np.pi * radius**2, rtol=1e-2), (radius, vol)


def test_pfix(cuda):
    hmin = 0.05
    bbox = (0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    pfix = np.linspace((0.0, 0.0, 0.0), (1.0, 0.0, 1.0), int(np.sqrt(2) / hmin))
    pfix = np.vstack((pfix, sm.geometry.corners(bbox)))
    points, cells = sm.generate_mesh(domain=sm.Cube(bbox), edge_length=hmin, pfix=pfix, verbose=0)
    for q in pfix:
        d = np.einsum("ij,ij->i", points - q, points - q)
        # fixed points are kept (float32 positions: to within their rounding)
        assert np.min(d) < 1e-12, (q, np.min(d))


def test_smooth_sets(cuda):
    domain = sm.Difference([sm.Ball((0.0, 0.0, 0.5), 0.85), sm.Cube((-0.5, 0.5, -0.5, 0.5, -0.5, 0.5))],
                           smoothness=0.20)
    points, cells = sm.generate_mesh(domain=domain, edge_length=0.10, verbose=0)
    points, cells = sm.sliver_removal(points=points, domain=domain, edge_length=0.10, verbose=0)
    assert np.abs(cells.shape[0] - 9004) < 100, cells.shape


@pytest.mark.parametrize("dim", [2, 3])
def test_rotations(cuda, dim):
    if dim == 2:
        geo = [sm.Disk((0.5, 0.5), 0.1, rotate=[0.2 * 3.14, 0, 0]),
               sm.Rectangle((0.0, 1.0, 0.0, 1.0), rotate=[0.3 * 3.14, 0, 0])]
    else:
        bbox = (0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
        geo = [sm.Ball((0.5, 0.5, 0.5), 0.1, rotate=[0.0, 0, 0]), sm.Cube(bbox, rotate=[0.4 * 3.14, 0, 0]),
               sm.Torus(1.0, 0.5, rotate=[0.4 * 3.14, 0, 0]), sm.Prism(0.5, 0.5, rotate=[0.5 * 3.14, 0, 0]),
               sm.Cylinder(1.0, 0.5, rotate=[0.6 * 3.14, 0, 0]),
               sm.Ball((0.5, 0.5, 0.5), 0.1, rotate=[0.0, 0.0, 0.0]),
               sm.Cube(bbox, rotate=[0.4 * 3.14, 0.4 * 3.14, 0.4 * 3.14]),
               sm.Torus(1.0, 0.5, rotate=[0.4 * 3.14, 0.4 * 3.14, 0.4 * 3.14]),
               sm.Prism(0.5, 0.5, rotate=[0.5 * 3.14, 0.2 * 3.14, 0.4 * 3.14]),
               sm.Cylinder(1.0, 0.5, rotate=[0.0, 0.6 * 3.14, 0.3 * 3.14])]
    for domain in geo:
        p, c = sm.generate_mesh(domain=domain, edge_length=0.1, verbose=0)
        assert len(c) > 0 and np.all(np.isfinite(p))
        assert np.all(sm.geometry.simp_vol(p, c) > 0)
