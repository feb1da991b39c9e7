"""The reference's own sizing and meshing tests that read its velocity
fixtures (tests/test_2dmesher*.py, tests/test_3dmesher*.py of SeismicMesh),
run through this package on the GPU.  Goldens: the counts the reference
tests assert (where they assert) and the counts of the reference itself run
through the oracle harness (tests/golden/make_golden.py gradient reftests2);
the decoded velocity fixtures are stored as arrays, not as the files.

Tolerances: the reference tests use atol=100 on vertex and cell counts;
here counts must agree with the reference run within 1 % (the generation
tolerance of the configurations).  The triangulations differ only on the
degenerate initial lattice (tie-breaking) and through float32 positions.
Every comparison prints its relative difference."""
import json
import os

import numpy as np
import pytest

import seismicmesh_gb300 as sm
from seismicmesh_gb300.sizing.mesh_size_function import _gradient_sizing

from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu

REFT = json.load(open(os.path.join(GOLDEN, "reference_tests2.json")))


def _close(got, want, rel=0.01):
    for g, w in zip(got, want):
        print(f"count: gpu {g} reference {w} rel {(g - w) / w:+.3e}")
    return all(abs(g - w) <= rel * w for g, w in zip(got, want))


@pytest.mark.parametrize("case", ["g2", "g2w", "g3"])
def test_gradient_sizing_matches_reference(cuda, case):
    g = golden("gradient.npz")
    st = g[case + "_stencil"]
    st = float(st[0]) if len(st) == 1 else tuple(int(x) for x in st)
    got = _gradient_sizing(g[case + "_vp"], 50.0, st)
    np.testing.assert_allclose(got, g[case + "_out"], rtol=1e-9)


def test_sizing_with_gradient_term_matches_reference(cuda):
    g = golden("gradient.npz")
    ef = sm.get_sizing_function_from_segy(None, tuple(g["bbox2"]), velocity_data=g["vp2"].copy(),
                                          nz=60, nx=90, hmin=75.0, wl=10, freq=2.0, grad=120.0, grade=0.15)
    np.testing.assert_allclose(ef.eval(g["xq2"]), g["eval2"], rtol=1e-5)


def _water_sizing(hmin):
    vs = np.zeros((200, 200))
    vs[0:150, :] = 1000
    return sm.get_sizing_function_from_segy(None, bbox=(-10000.0, 0.0, 0.0, 10000.0), grade=0.0, grad=0.0,
                                            wl=5, freq=2.0, hmin=hmin, hmax=10e6, velocity_data=vs,
                                            nz=200, nx=200)


def test_2dmesher_vs_water(cuda):
    ef = _water_sizing(10)
    assert ef.eval((-5000, 5000)) == 100
    assert ef.eval((-1, 5000)) == 150
    ef.hmin = None
    p, t = sm.generate_mesh(sm.Rectangle((-10000.0, 0.0, 0.0, 10000.0)), ef, h0=125, perform_checks=True,
                            verbose=0)
    r = REFT["vs_water"]
    assert np.allclose([len(p), len(t)], r["golden"], atol=r["atol"]), (len(p), len(t))
    assert _close([len(p), len(t)], r["harness"]), (len(p), len(t), r["harness"])


def test_2dmesher_r0m_values(cuda):
    ef = _water_sizing(75)
    assert ef.eval((-5000, 5000)) == 100
    assert ef.eval((-1, 5000)) == 150
    rect = sm.Rectangle((-10000.0, 0.0, 0.0, 10000.0))
    r = REFT["r0m"]
    for k, (r0m, efh) in enumerate(((False, 75), (True, 75), (True, 100))):
        ef.hmin = efh
        p, t = sm.generate_mesh(rect, ef, h0=125, perform_checks=True, r0m_is_h0=r0m, verbose=0)
        assert np.allclose([len(p), len(t)], r["golden"][k], atol=r["atol"]), (k, len(p), len(t))
        assert _close([len(p), len(t)], r["harness"][k]), (k, len(p), len(t), r["harness"][k])


def _segy_sizing(**kw):
    vp = golden("velocity_fixtures.npz")["segy_vp"]
    nz, nx = vp.shape
    return sm.get_sizing_function_from_segy(None, bbox=(-10000.0, 0.0, 0.0, 10000.0), grade=0.005,
                                            grad=50.0, wl=5, freq=5.0, hmin=100, hmax=10e6,
                                            velocity_data=vp.copy(), nz=nz, nx=nx, **kw)


def test_2dmesher_segy(cuda):
    ef = _segy_sizing()
    p, t = sm.generate_mesh(sm.Rectangle((-10000.0, 0.0, 0.0, 10000.0)), ef, h0=100, perform_checks=True,
                            verbose=0)
    assert _close([len(p), len(t)], REFT["segy2d"]["harness"]), (len(p), len(t), REFT["segy2d"])


@pytest.mark.parametrize("style", ["linear_ramp", "edge", "constant"])
def test_2dmesher_domain_extension(cuda, style):
    ef = _segy_sizing(stencil_size=100, pad_style=style, domain_pad=1e3)
    p, t = sm.generate_mesh(sm.Rectangle((-10000.0, 0.0, 0.0, 10000.0)), ef, h0=100, perform_checks=True,
                            verbose=0)
    r = REFT["domain_extension_2d"][style]
    assert _close([len(p), len(t)], r["harness"]), (style, len(p), len(t), r)


def _bin_sizing(**kw):
    vp = golden("velocity_fixtures.npz")["bin_vp"]
    return sm.get_sizing_function_from_segy(None, (-2e3, 0.0, 0.0, 1e3, 0.0, 1e3), grade=0.005, nz=20,
                                            nx=10, ny=10, velocity_data=vp.copy(), **kw)


def test_3dmesher_bin(cuda):
    bbox = (-2e3, 0.0, 0.0, 1e3, 0.0, 1e3)
    ef = _bin_sizing(grad=50, freq=2, wl=10, hmin=50, domain_pad=0.0)
    cube = sm.Cube(bbox)
    p, t = sm.generate_mesh(domain=cube, edge_length=ef, h0=50, max_iter=25, perform_checks=False, verbose=0)
    p, t = sm.sliver_removal(points=p, edge_length=ef, domain=cube, h0=50, verbose=0)
    assert _close([len(p), len(t)], REFT["bin3d"]["harness"]), (len(p), len(t), REFT["bin3d"])


@pytest.mark.parametrize("style", ["linear_ramp", "edge", "constant"])
def test_3dmesher_domain_extension(cuda, style):
    bbox = (-2e3, 0.0, 0.0, 1e3, 0.0, 1e3)
    ef = _bin_sizing(grad=150, freq=2, wl=5, hmin=150, domain_pad=200, pad_style=style)
    cube = sm.Cube(bbox)
    p, t = sm.generate_mesh(domain=cube, edge_length=ef, h0=150, perform_checks=False, verbose=0)
    p, t = sm.sliver_removal(points=p, domain=cube, edge_length=ef, h0=150, verbose=0)
    r = REFT["domain_extension_3d"][style]
    assert _close([len(p), len(t)], r["harness"]), (style, len(p), len(t), r)


def test_sizing_from_binary_file_streams_to_the_device(cuda, tmp_path):
    """a binary model given by file name is streamed into the device grid
    (read_velocity_model_to_device); the size function equals, bit for bit,
    the ones built from the same model passed as a host array and as a
    device tensor"""
    import torch

    from seismicmesh_gb300.sizing.mesh_size_function import _read_bin

    vp = golden("velocity_fixtures.npz")["bin_vp"]
    f = tmp_path / "bin_vp.bin"
    np.asarray(vp, dtype=np.float32).reshape(-1, order="F").astype("<f4").tofile(str(f))
    host, *_ = _read_bin(str(f), 20, 10, 10, "little", (0, 1, 2), "F", "float32")
    bbox = (-2e3, 0.0, 0.0, 1e3, 0.0, 1e3)
    kw = dict(grade=0.005, nz=20, nx=10, ny=10, grad=50, freq=2, wl=10, hmin=50, domain_pad=0.0)
    ef_file = sm.get_sizing_function_from_segy(str(f), bbox, byte_order="little", **kw)
    ef_host = sm.get_sizing_function_from_segy(None, bbox, velocity_data=host.copy(), **kw)
    dev = torch.from_numpy(np.ascontiguousarray(host)).cuda()
    ef_dev = sm.get_sizing_function_from_segy(None, bbox, velocity_data=dev, **kw)
    assert torch.equal(dev, torch.from_numpy(np.ascontiguousarray(host)).cuda())  # input untouched
    rng = np.random.default_rng(8)
    x = rng.uniform([-2e3, 0.0, 0.0], [0.0, 1e3, 1e3], size=(5000, 3))
    want = ef_host.eval(x)
    np.testing.assert_array_equal(ef_file.eval(x), want)
    np.testing.assert_array_equal(ef_dev.eval(x), want)
