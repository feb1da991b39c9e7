"""Isosurface SDF kernels against the numpy oracle (oracle/iso_np.py) on a
small field of two Gaussian bumps, through the C ABI.

Tolerances: triangle vertices within 1e-5 of the grid extent (float32 edge
parameters against float64); signed distances within 1e-4 of the extent
(float32 point-triangle arithmetic); signs identical away from the surface
(|d| > 1e-4 of the extent); gradients within 1e-3."""
import numpy as np
import pytest
import torch

import seismicmesh_gb300 as sm
from oracle import iso_np as I
from seismicmesh_gb300 import _device as D
from seismicmesh_gb300 import _native as N

pytestmark = pytest.mark.gpu

BBOX = (-1.0, 0.0, 0.0, 2.5, 0.0, 2.0)


def _field(n=(14, 23, 19)):
    axes = [np.linspace(BBOX[2 * k], BBOX[2 * k + 1], n[k]) for k in range(3)]
    Z, X, Y = np.meshgrid(*axes, indexing="ij")
    B = (0.9 * np.exp(-(((Z + 0.5) / 0.25) ** 2 + ((X - 0.9) / 0.5) ** 2 + ((Y - 1.0) / 0.45) ** 2) / 2)
         + 0.8 * np.exp(-(((Z + 0.45) / 0.2) ** 2 + ((X - 1.7) / 0.4) ** 2 + ((Y - 0.8) / 0.5) ** 2) / 2))
    return B.astype(np.float32)


def test_marching_tetrahedra_matches_oracle(cuda):
    B = _field()
    iso = sm.Isosurface(B, BBOX, level=0.5, box_cells=3)
    ref = I.marching_tets(B, BBOX, 0.5)
    got = iso.tris[: iso.ntri, :, :3].double().cpu().numpy()
    assert iso.ntri == len(ref) > 100
    np.testing.assert_allclose(got, ref, atol=1e-5 * 2.5)


def test_signed_distance_matches_oracle(cuda):
    B = _field()
    iso = sm.Isosurface(B, BBOX, level=0.5, box_cells=3)
    tris = I.marching_tets(B, BBOX, 0.5)
    rng = np.random.default_rng(4)
    lo, hi = np.array(BBOX[0::2]), np.array(BBOX[1::2])
    # uniform, near-surface and outside-the-box points
    X = [lo + (hi - lo) * rng.uniform(size=(300, 3))]
    t = rng.integers(0, len(tris), 200)
    X.append(tris[t].mean(1) + 0.05 * rng.normal(size=(200, 3)))
    X.append(lo - 0.3 + (hi - lo + 0.6) * rng.uniform(size=(100, 3)))
    X = np.concatenate(X)
    X = X.astype(np.float32).astype(np.float64)
    d, g = iso.eval_with_gradient(X)
    dr, gr = I.signed_distance(X, tris, B, BBOX, 0.5)
    ext = 2.5
    np.testing.assert_allclose(d, dr, atol=1e-4 * ext)
    far = np.abs(dr) > 1e-4 * ext
    assert np.all(np.sign(d[far]) == np.sign(dr[far]))
    np.testing.assert_allclose(g[far], gr[far], atol=1e-3)


def test_batched_steps_filter_and_project(cuda):
    """dm_filter_cells_by_value keeps exactly the cells with d < -geps;
    dm_project_by_value moves exactly the points with d > 0, by -d grad"""
    rng = np.random.default_rng(2)
    n = 5000
    P = torch.from_numpy(np.column_stack([rng.normal(size=(n, 3)), np.zeros(n)]).astype(np.float32)).cuda()
    d = torch.from_numpy(rng.normal(size=n).astype(np.float32)).cuda()
    g = torch.from_numpy(rng.normal(size=(n, 4)).astype(np.float32)).cuda()
    before = P.clone()
    N.call("dm_project_by_value", 3, D.ptr(P), n, D.ptr(d), D.ptr(g), N.DM_NO_GRID, D.stream_ptr())
    exp = before.clone()
    pos = d > 0
    exp[pos, :3] = before[pos, :3] - d[pos, None] * g[pos, :3]
    # one rounding apart at most (the kernel may fuse the multiply-add)
    assert torch.equal(P[~pos], exp[~pos])
    torch.testing.assert_close(P, exp, rtol=2e-7, atol=1e-7)
    cells = torch.from_numpy(rng.integers(0, n, size=(7000, 4)).astype(np.int32)).cuda()
    cnt = torch.zeros(N.NCOUNTERS, dtype=torch.int64, device="cuda")
    cnt[N.CNT_CELLS] = 7000
    dc = torch.from_numpy(rng.normal(size=7000).astype(np.float32)).cuda()
    out = torch.empty_like(cells)
    N.call("dm_filter_cells_by_value", 3, D.ptr(cells), 7000, D.ptr(dc), 0.1, D.ptr(out),
           D.ptr(cnt), D.stream_ptr())
    k = int(cnt[N.CNT_KEPT].item())
    keep = (dc < -0.1).cpu().numpy()
    assert k == keep.sum()
    got = sorted(tuple(r) for r in out[:k].cpu().numpy())
    assert got == sorted(tuple(r) for r in cells.cpu().numpy()[keep])
