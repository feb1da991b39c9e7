"""The isosurface / MLP oracle (oracle/iso_np.py) against closed forms, on
the CPU: a linear field's level set is a plane, so marching tetrahedra must
reproduce it and the signed distance must equal the plane distance; the
float64 backward must match central finite differences of the forward."""
import numpy as np

from oracle import iso_np as I


def _plane_field(n=(6, 7, 5), bbox=(0.0, 1.0, -1.0, 2.0, 0.5, 1.5)):
    axes = [np.linspace(bbox[2 * k], bbox[2 * k + 1], n[k]) for k in range(3)]
    Z, X, Y = np.meshgrid(*axes, indexing="ij")
    nrm = np.array([0.3, -0.5, 0.8])
    nrm /= np.linalg.norm(nrm)
    B = (0.6 - (nrm[0] * Z + nrm[1] * X + nrm[2] * Y)).astype(np.float32)
    return B, bbox, nrm


def test_marching_tets_of_a_linear_field_is_the_plane():
    B, bbox, nrm = _plane_field()
    tris = I.marching_tets(B, bbox, 0.0)
    assert len(tris) > 10
    # every vertex on the plane nrm . x = 0.6 (up to the float32 field)
    assert np.abs(tris.reshape(-1, 3) @ nrm - 0.6).max() < 1e-6


def test_signed_distance_to_a_plane():
    B, bbox, nrm = _plane_field()
    tris = I.marching_tets(B, bbox, 0.0)
    rng = np.random.default_rng(0)
    lo, hi = np.array(bbox[0::2]), np.array(bbox[1::2])
    X = lo + (hi - lo) * rng.uniform(0.3, 0.7, size=(40, 3))
    d, g = I.signed_distance(X, tris, B, bbox, 0.0)
    # inside where B >= 0, i.e. nrm . x <= 0.6; the surface patch is large
    # enough that the nearest point is the foot of the perpendicular
    ref = X @ nrm - 0.6
    ok = np.abs(ref) < 0.15
    assert ok.sum() > 5
    np.testing.assert_allclose(d[ok], ref[ok], atol=1e-6)
    np.testing.assert_allclose(g[ok], np.tile(nrm, (ok.sum(), 1)), atol=1e-5)


def test_mlp_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    params = rng.normal(0, 0.2, size=57985)
    freq = rng.normal(0, 2.0, size=96)
    x = rng.uniform(-1, 1, size=(7, 3))
    t = rng.normal(size=7)
    g, _ = I.mlp_grad(params, x, t, freq, (0, 0, 0), 1.0)
    for idx in rng.choice(len(params), size=40, replace=False):
        e = np.zeros_like(params)
        e[idx] = 1e-6
        lp = I.mlp_grad(params + e, x, t, freq, (0, 0, 0), 1.0)[1]
        lm = I.mlp_grad(params - e, x, t, freq, (0, 0, 0), 1.0)[1]
        assert abs((lp - lm) / 2e-6 - g[idx]) <= 1e-5 * max(1.0, abs(g[idx]))


def test_bf16_rounding():
    a = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-9, -3.14159, 65504.0], dtype=np.float32)
    r = I.bf16(a)
    assert r[0] == 1.0
    # ties to even: 1 + 2^-8 is halfway between 1 and 1 + 2^-7 -> 1
    assert r[1] == 1.0
    assert r[2] == 1.0 + 2**-7
    assert abs(r[3] - (-3.140625)) < 1e-12
