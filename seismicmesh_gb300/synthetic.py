"""Seeded synthetic velocity models with the shapes of the benchmark
workloads (no field data is read or reproduced).

layered_model_2d: float32 (nz=1911, nx=5395), dz = 6.25 m, dx = 12.5 m,
    bbox (z0, z1, x0, x1) = (-11943.75, 0, 0, 67437.5): 8 horizontal layers
    with velocities linearly spaced 1500 -> 4500 m/s, N(0, 50) noise
    (numpy default_rng(seed)), and an ellipse of 4500 m/s centred at depth
    6000 m, x = 30000 m, semi-axes 2000 m (depth) x 8000 m (x).

salt_model_3d: float32 (nz=210, nx=676, ny=676) on bbox (-4200, 0, 0, 13520,
    0, 13520) (20 m nominal spacing; nodes at linspace over the box): 8
    layers 1500 -> 4000 m/s by depth, and a salt body at 4482 m/s where the
    field B = sum_k a_k exp(-|(x - c_k) / s_k|^2 / 2) (8 seeded Gaussian
    bumps, each truncated at 4 s_k) is >= 0.5.  B is returned too: its 0.5
    level set is the salt surface.
"""
import numpy as np

__all__ = ["layered_model_2d", "salt_model_3d", "salt_bumps"]


def layered_model_2d(seed=0):
    nz, nx = 1911, 5395
    dz, dx = 6.25, 12.5
    bbox = (-11943.75, 0.0, 0.0, 67437.5)
    depth = dz * np.arange(nz)
    layer = np.minimum((depth / (dz * nz) * 8).astype(int), 7)
    v_layer = np.linspace(1500.0, 4500.0, 8)
    vp = np.repeat(v_layer[layer][:, None], nx, axis=1)
    rng = np.random.default_rng(seed)
    vp = vp + rng.normal(0.0, 50.0, size=vp.shape)
    z = depth[:, None]
    x = dx * np.arange(nx)[None, :]
    ell = ((z - 6000.0) / 2000.0) ** 2 + ((x - 30000.0) / 8000.0) ** 2 <= 1.0
    vp[ell] = 4500.0
    return vp.astype(np.float32), bbox


def salt_bumps(seed=5):
    """the 8 bumps: centres (z, x, y), widths, amplitudes"""
    rng = np.random.default_rng(seed)
    K = 8
    c = np.stack([rng.uniform(-3300, -1000, K), rng.uniform(3000, 10500, K),
                  rng.uniform(3000, 10500, K)], 1)
    s = np.stack([rng.uniform(400, 800, K), rng.uniform(900, 1800, K),
                  rng.uniform(900, 1800, K)], 1)
    a = rng.uniform(0.7, 1.0, K)
    return c, s, a


def salt_model_3d(seed=5, shape=(210, 676, 676), bbox=(-4200.0, 0.0, 0.0, 13520.0, 0.0, 13520.0)):
    nz, nx, ny = shape
    axes = [np.linspace(bbox[2 * k], bbox[2 * k + 1], shape[k]) for k in range(3)]
    c, s, a = salt_bumps(seed)
    B = np.zeros(shape, dtype=np.float32)
    for k in range(len(a)):
        g, sl = [], []
        for ax in range(3):
            u = axes[ax]
            lo = np.searchsorted(u, c[k, ax] - 4 * s[k, ax])
            hi = np.searchsorted(u, c[k, ax] + 4 * s[k, ax], side="right")
            sl.append(slice(lo, hi))
            g.append(np.exp(-0.5 * ((u[lo:hi] - c[k, ax]) / s[k, ax]) ** 2).astype(np.float32))
        B[sl[0], sl[1], sl[2]] += (np.float32(a[k]) * g[0][:, None, None]
                                   * g[1][None, :, None] * g[2][None, None, :])
    depth = -axes[0]
    layer = np.minimum((depth / (bbox[1] - bbox[0]) * 8).astype(int), 7)
    v_layer = np.linspace(1500.0, 4000.0, 8).astype(np.float32)
    vp = np.broadcast_to(v_layer[layer][:, None, None], shape).copy()
    vp[B >= 0.5] = 4482.0
    return vp, B, tuple(float(b) for b in bbox)
