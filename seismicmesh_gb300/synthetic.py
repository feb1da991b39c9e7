"""Seeded synthetic velocity models with the shapes of the benchmark
workloads (no field data is read or reproduced).

layered_model_2d: float32 (nz=1911, nx=5395), dz = 6.25 m, dx = 12.5 m,
    bbox (z0, z1, x0, x1) = (-11943.75, 0, 0, 67437.5): 8 horizontal layers
    with velocities linearly spaced 1500 -> 4500 m/s, N(0, 50) noise
    (numpy default_rng(seed)), and an ellipse of 4500 m/s centred at depth
    6000 m, x = 30000 m, semi-axes 2000 m (depth) x 8000 m (x).

batch_domains: n independent domains (problem i seeded by
    numpy default_rng(seed + i)), the first half 2D and the rest 3D, each the
    union of 1-4 random disks / rectangles (balls / randomly rotated cubes)
    with radii or half-widths U(0.1, 1) minus 1-4 smaller ones (scaled by
    0.4), and a constant edge length
    chosen so the vertex counts spread log-uniformly over [2e3, 2e5]
    (estimated from the initial lattice's count, refined once).

salt_model_3d: float32 (nz=210, nx=676, ny=676) on bbox (-4200, 0, 0, 13520,
    0, 13520) (20 m nominal spacing; nodes at linspace over the box): 8
    layers 1500 -> 4000 m/s by depth, and a salt body at 4482 m/s where the
    field B = sum_k a_k exp(-|(x - c_k) / s_k|^2 / 2) (8 seeded Gaussian
    bumps, each truncated at 4 s_k) is >= 0.5.  B is returned too: its 0.5
    level set is the salt surface.
"""
import numpy as np

__all__ = ["layered_model_2d", "salt_model_3d", "salt_bumps", "batch_domains"]


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


def _random_domain(rng, dim, rotate_cubes=True):
    from . import geometry as G

    k = int(rng.integers(2, 9))
    n_add = max(1, (k + 1) // 2)

    def prim(scale):
        c = rng.uniform(-1.0, 1.0, dim)
        if rng.uniform() < 0.5:
            r = scale * rng.uniform(0.1, 1.0)
            return (G.Disk if dim == 2 else G.Ball)(list(c), r)
        hw = scale * rng.uniform(0.1, 1.0, dim)
        box = tuple(v for j in range(dim) for v in (c[j] - hw[j], c[j] + hw[j]))
        if dim == 2 or not rotate_cubes:
            return (G.Rectangle if dim == 2 else G.Cube)(box)
        # a randomly oriented cube: an axis-aligned cavity wall would be a
        # whole lattice plane of the initial points (see the design notes)
        return G.Cube(box, rotate=list(rng.uniform(0.0, 2 * np.pi, 3)))

    adds = [prim(1.0) for _ in range(n_add)]
    body = adds[0] if n_add == 1 else G.Union(adds)
    subs = [prim(0.4) for _ in range(k - n_add)]
    return body if not subs else G.Difference([body] + subs)


def _lattice_count(domain, h, dim):
    from .generation import utils as mutils

    bbox = np.array(domain.bbox).reshape(-1, 2)
    p = mutils.create_staggered_grid(h, dim, bbox)
    return int(np.count_nonzero(domain.eval(p) < 0.1 * h))


def batch_domains(n=256, seed=0, lo=2e3, hi=2e5, rotate_cubes=True):
    out = []
    for i in range(n):
        rng = np.random.default_rng(seed + i)
        dim = 2 if i < n // 2 else 3
        target = 10 ** rng.uniform(np.log10(lo), np.log10(hi))
        for _ in range(20):  # a domain whose lattice holds points
            dom = _random_domain(rng, dim, rotate_cubes)
            bbox = np.array(dom.bbox).reshape(-1, 2)
            ext = (bbox[:, 1] - bbox[:, 0]).prod()
            h = (ext / target) ** (1.0 / dim)
            cnt = _lattice_count(dom, h, dim)
            if cnt > 0:
                break
        h *= (cnt / target) ** (1.0 / dim)
        out.append((dom, float(h)))
    return out
