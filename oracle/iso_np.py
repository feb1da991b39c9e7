"""Isosurface SDF and Fourier-feature MLP in plain numpy (test
infrastructure: small grids and batches only).

The reference has no isosurface-derived SDF and no learned SDF (its domains
are analytic, geometry/signed_distance_functions.py), so these restate the
project's own definitions independently of its kernels:

* marching_tets: the zero set of the piecewise-linear interpolant of
  B - level over the Kuhn split of every cell (tetrahedra along the main
  diagonal, one per axis permutation), in the kernels' triangle order (row
  (i, j), cell k, tetrahedron, then the quad's two triangles).
* signed_distance: brute-force nearest triangle (closest point by the
  Voronoi-region tests of Ericson, "Real-Time Collision Detection", 2005,
  5.1.5) in float64; negative where the interpolant is >= level.
* mlp_*: the MLP's forward / backward in float64, and the forward with BF16
  rounding of weights and activations (the tensor-core inference's
  arithmetic up to accumulation order).
"""
import numpy as np

KUHN = [(0, 1, 3, 7), (0, 1, 5, 7), (0, 2, 3, 7), (0, 2, 6, 7), (0, 4, 5, 7), (0, 4, 6, 7)]


def _node_xyz(origin, h, i, j, k, q):
    return np.array([origin[0] + (i + (q & 1)) * h[0], origin[1] + (j + ((q >> 1) & 1)) * h[1],
                     origin[2] + (k + ((q >> 2) & 1)) * h[2]])


def marching_tets(B, bbox, level):
    B = np.asarray(B, dtype=np.float32)
    n = B.shape
    origin = np.array(bbox[0::2], dtype=np.float64)
    h = (np.array(bbox[1::2]) - origin) / (np.array(n) - 1)
    out = []
    for i in range(n[0] - 1):
        for j in range(n[1] - 1):
            for k in range(n[2] - 1):
                fv = [float(np.float32(B[i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1)])
                            - np.float32(level)) for q in range(8)]

                def edge(u, v):
                    if u > v:
                        u, v = v, u
                    t = fv[u] / (fv[u] - fv[v])
                    a = _node_xyz(origin, h, i, j, k, u)
                    b = _node_xyz(origin, h, i, j, k, v)
                    return a + t * (b - a)

                for tv in KUHN:
                    ins = [v for v in range(4) if fv[tv[v]] >= 0]
                    outs = [v for v in range(4) if fv[tv[v]] < 0]
                    if len(ins) in (1, 3):
                        lone = ins[0] if len(ins) == 1 else outs[0]
                        o = [v for v in range(4) if v != lone]
                        out.append([edge(tv[lone], tv[w]) for w in o])
                    elif len(ins) == 2:
                        ac = edge(tv[ins[0]], tv[outs[0]])
                        ad = edge(tv[ins[0]], tv[outs[1]])
                        bd = edge(tv[ins[1]], tv[outs[1]])
                        bc = edge(tv[ins[1]], tv[outs[0]])
                        out.append([ac, ad, bd])
                        out.append([ac, bd, bc])
    return np.array(out, dtype=np.float64).reshape(-1, 3, 3)


def closest_points(p, tris):
    """closest point of every triangle to the point p (float64, vectorised)"""
    a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = (ab * ap).sum(1), (ac * ap).sum(1)
    bp = p - b
    d3, d4 = (ab * bp).sum(1), (ac * bp).sum(1)
    cp = p - c
    d5, d6 = (ab * cp).sum(1), (ac * cp).sum(1)
    vc = d1 * d4 - d3 * d2
    vb = d5 * d2 - d1 * d6
    va = d3 * d6 - d5 * d4
    out = np.empty_like(a)
    done = np.zeros(len(a), dtype=bool)

    def put(mask, val):
        m = mask & ~done
        out[m] = val[m]
        done[:] = done | m

    with np.errstate(divide="ignore", invalid="ignore"):
        put((d1 <= 0) & (d2 <= 0), a)
        put((d3 >= 0) & (d4 <= d3), b)
        put((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + (d1 / (d1 - d3))[:, None] * ab)
        put((d6 >= 0) & (d5 <= d6), c)
        put((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + (d2 / (d2 - d6))[:, None] * ac)
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6))
        put((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0), b + w[:, None] * (c - b))
        den = va + vb + vc
        put(den > 0, a + (vb / den)[:, None] * ab + (vc / den)[:, None] * ac)
    # degenerate triangles: nearest of the edges
    for t in np.nonzero(~done)[0]:
        best = None
        for u, v in ((a[t], b[t]), (b[t], c[t]), (a[t], c[t])):
            e = v - u
            l2 = e @ e
            s = 0.0 if l2 == 0 else min(max((p - u) @ e / l2, 0.0), 1.0)
            q = u + s * e
            if best is None or (p - q) @ (p - q) < (p - best) @ (p - best):
                best = q
        out[t] = best
    return out


def field_value(x, B, bbox, level):
    """the piecewise-linear (Kuhn) interpolant of B - level at x; -1 outside
    the node box"""
    B = np.asarray(B, dtype=np.float64)
    n = np.array(B.shape)
    origin = np.array(bbox[0::2], dtype=np.float64)
    h = (np.array(bbox[1::2]) - origin) / (n - 1)
    t = (np.asarray(x, dtype=np.float64) - origin) / h
    if np.any(t < 0) or np.any(t > n - 1):
        return -1.0
    c = np.minimum(np.floor(t).astype(int), n - 2)
    u = t - c
    order = sorted(range(3), key=lambda a: -u[a])
    q1 = 1 << order[0]
    q2 = q1 | (1 << order[1])

    def val(q):
        return B[c[0] + (q & 1), c[1] + ((q >> 1) & 1), c[2] + ((q >> 2) & 1)] - level

    f0, f1, f2, f3 = val(0), val(q1), val(q2), val(7)
    return f0 + u[order[0]] * (f1 - f0) + u[order[1]] * (f2 - f1) + u[order[2]] * (f3 - f2)


def signed_distance(X, tris, B, bbox, level):
    """signed distance and unit gradient at every row of X"""
    X = np.asarray(X, dtype=np.float64)
    d = np.empty(len(X))
    g = np.empty((len(X), 3))
    for r, p in enumerate(X):
        cp = closest_points(p, tris)
        dist2 = ((p - cp) ** 2).sum(1)
        t = int(np.argmin(dist2))
        dist = np.sqrt(dist2[t])
        s = -1.0 if field_value(p, B, bbox, level) >= 0 else 1.0
        d[r] = s * dist
        g[r] = s * (p - cp[t]) / dist if dist > 0 else 0.0
    return d, g


# ---------------------------------------------------------------------------
# the MLP
OFF_W = [0, 8320, 24832, 41344]
KDIM = [64, 128, 128, 128]
OFF_W5, OFF_B5 = 57856, 57984


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    Ws = [p[OFF_W[l]:OFF_W[l] + 128 * KDIM[l]].reshape(128, KDIM[l]) for l in range(4)]
    bs = [p[OFF_W[l] + 128 * KDIM[l]:OFF_W[l] + 128 * KDIM[l] + 128] for l in range(4)]
    return Ws, bs, p[OFF_W5:OFF_W5 + 128], p[OFF_B5]


def features(x, freq, center, inv_scale):
    """sin / cos of 2 pi (F x_n), with x_n and F x_n rounded to float32 at
    every operation as the kernels compute them"""
    x = np.asarray(x, dtype=np.float32)[:, :3]
    xn = (x - np.asarray(center, dtype=np.float32)) * np.float32(inv_scale)
    F = np.asarray(freq, dtype=np.float32).reshape(32, 3)
    t = F[None, :, 0] * xn[:, 0:1]
    t = t + F[None, :, 1] * xn[:, 1:2]
    t = t + F[None, :, 2] * xn[:, 2:3]
    t = (t - np.rint(t)).astype(np.float64)
    return np.concatenate([np.sin(2 * np.pi * t), np.cos(2 * np.pi * t)], 1)


def mlp_forward(params, x, freq, center, inv_scale):
    Ws, bs, w5, b5 = unpack(params)
    a = features(x, freq, center, inv_scale)
    zs, hs = [], [a]
    for l in range(4):
        z = a @ Ws[l].T + bs[l]
        a = np.maximum(z, 0)
        zs.append(z)
        hs.append(a)
    return a @ w5 + b5, zs, hs


def mlp_grad(params, x, target, freq, center, inv_scale, weight=None):
    """d loss / d params, loss = sum w (y - t)^2 / B (float64)"""
    B = len(x)
    w = np.ones(B) if weight is None else np.asarray(weight, dtype=np.float64)
    y, zs, hs = mlp_forward(params, x, freq, center, inv_scale)
    Ws, bs, w5, b5 = unpack(params)
    dy = 2 * w * (y - target) / B
    g = np.zeros(len(params))
    g[OFF_W5:OFF_W5 + 128] = hs[4].T @ dy
    g[OFF_B5] = dy.sum()
    dz = np.outer(dy, w5) * (zs[3] > 0)
    for l in range(3, -1, -1):
        g[OFF_W[l]:OFF_W[l] + 128 * KDIM[l]] = (dz.T @ hs[l]).ravel()
        g[OFF_W[l] + 128 * KDIM[l]:OFF_W[l] + 128 * KDIM[l] + 128] = dz.sum(0)
        if l:
            dz = (dz @ Ws[l]) * (zs[l - 1] > 0)
    return g, float((w * (y - target) ** 2).sum() / B)


def bf16(a):
    """round to the nearest BF16 (ties to even), as float64"""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def mlp_forward_bf16(params, x, freq, center, inv_scale):
    """the forward with BF16 weights (W1..W4) and BF16 layer inputs; sums,
    biases and the output layer in float64"""
    Ws, bs, w5, b5 = unpack(params)
    a = bf16(features(x, freq, center, inv_scale))
    for l in range(4):
        z = a @ bf16(Ws[l]).T + bs[l]
        a = np.maximum(z, 0)
        if l < 3:
            a = bf16(a)
    return a @ w5 + b5

