"""Signed distance functions in float64 numpy (test infrastructure).

Restates geometry/signed_distance_functions.py of the reference: the
inverse transforms of _manipulate (89-101), the primitives (429-623) and the
sharp/smooth set operations (307-426).  Each builder returns a callable
x[n, dim] -> d[n].
"""
import numpy as np


def _rot2(a):
    return np.array([[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]])


def _rot3(r):
    Rx = np.array([[1, 0, 0], [0, np.cos(r[0]), -np.sin(r[0])], [0, np.sin(r[0]), np.cos(r[0])]])
    Ry = np.array([[np.cos(r[1]), 0, np.sin(r[1])], [0, 1, 0], [-np.sin(r[1]), 0, np.cos(r[1])]])
    Rz = np.array([[np.cos(r[2]), -np.sin(r[2]), 0], [np.sin(r[2]), np.cos(r[2]), 0], [0, 0, 1]])
    return Rx, Ry, Rz


def transformed(f, dim, rotate=(0, 0, 0), stretch=None, translate=None):
    """compose f with the inverse transforms in _manipulate's order:
    translate back, Rx^-1, Ry^-1, Rz^-1 (non-zero angles only), stretch back"""
    mats = []
    if dim == 2:
        if rotate[0] != 0.0:
            mats.append(_rot2(rotate[0]).T)
    else:
        for k, R in enumerate(_rot3(rotate)):
            if rotate[k] != 0.0:
                mats.append(R.T)
    v = alpha = None
    if stretch is not None:
        v = np.asarray(stretch, float)
        alpha = np.sqrt(v @ v)
        v = v / alpha
    t = None if translate is None else np.asarray(translate, float)

    def g(x):
        x = np.asarray(x, float)
        if t is not None:
            x = x - t
        for M in mats:
            x = x @ M.T
        if v is not None:
            vx = np.outer(x @ v, v)
            x = vx / alpha + (x - vx)
        return f(x)

    return g


def disk(xc, yc, r, **kw):
    return transformed(lambda x: np.sqrt(((x - [xc, yc]) ** 2).sum(-1)) - r, 2, **kw)


def ball(xc, yc, zc, r, **kw):
    return transformed(lambda x: np.sqrt(((x - [xc, yc, zc]) ** 2).sum(-1)) - r, 3, **kw)


def rectangle(b, **kw):
    x1, x2, y1, y2 = b
    return transformed(
        lambda p: -np.minimum(np.minimum(np.minimum(-y1 + p[:, 1], y2 - p[:, 1]), -x1 + p[:, 0]), x2 - p[:, 0]),
        2, **kw)


def cube(b, **kw):
    x1, x2, y1, y2, z1, z2 = b

    def f(p):
        m = np.minimum(np.minimum(-z1 + p[:, 2], z2 - p[:, 2]), -y1 + p[:, 1])
        m = np.minimum(np.minimum(np.minimum(m, y2 - p[:, 1]), -x1 + p[:, 0]), x2 - p[:, 0])
        return -m

    return transformed(f, 3, **kw)


def torus(r1, r2, **kw):
    def f(x):
        q0 = np.sqrt(x[:, 0] ** 2 + x[:, 2] ** 2) - r1
        return np.sqrt(q0**2 + x[:, 1] ** 2) - r2

    return transformed(f, 3, **kw)


def prism(b, h, **kw):
    def f(x):
        q = np.abs(x)
        return np.maximum(q[:, 2] - h, np.maximum(q[:, 0] * 0.866025 + x[:, 1] * 0.5, -x[:, 1]) - b * 0.5)

    return transformed(f, 3, **kw)


def cylinder(h=1.0, r=0.5, **kw):
    hh = h / 2.0

    def f(x):
        d0 = np.sqrt(x[:, 0] ** 2 + x[:, 2] ** 2) - r
        d1 = np.abs(x[:, 1]) - hh
        return np.minimum(np.maximum(d0, d1), 0.0) + np.sqrt(np.maximum(d0, 0) ** 2 + np.maximum(d1, 0) ** 2)

    return transformed(f, 3, **kw)


def union(fs, k=0.0):
    def f(x):
        d = [g(x) for g in fs]
        if k == 0.0:
            return np.minimum.reduce(d)
        r = d[0]
        for e in d[1:]:
            h = np.maximum(k - np.abs(r - e), 0.0)
            r = np.minimum(r, e) - h * h * 0.25 / k
        return r

    return f


def intersection(fs, k=0.0):
    def f(x):
        d = [g(x) for g in fs]
        if k == 0.0:
            return np.maximum.reduce(d)
        r = d[0]
        for e in d[1:]:
            h = np.maximum(k - np.abs(r - e), 0.0)
            r = np.maximum(r, e) + h * h * 0.25 / k
        return r

    return f


def difference(fs, k=0.0):
    def f(x):
        d = [g(x) for g in fs]
        if k == 0.0:
            return np.maximum.reduce([d[0]] + [-e for e in d[1:]])
        r = d[-1]
        for e in d[-2::-1]:
            h = np.maximum(k - np.abs(-r - e), 0.0)
            r = np.maximum(-r, e) + h * h * 0.25 / k
        return r

    return f
