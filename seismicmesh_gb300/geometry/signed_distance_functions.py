"""Signed distance functions, evaluated on the GPU.

Same classes, constructor arguments and attributes (``dim``, ``bbox``,
``corners``, ``eval``) as geometry/signed_distance_functions.py of the
reference.  Each object compiles to a postfix *SDF program* (op records +
float parameters, see csrc/dm_sdf.cuh) that the device kernels interpret:
the Delaunay cell filter, the Newton projection and ``eval``.

Reference map:
  _manipulate / _build_stretch / _build_rotation / _build_translation  89-280
  Repeat 283-297, Union 307-344, Intersection 347-384, Difference 387-426,
  Disk 429-447, Ball 450-471, Rectangle 474-492, Cube 495-519,
  Torus 522-543, Prism 546-566, Cylinder 569-593, corners 74-78.
"""
import itertools
from functools import reduce

import numpy as np

from .. import _native as N

# op codes of csrc/dm_sdf.cuh
OP_DISK, OP_BALL, OP_RECT, OP_CUBE, OP_TORUS, OP_PRISM, OP_CYLINDER, OP_GRID = range(1, 9)
OP_UNION, OP_INTERSECTION, OP_DIFFERENCE = 20, 21, 22
XF_TRANSLATE, XF_RX, XF_RY, XF_RZ, XF_STRETCH, XF_REPEAT = 1, 2, 4, 8, 16, 32


def corners(bbox):
    """Get the corners of a box in N-dim (reference 74-78)."""
    mins = bbox[::2]
    maxs = bbox[1::2]
    return np.array(list(itertools.product(*zip(mins, maxs))))


def _gather_corners(domains):
    cs = [d.corners for d in domains if d.corners is not None]
    if len(cs) == 0:
        return None
    return np.concatenate(cs)


# ---------------------------------------------------------------------------
# rigid transforms (construction-time bookkeeping identical to the reference)
def _build_stretch(obj):
    if obj.v is not None:
        assert len(obj.v) == obj.dim, "Length of stretch vector does not equal dimension"
        obj.v = np.asarray(obj.v, dtype=float)
        obj.alpha = np.sqrt(np.dot(obj.v, obj.v))
        obj.v = obj.v / obj.alpha
        _c = corners(obj.bbox)
        vx = np.multiply.outer(np.dot(obj.v, _c.T), obj.v)
        tmp = (vx * obj.alpha + (_c - vx)).T
        obj.bbox = tuple(
            v for k in range(obj.dim) for v in (np.min(tmp[k]), np.max(tmp[k]))
        )
        obj.corners = corners(obj.bbox)
    return obj


def _build_rotation(obj):
    bbox_x = bbox_y = bbox_z = obj.bbox
    r = obj.rotation
    if obj.dim == 2:
        obj.R = np.array([[np.cos(r[0]), -np.sin(r[0])], [np.sin(r[0]), np.cos(r[0])]])
        obj.Rx_inv = obj.R.T
        if r[0] != 0.0:
            obj.corners = corners(obj.bbox)
            tmp = np.dot(obj.R, obj.corners.T).T
            obj.bbox = (np.min(tmp[:, 0]), np.max(tmp[:, 0]), np.min(tmp[:, 1]), np.max(tmp[:, 1]))
            obj.corners = corners(obj.bbox)
    elif obj.dim == 3:
        obj.Rx = np.array(
            [[1, 0, 0], [0, np.cos(r[0]), -np.sin(r[0])], [0, np.sin(r[0]), np.cos(r[0])]]
        )
        obj.Ry = np.array(
            [[np.cos(r[1]), 0, np.sin(r[1])], [0, 1, 0], [-np.sin(r[1]), 0, np.cos(r[1])]]
        )
        obj.Rz = np.array(
            [[np.cos(r[2]), -np.sin(r[2]), 0], [np.sin(r[2]), np.cos(r[2]), 0], [0, 0, 1]]
        )
        obj.Rx_inv, obj.Ry_inv, obj.Rz_inv = obj.Rx.T, obj.Ry.T, obj.Rz.T
        if reduce(lambda a, b: a or b, r):
            obj.corners = corners(obj.bbox)

            def rotated_box(R):
                obj.corners = corners(obj.bbox)
                t = np.dot(R, obj.corners.T).T
                return tuple(v for k in range(3) for v in (np.min(t[:, k]), np.max(t[:, k])))

            if r[0] != 0.0:
                bbox_x = rotated_box(obj.Rx)
            if r[1] != 0.0:
                bbox_y = rotated_box(obj.Ry)
            if r[2] != 0.0:
                bbox_z = rotated_box(obj.Rz)
            out = []
            for c, (i, j, k) in enumerate(zip(bbox_x, bbox_y, bbox_z)):
                out.append(min(i, j, k) if c % 2 == 0 else max(i, j, k))
            obj.bbox = tuple(out)
            obj.corners = corners(obj.bbox)
    return obj


def _build_translation(obj):
    v = obj.translation_vec
    if v is not None:
        assert len(v) == obj.dim, "Length of translation vector does not equal dimension"
        obj.bbox = tuple(b + v[k // 2] for k, b in enumerate(obj.bbox))
    return obj


def _configure_manipulations(obj):
    obj = _build_stretch(obj)
    obj = _build_rotation(obj)
    obj = _build_translation(obj)
    return obj


# ---------------------------------------------------------------------------
class _Program:
    """Host image of an SDF program: int32 op records and float32 params."""

    def __init__(self, dim):
        self.dim = dim
        self.ops = []
        self.params = []
        self.repeat = None  # period while a Repeat's domain is emitted

    def add(self, op, params, count=0, xf=0):
        off = len(self.params)
        self.params.extend(float(x) for x in params)
        self.ops.append((op, off, count, xf))

    def extend_params(self, values):
        off = len(self.params)
        self.params.extend(float(x) for x in values)
        return off


class _DeviceProgram:
    """Device copy of a program plus the ctypes struct pointing at it."""

    def __init__(self, prog):
        from .. import _device as D
        import torch

        dev = D.device()
        self.ops = torch.tensor(np.asarray(prog.ops, dtype=np.int32).reshape(-1), device=dev)
        params = np.asarray(prog.params if prog.params else [0.0], dtype=np.float32)
        self.params = torch.tensor(params, device=dev)
        self.struct = N.SdfProgram(
            self.ops.data_ptr(), self.params.data_ptr(), len(prog.ops), prog.dim
        )


class _SDFBase:
    """Common evaluation machinery of the geometry classes."""

    _device_prog = None

    def program(self):
        prog = _Program(self.dim)
        self._emit(prog)
        return prog

    def device_program(self):
        if self._device_prog is None:
            self._device_prog = _DeviceProgram(self.program())
        return self._device_prog

    def eval(self, x, grad=False):
        """Signed distance at the rows of x (numpy, shape (n, dim))."""
        from .. import _device as D
        import torch

        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(-1, self.dim))
        n = x.shape[0]
        dp = self.device_program()
        xd = torch.from_numpy(x).to(D.device())
        d = D.empty((n,), torch.float32)
        g = D.empty((n, self.dim), torch.float32) if grad else None
        N.call(
            "dm_sdf_eval", dp.struct, D.ptr(xd), n, self.dim, D.ptr(d), D.ptr(g), D.stream_ptr()
        )
        dn = d.double().cpu().numpy()
        if grad:
            return dn, g.double().cpu().numpy()
        return dn

    __call__ = eval

    def show(self, filename=None, samples=10000):
        raise NotImplementedError("plotting is not part of the GPU engine")


class _Primitive(_SDFBase):
    def _xform(self, prog):
        """transform flags + parameter tail in the order _manipulate applies them"""
        flags, tail = 0, []
        if self.translation_vec is not None:
            flags |= XF_TRANSLATE
            tail += list(np.asarray(self.translation_vec, dtype=float))
        rot = self.rotation
        if self.dim == 2:
            if rot[0] != 0.0:
                flags |= XF_RX
                tail += list(self.Rx_inv.reshape(-1))
        else:
            for k, (bit, name) in enumerate(((XF_RX, "Rx_inv"), (XF_RY, "Ry_inv"), (XF_RZ, "Rz_inv"))):
                if rot[k] != 0.0:
                    flags |= bit
                    tail += list(getattr(self, name).reshape(-1))
        if self.v is not None:
            flags |= XF_STRETCH
            tail += list(self.v) + [self.alpha]
        return flags, tail

    def _emit(self, prog):
        flags, tail = self._xform(prog)
        if prog.repeat is not None:  # inside a Repeat: its period comes first
            flags |= XF_REPEAT
            tail = list(prog.repeat) + tail
        prog.add(self._op, list(self._prim_params()) + tail, 0, flags)


class Disk(_Primitive):
    _op = OP_DISK

    def __init__(self, x0, r, rotate=[0, 0, 0], stretch=None, translate=None):
        self.dim = 2
        self.xc, self.yc, self.r = x0[0], x0[1], r
        self.bbox = (x0[0] - r, x0[0] + r, x0[1] - r, x0[1] + r)
        self.rotation = rotate
        self.v = stretch
        self.translation_vec = translate
        _configure_manipulations(self)
        self.corners = None

    def _prim_params(self):
        return (self.xc, self.yc, self.r)


class Ball(_Primitive):
    _op = OP_BALL

    def __init__(self, x0, r, rotate=[0, 0, 0], stretch=None, translate=None):
        if stretch is not None:
            assert len(stretch) == 3
        self.dim = 3
        self.xc, self.yc, self.zc, self.r = x0[0], x0[1], x0[2], r
        self.bbox = (x0[0] - r, x0[0] + r, x0[1] - r, x0[1] + r, x0[2] - r, x0[2] + r)
        self.rotation = rotate
        self.v = stretch
        self.translation_vec = translate
        _configure_manipulations(self)
        self.corners = None

    def _prim_params(self):
        return (self.xc, self.yc, self.zc, self.r)


class Rectangle(_Primitive):
    _op = OP_RECT

    def __init__(self, bbox, rotate=[0.0, 0.0, 0.0], stretch=None, translate=None):
        self.dim = 2
        self.corners = corners(bbox)
        self.bbox0 = bbox
        self.bbox = bbox
        self.rotation = rotate
        self.v = stretch
        self.translation_vec = translate
        _configure_manipulations(self)

    def _prim_params(self):
        return tuple(self.bbox0[:4])


class Cube(_Primitive):
    _op = OP_CUBE

    def __init__(self, bbox, rotate=[0, 0, 0], stretch=None, translate=None):
        self.dim = 3
        self.corners = corners(bbox)
        self.bbox0 = bbox
        self.bbox = bbox
        self.rotation = rotate
        self.v = stretch
        self.translation_vec = translate
        _configure_manipulations(self)

    def _prim_params(self):
        return tuple(self.bbox0[:6])


class Torus(_Primitive):
    _op = OP_TORUS

    def __init__(self, r1, r2, rotate=[0, 0, 0], stretch=None, translate=None):
        """A torus with outer radius `r1` and inner radius of `r2`"""
        assert r1 > 0.0 and r2 > 0.0
        z = 2 * max(r1, r2)
        self.dim = 3
        self.bbox = (-2 * z, 2 * z, -2 * z, 2 * z, -2 * z, 2 * z)
        self.t = (r1, r2)
        self.rotation = rotate
        self.v = stretch
        self.translation_vec = translate
        _configure_manipulations(self)
        self.corners = None

    def _prim_params(self):
        return self.t


class Prism(_Primitive):
    _op = OP_PRISM

    def __init__(self, b, h, rotate=[0, 0, 0], stretch=None, translate=None):
        self.bbox = (-b, +b, -b, +b, -h, +h)
        self.h = (b, h)
        self.dim = 3
        self.rotation = rotate
        self.v = stretch
        self.translation_vec = translate
        _configure_manipulations(self)
        self.corners = None

    def _prim_params(self):
        return self.h


class Cylinder(_Primitive):
    _op = OP_CYLINDER

    def __init__(self, h=1.0, r=0.5, rotate=[0, 0, 0], stretch=None, translate=None):
        assert h > 0.0 and r > 0.0
        h /= 2.0
        sz = max(h, r)
        self.dim = 3
        self.bbox = (-2 * sz, 2 * sz, -2 * sz, 2 * sz, -2 * sz, 2 * sz)
        self.h = (r, h)
        self.rotation = rotate
        self.v = stretch
        self.translation_vec = translate
        _configure_manipulations(self)
        self.corners = None

    def _prim_params(self):
        return self.h


class GridSDF(_SDFBase):
    """Signed distance sampled on a regular grid, linearly interpolated.

    ``values`` has shape (n0, n1[, n2]); axis k spans linspace(lo[k], hi[k]).
    Not in the reference (whose EAGE example meshes a Cube); used for
    isosurface-defined domains such as a salt body.
    """

    def __init__(self, values, bbox):
        values = np.asarray(values, dtype=np.float32)
        self.dim = values.ndim
        assert self.dim in (2, 3)
        self.values = values
        self.bbox = tuple(float(b) for b in bbox)
        self.corners = None

    def _emit(self, prog):
        if prog.repeat is not None:
            raise NotImplementedError("a gridded SDF inside Repeat is not supported")
        n = list(self.values.shape) + [1] * (3 - self.dim)
        lo = [self.bbox[2 * k] for k in range(self.dim)] + [0.0] * (3 - self.dim)
        hi = [self.bbox[2 * k + 1] for k in range(self.dim)] + [1.0] * (3 - self.dim)
        head = n + lo + hi
        base = len(prog.params)
        data_off = 10  # relative to the primitive's own parameter block
        prog.add(OP_GRID, head + [float(data_off)], 0, 0)
        prog.extend_params(self.values.reshape(-1))
        assert prog.ops[-1][1] == base


class _SetOp(_SDFBase):
    _op = None

    def __init__(self, domains, smoothness=0.0):
        geom_dim = [d.dim for d in domains]
        assert np.all(np.asarray(geom_dim) != 2) or np.all(np.asarray(geom_dim) != 3)
        self.dim = geom_dim[0]
        self.k = smoothness
        self.bbox = tuple(
            (min if c % 2 == 0 else max)(d.bbox[c] for d in domains) for c in range(2 * self.dim)
        )
        self.corners = _gather_corners(domains)
        self.domains = domains

    def _emit(self, prog):
        for d in self.domains:
            d._emit(prog)
        prog.add(self._op, [self.k], len(self.domains), 0)


class Union(_SetOp):
    _op = OP_UNION


class Intersection(_SetOp):
    _op = OP_INTERSECTION


class Difference(_SetOp):
    _op = OP_DIFFERENCE


class Repeat(_SDFBase):
    """Periodic repetition of a domain inside a Cube (reference 283-297):
    max(domain(mod(x + p/2, p) - p/2), Cube(bbox)(x)).  On the device the
    periodic map is a transform of every primitive of the repeated domain."""

    def __init__(self, bbox, domain, period):
        self.bbox = bbox
        self.domain = domain
        self.corners = None
        self.period = np.array(period)
        self.parent = Cube(bbox)
        self.dim = 3

    def _emit(self, prog):
        if prog.repeat is not None:
            raise NotImplementedError("nested Repeat is not supported")
        prog.repeat = [float(v) for v in np.broadcast_to(self.period, (3,))]
        try:
            self.domain._emit(prog)
        finally:
            prog.repeat = None
        self.parent._emit(prog)
        prog.add(OP_INTERSECTION, [0.0], 2, 0)


def _ddisk(p, xc, yc, r):
    return Disk([xc, yc], r).eval(p)


def dball(p, xc, yc, zc, r):
    return Ball([xc, yc, zc], r).eval(p)


def drectangle(p, x1, x2, y1, y2):
    return Rectangle((x1, x2, y1, y2)).eval(p)


def dblock(p, x1, x2, y1, y2, z1, z2):
    return Cube((x1, x2, y1, y2, z1, z2)).eval(p)
