"""Mesh size from a velocity grid, float64 numpy + the C limgrad restatement.

TEST INFRASTRUCTURE ONLY.  Restates get_sizing_function_from_segy
(sizing/mesh_size_function.py:34-239): water replacement, wavelength sizing,
[hmin, hmax] clamp, Courant bound, gradation limiting (FastHJ.cpp), domain
pad and the linear RegularGridInterpolator on float32 axis vectors.
"""
import ctypes

import numpy as np
from scipy.interpolate import RegularGridInterpolator

from . import build as _build

_lib = None


def _liboracle():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build_oracle_c())
        _lib.oracle_limgrad.restype = ctypes.c_int
        _lib.oracle_limgrad.argtypes = [
            ctypes.POINTER(ctypes.c_int), ctypes.c_double, ctypes.c_double, ctypes.c_int,
            ctypes.POINTER(ctypes.c_double),
        ]
    return _lib


def limgrad(dims, elen, dfdx, imax, ffun):
    """FastHJ.limgrad on a column-major flat array; returns a new array."""
    f = np.ascontiguousarray(np.asarray(ffun, dtype=np.float64).reshape(-1)).copy()
    d = (ctypes.c_int * 3)(*[int(x) for x in dims])
    _liboracle().oracle_limgrad(d, float(elen), float(dfdx), int(imax),
                                f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return f


def size_grid(vp, bbox, hmin=150.0, hmax=10000.0, wl=0, freq=2.0, grade=0.0, dt=0.0,
              cr_max=1.0, space_order=1, domain_pad=0.0, pad_style="edge", units="m-s",
              vp_water=1500.0):
    vp = np.array(vp, dtype=np.float64)
    if units == "km-s":
        vp *= 1000.0
    elif units == "ft-s":
        vp *= 0.30
    pos = np.where(vp < 1e-3)
    if len(pos) > 0 and any(pos[0]):
        vp[pos] = vp_water
    dim = vp.ndim
    cell = np.full(vp.shape, hmin, dtype=float)
    if wl > 0:
        cell = np.minimum(vp / (freq * wl), 99999)
    cell[cell < hmin] = hmin
    cell[cell > hmax] = hmax
    if cr_max != 0.0 and dt != 0.0 and space_order != 0.0:
        cr_old = (vp * dt) / (dim * cell)
        crm = cr_max / (dim * space_order)
        dxn = (vp * dt) / (dim * crm)
        cell = np.where(cr_old > crm, dxn, cell)
    if grade != 0.0:
        sz = cell.shape if dim == 3 else (cell.shape[0], cell.shape[1], 1)
        elen = (bbox[1] - bbox[0]) / vp.shape[0]
        flat = limgrad(sz, elen, grade, 10000, cell.flatten("F"))
        cell = np.reshape(flat, cell.shape, "F")
    if domain_pad > 0:
        d = [(bbox[2 * k + 1] - bbox[2 * k]) / vp.shape[k] for k in range(dim)]
        nn = [int(domain_pad / dk) for dk in d]
        if dim == 2:
            bbox = (bbox[0] - domain_pad, bbox[1], bbox[2] - domain_pad, bbox[3] + domain_pad)
            padding = ((nn[0], 0), (nn[1], nn[1]))
        else:
            bbox = (bbox[0] - domain_pad, bbox[1], bbox[2] - domain_pad, bbox[3] + domain_pad,
                    bbox[4] - domain_pad, bbox[5] + domain_pad)
            padding = ((nn[0], 0), (nn[1], nn[1]), (nn[2], nn[2]))
        mx = np.amax(cell)
        if pad_style == "edge":
            cell = np.pad(cell, padding, "edge")
        elif pad_style == "constant":
            cell = np.pad(cell, padding, "constant", constant_values=(mx, mx))
        elif pad_style == "linear_ramp":
            cell = np.pad(cell, padding, "linear_ramp", end_values=(mx, mx))
    return cell, bbox


def interpolant(cell, bbox):
    """RegularGridInterpolator on float32 linspace axes, linear, extrapolating
    (sizing/mesh_size_function.py:391-408, 514-523)"""
    axes = [np.linspace(bbox[2 * k], bbox[2 * k + 1], cell.shape[k], dtype=np.float32)
            for k in range(cell.ndim)]
    f = RegularGridInterpolator(tuple(axes), cell, bounds_error=False, fill_value=None)
    return lambda x: f(np.asarray(x))
