"""Initial point helpers (host, numpy) - generation/utils.py of the reference.

The lattice and the seeded decimation run once on the host so the initial
point set is bit-identical to the reference's (generation/utils.py:15-45,
generation/mesh_generator.py:808-852).
"""
import copy

import numpy as np


def _odd(r):
    return [i for i in range(r) if i % 2 != 0]


def create_staggered_grid(h0, dim, bbox):
    """Staggered lattice (generation/utils.py:15-25): odd rows of axis 0 are
    shifted by h0/2 along axis 1; in 3D odd rows of axis 1 shift axis 2."""
    points = np.mgrid[tuple(slice(mn, mx + h0, h0) for mn, mx in bbox)].astype(float)
    odds_rows = _odd(points[0].shape[0])
    odds_cols = _odd(points[1].shape[0])
    points[1][odds_rows] += h0 / 2
    if dim == 3:
        points[2][odds_cols] += h0 / 2
    return points.reshape(dim, -1).T


def make_init_points(bbox, rank, size, axis, h0, dim):
    """Slab of the staggered lattice owned by `rank` (generation/utils.py:28-45);
    with size == 1 this is create_staggered_grid on the whole box."""
    _bbox = copy.deepcopy(bbox)
    for i in range(dim):
        if i == axis:
            new_lims = np.linspace(_bbox[i, 0], _bbox[i, 1], size + 1)
            _bbox[i, :] = new_lims[rank : rank + 2]
            if rank != 0:
                prev = new_lims[rank - 1 : rank - 1 + 2]
                tmp = np.mgrid[slice(prev[0], prev[1] + h0, h0)]
                _bbox[i, 0] = tmp[-1] + h0
    return create_staggered_grid(h0, dim, _bbox)
