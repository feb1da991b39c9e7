"""Domains bounded by a level set of a gridded field, with exact distances.

The reference's domains are analytic primitives and their CSG
(geometry/signed_distance_functions.py); a salt body in a velocity model has
no analytic form.  `Isosurface` is the body {B >= level} of a field B given
at the nodes of a regular grid: the surface is the zero set of the
piecewise-linear interpolant of B over the Kuhn split of each grid cell (6
tetrahedra along the cell's main diagonal), extracted by marching
tetrahedra on the GPU (dm_iso_count / dm_iso_emit), and `eval` returns the
exact signed distance to it (negative inside) by a nearest-triangle search
over a uniform grid of boxes grouped in coarse blocks: rings of blocks
around the query, descending only into blocks that hold triangles and may
hold a nearer one (dm_iso_eval).
"""
import numpy as np
import torch

from .. import _device as D
from .. import _native as N

__all__ = ["Isosurface"]


class Isosurface:
    """Body {B >= level} of the node field B[n0, n1, n2] on the box
    bbox = (lo0, hi0, lo1, hi1, lo2, hi2) (node (i, j, k) at lo + (i, j, k) h
    with h = (hi - lo) / (n - 1)), with exact signed distances.

    box_cells: edge of the search boxes in grid cells; block: edge of the
    coarse blocks in boxes."""

    def __init__(self, field, bbox, level=0.5, box_cells=4, block=4):
        if isinstance(field, torch.Tensor):
            f = field.to(device=D.device(), dtype=torch.float32).contiguous()
        else:
            f = torch.from_numpy(np.ascontiguousarray(field, dtype=np.float32)).to(D.device())
        if f.dim() != 3 or min(f.shape) < 2:
            raise ValueError("field must be a 3D grid with at least 2 nodes per axis")
        bbox = tuple(float(b) for b in bbox)
        if len(bbox) != 6:
            raise ValueError("bbox must be (lo0, hi0, lo1, hi1, lo2, hi2)")
        self.dim = 3
        self.bbox = bbox
        self.corners = None
        self.level = float(level)
        self.field = f
        n = f.shape
        iso = N.Iso()
        iso.field = f.data_ptr()
        iso.level = self.level
        for k in range(3):
            iso.n[k] = n[k]
            iso.origin[k] = bbox[2 * k]
            iso.h[k] = (bbox[2 * k + 1] - bbox[2 * k]) / (n[k] - 1)
        nrow = (n[0] - 1) * (n[1] - 1)
        rowstart = D.empty((2 * nrow + 1,), torch.int32)
        nb = nrow // 1024 + 2
        tmp = D.empty((2 * (nb + 1) + nb // 1024 + 32,), torch.int32)
        ntri = N.c_i64(0)
        N.call("dm_iso_count", iso, D.ptr(rowstart), D.ptr(tmp), ntri, D.stream_ptr())
        self.ntri = int(ntri.value)
        self.tris = D.empty((max(self.ntri, 1), 3, 4), torch.float32)
        N.call("dm_iso_emit", iso, D.ptr(rowstart), D.ptr(self.tris), D.stream_ptr())
        iso.tris = self.tris.data_ptr()
        iso.ntri = self.ntri
        nbk = 1
        for k in range(3):
            iso.nb[k] = max(1, -(-(n[k] - 1) // box_cells))
            iso.bsize[k] = box_cells * iso.h[k]
            nbk *= iso.nb[k]
        iso.cf = block
        ncb = 1
        for k in range(3):
            iso.ncb[k] = -(-iso.nb[k] // block)
            ncb *= iso.ncb[k]
        self.bstart = D.empty((nbk + 1,), torch.int32)
        self.btri = D.empty((max(self.ntri, 1),), torch.int32)
        self.bring = D.empty((nbk,), torch.int32)
        self.coarse = D.empty((2 * ncb,), torch.int32)
        ws = N.c_sz(0)
        N.call("dm_iso_bucket_workspace_size", self.ntri, nbk, ws)
        w = D.workspace(ws.value)
        N.call("dm_iso_bucket", iso, D.ptr(self.bstart), D.ptr(self.btri), D.ptr(self.bring),
               D.ptr(self.coarse), D.ptr(w), w.numel(), D.stream_ptr())
        self.struct = iso

    def batched_eval(self, pts, stride, n, d, grad=None, mode=None, idx=None, count=None):
        """exact signed distances of the device points pts (float[n][stride])
        into d (and unit gradients into grad float[n][4]); with idx/count
        only the listed points (count on the device, n an upper bound)"""
        N.call("dm_iso_eval", self.struct, D.ptr(pts), stride, n, D.ptr(idx), D.ptr(count),
               D.ptr(d), D.ptr(grad), D.stream_ptr())

    def eval_with_gradient(self, x):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(-1, 3))
        n = len(x)
        P = torch.from_numpy(x).to(D.device())
        d = D.empty((max(n, 1),), torch.float32)
        g = D.empty((max(n, 1), 4), torch.float32)
        if n:
            self.batched_eval(P, 3, n, d, g)
        return d[:n].double().cpu().numpy(), g[:n, :3].double().cpu().numpy()

    def eval(self, x):
        """signed distance of host points x[m, 3] (float64 out)"""
        return self.eval_with_gradient(x)[0]
