"""Mesh utilities backed by libdmgb.so kernels.

Counterparts of geometry/utils.py and the geometry entry points of
geometry/cpp/fast_geometry.cpp in the reference.  Inputs and outputs are
numpy arrays like the reference's; the arithmetic runs on the GPU.
"""
import numpy as np
import torch

from .. import _device as D
from .. import _native as N


def _cells_dev(t):
    return torch.from_numpy(np.ascontiguousarray(t, dtype=np.int32)).to(D.device())


def _counter_block(n_cells, index=N.CNT_KEPT):
    c = D.zeros((N.NCOUNTERS,), torch.int64)
    c[index] = int(n_cells)
    return c


def simp_vol(p, t):
    """Signed volumes of the simplices (geometry/utils.py:175-201)."""
    p = np.asarray(p)
    dim = p.shape[1]
    if len(t) == 0:
        return np.zeros(0)
    P = D.to_points(p, dim)
    T = _cells_dev(t)
    vol = D.empty((len(t),), torch.float64)
    N.call("dm_simplex_metrics", dim, D.ptr(P), D.ptr(T), len(t), D.ptr(vol), None, D.stream_ptr())
    return vol.cpu().numpy()


def simp_qual(p, t):
    """Radius-ratio quality 2 r / R of the triangle of the first three vertices
    of each simplex (geometry/utils.py:252-274)."""
    p = np.asarray(p)
    assert p.ndim == 2 and t.ndim == 2 and p.shape[1] + 1 == t.shape[1]
    dim = p.shape[1]
    if len(t) == 0:
        return np.zeros(0)
    P = D.to_points(p, dim)
    T = _cells_dev(t)
    q = D.empty((len(t),), torch.float64)
    N.call("dm_simplex_metrics", dim, D.ptr(P), D.ptr(T), len(t), None, D.ptr(q), D.stream_ptr())
    return q.cpu().numpy()


def calc_dihedral_angles(p, t):
    """6 dihedral angles per tetrahedron, shape (6 T, 1)
    (geometry/cpp/fast_geometry.cpp:351-418)."""
    P = D.to_points(np.asarray(p), 3)
    T = _cells_dev(t)
    out = D.empty((6 * len(t),), torch.float64)
    if len(t):
        N.call("dm_dihedral_angles", D.ptr(P), D.ptr(T), len(t), D.ptr(out), D.stream_ptr())
    return out.cpu().numpy().reshape(-1, 1)


def calc_circumsphere_grad(p0, p1, p2, p3):
    """Gradient of the squared circumradius w.r.t. p0
    (geometry/cpp/fast_geometry.cpp:580-666)."""
    dev = D.device()
    arrs = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3)).to(dev)
            for a in (p0, p1, p2, p3)]
    m = arrs[0].shape[0]
    g = D.empty((m, 3), torch.float64)
    if m:
        N.call("dm_circumsphere_grad", *[D.ptr(a) for a in arrs], m, D.ptr(g), D.stream_ptr())
    return g.cpu().numpy()


def unique_edges(edges):
    """Sorted unique (min, max) pairs (geometry/cpp/fast_geometry.cpp:30-77)."""
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.int32).reshape(-1, 2))
    m = e.shape[0]
    if m == 0:
        return np.zeros((0, 2), dtype=np.int32)
    n = int(e.max()) + 1
    E = torch.from_numpy(e).to(D.device())
    out = D.empty((m, 2), torch.int32)
    ws = N.c_sz(0)
    N.call("dm_unique_edges_workspace_size", n, m, ws)
    w = D.workspace(ws.value)
    nout = N.c_i64(0)
    N.call("dm_unique_edges", D.ptr(E), m, n, D.ptr(out), nout, D.ptr(w), w.numel(), D.stream_ptr())
    return out[: nout.value].cpu().numpy()


def _boundary(t, dim, faces=False):
    t = np.asarray(t)
    n = int(t.max()) + 1 if len(t) else 0
    T = _cells_dev(t)
    cnt = _counter_block(len(t))
    ws = N.c_sz(0)
    N.call("dm_boundary_workspace_size", dim, n, len(t), ws)
    w = D.workspace(ws.value)
    flags = D.empty((max(n, 1),), torch.int32)
    cap = len(t) * (dim + 1)
    out = D.empty((max(cap, 1), dim), torch.int32) if faces else None
    N.call(
        "dm_boundary", dim, n, D.ptr(T), len(t), N.CNT_KEPT, D.ptr(flags), D.ptr(out),
        cap, D.ptr(cnt), D.ptr(w), w.numel(), D.stream_ptr(),
    )
    if faces:
        nf = int(cnt[N.CNT_AUX].item())
        f = out[:nf].cpu().numpy()
        # canonical order (the reference returns facets sorted by np.unique)
        order = np.lexsort(f.T[::-1])
        return f[order]
    return np.nonzero(flags[:n].cpu().numpy())[0]


def get_boundary_edges(entities, dim=2):
    """Edges that occur once (geometry/utils.py:310-326)."""
    return _boundary(entities, 2, faces=True)


def get_boundary_facets(entities):
    """Triangles that occur once (geometry/utils.py:421-437)."""
    if entities.shape[1] < 4:
        raise ValueError("Only works for triangles")
    return _boundary(entities, 3, faces=True)


def get_boundary_vertices(entities, dim=2):
    """Sorted indices of boundary vertices (geometry/utils.py:364-382)."""
    if dim not in (2, 3):
        raise ValueError("Dimension not supported.")
    return _boundary(entities, dim)


def _laplacian_device(eng):
    """Dirichlet Laplacian smoothing of a 2D engine state in place."""
    nk = int(eng.counters[N.CNT_KEPT].item())
    if nk == 0:
        return
    eng.build_adjacency()
    bflag = D.zeros((eng.n,), torch.int32)
    bid = eng.boundary_vertices(N.CNT_KEPT).long()
    bflag[bid] = 1
    ws = N.c_sz(0)
    N.call("dm_laplacian_workspace_size", eng.n, ws)
    w = D.workspace(ws.value)
    iters = N.c_int(0)
    N.call(
        "dm_laplacian_smooth", D.ptr(eng.P), eng.n, D.ptr(eng.adj), eng.adj_cap,
        D.ptr(eng.deg), D.ptr(bflag), 100000, 1e-10, iters, D.ptr(w), w.numel(),
        D.stream_ptr(),
    )


def laplacian2_fixed_point(vertices, entities):
    """Solve the Dirichlet graph Laplacian once (geometry/utils.py:494-547)."""
    from ..generation.mesh_generator import _Engine

    vertices = np.asarray(vertices)
    if vertices.ndim != 2 or vertices.shape[1] != 2:
        raise NotImplementedError("Laplacian smoothing only works in 2D for now")
    eng = _Engine(2, vertices, 0, grid=False)
    t = np.ascontiguousarray(entities, dtype=np.int32)
    eng.kept[: len(t)] = torch.from_numpy(t).to(eng.P.device)
    eng.counters[N.CNT_KEPT] = len(t)
    _laplacian_device(eng)
    return D.from_points(eng.P, 2), entities


def fix_mesh(p, t, ptol=2e-13, dim=2, delete_unused=False, fix_orientation=True):
    """Remove duplicated/unused vertices and duplicated cells, orient cells
    positively (geometry/utils.py:204-249).  Returns (p, t, jx)."""
    p = np.asarray(p, dtype=float)
    t = np.asarray(t)
    snap = (p.max(0) - p.min(0)).max() * ptol
    _, ix, jx = np.unique(np.round(p / snap) * snap, axis=0, return_index=True, return_inverse=True)
    jx = jx.reshape(-1)
    p = p[ix]
    t = jx[t]
    t = np.sort(t, axis=1)
    t = np.unique(t, axis=0)
    if delete_unused:
        pix, _, jx = np.unique(t, return_index=True, return_inverse=True)
        t = np.reshape(jx, t.shape)
        p = p[pix, :]
    if fix_orientation and len(t):
        flip = simp_vol(p, t) < 0
        t[flip, :2] = t[flip, 1::-1]
    return p, t, jx


def delete_boundary_entities(vertices, entities, dim=2, min_qual=0.10, verbose=1):
    """Delete boundary cells of quality < min_qual (geometry/utils.py:440-469)."""
    from ..generation.mesh_generator import _Engine

    eng = _Engine(dim, np.asarray(vertices), 0, grid=False)
    t = np.ascontiguousarray(entities, dtype=np.int32)
    eng.kept[: len(t)] = torch.from_numpy(t).to(eng.P.device)
    eng.counters[N.CNT_KEPT] = len(t)
    eng.delete_boundary_entities(min_qual, verbose)
    return eng.result()
