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


def _points_f64(p, dim):
    """caller points as a device float64 [n, dim] array (no narrowing: the
    reference's drop-ins compute in FP64 on FP64 inputs)"""
    return torch.from_numpy(np.ascontiguousarray(np.asarray(p)[:, :dim], dtype=np.float64)).to(D.device())


def simp_vol(p, t):
    """Signed volumes of the simplices (geometry/utils.py:175-201), FP64."""
    p = np.asarray(p)
    dim = p.shape[1]
    if len(t) == 0:
        return np.zeros(0)
    X = _points_f64(p, dim)
    T = _cells_dev(t)
    vol = D.empty((len(t),), torch.float64)
    N.call("dm_simplex_metrics_f64", dim, D.ptr(X), D.ptr(T), len(t), D.ptr(vol), None, D.stream_ptr())
    return vol.cpu().numpy()


def calc_re_ratios(vertices, entities, dim=2):
    """Radius-edge ratios, circumradius / shortest edge of each simplex
    (geometry/utils.py:17-54), on the GPU in FP64."""
    p = np.asarray(vertices)
    t = np.asarray(entities)
    if dim not in (2, 3):
        raise ValueError("Dimension invalid")
    if len(t) == 0:
        return np.zeros(0)
    X = torch.from_numpy(np.ascontiguousarray(p, dtype=np.float64)).to(D.device())
    T = _cells_dev(t)
    out = D.empty((len(t),), torch.float64)
    N.call("dm_radius_edge_ratios", dim, D.ptr(X), D.ptr(T), len(t), D.ptr(out), D.stream_ptr())
    return out.cpu().numpy()


def simp_qual(p, t):
    """Radius-ratio quality 2 r / R of the triangle of the first three vertices
    of each simplex (geometry/utils.py:252-274), FP64."""
    p = np.asarray(p)
    assert p.ndim == 2 and t.ndim == 2 and p.shape[1] + 1 == t.shape[1]
    dim = p.shape[1]
    if len(t) == 0:
        return np.zeros(0)
    X = _points_f64(p, dim)
    T = _cells_dev(t)
    q = D.empty((len(t),), torch.float64)
    N.call("dm_simplex_metrics_f64", dim, D.ptr(X), D.ptr(T), len(t), None, D.ptr(q), D.stream_ptr())
    return q.cpu().numpy()


def calc_dihedral_angles(p, t):
    """6 dihedral angles per tetrahedron, shape (6 T, 1)
    (geometry/cpp/fast_geometry.cpp:351-418), FP64."""
    X = _points_f64(p, 3)
    T = _cells_dev(t)
    out = D.empty((6 * len(t),), torch.float64)
    if len(t):
        N.call("dm_dihedral_angles_f64", D.ptr(X), D.ptr(T), len(t), D.ptr(out), D.stream_ptr())
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
    """Sorted unique (min, max) pairs (geometry/cpp/fast_geometry.cpp:30-77).
    Vertex indices must be non-negative (they index the mesh's vertices)."""
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.int32).reshape(-1, 2))
    m = e.shape[0]
    if m == 0:
        return np.zeros((0, 2), dtype=np.int32)
    if int(e.min()) < 0:
        raise ValueError("unique_edges: negative vertex index %d" % int(e.min()))
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


def get_boundary_entities(vertices, entities, dim=2):
    """Sorted indices of the cells touching a boundary vertex
    (geometry/utils.py:385-405)."""
    t = np.asarray(entities)
    flag = np.zeros(max(len(vertices), int(t.max()) + 1 if len(t) else 0), dtype=bool)
    flag[get_boundary_vertices(t, dim=dim)] = True
    return np.nonzero(flag[t].any(1))[0]


def delete_boundary_entities(vertices, entities, dim=2, min_qual=0.10, verbose=1):
    """Delete boundary cells of quality < min_qual, then fix_mesh with
    delete_unused (geometry/utils.py:440-469).  Vertices keep their float64
    coordinates; the selection runs on the GPU."""
    from ..generation.mesh_generator import _Engine

    vertices = np.asarray(vertices, dtype=float)
    t = np.ascontiguousarray(entities, dtype=np.int32)
    if len(t) == 0:
        return vertices, t
    eng = _Engine(dim, vertices, 0, grid=False)
    eng.kept[: len(t)] = torch.from_numpy(t).to(eng.P.device)
    eng.counters[N.CNT_KEPT] = len(t)
    delete = eng.boundary_delete_mask(min_qual).cpu().numpy()
    if verbose:
        print("Deleting " + str(int(delete.sum())) + " poor quality boundary entities...", flush=True)
    vertices, entities, _ = fix_mesh(vertices, t[~delete], delete_unused=True, dim=dim)
    return vertices, entities


def get_edges(entities, dim=2):
    """Undirected edges of every cell, repeated (geometry/utils.py:277-296)."""
    t = np.asarray(entities)
    if dim == 2:
        return t[:, [[0, 1], [0, 2], [1, 2]]].reshape((len(t) * 3, 2))
    return t[:, [[0, 1], [1, 2], [2, 0], [0, 3], [1, 3], [2, 3]]].reshape((len(t) * 6, 2))


def get_centroids(vertices, entities, dim=2):
    """Cell centroids (geometry/utils.py:731-742)."""
    return np.asarray(vertices)[np.asarray(entities)].sum(1) / (dim + 1)


def vertex_to_entities(vertices, entities, dim=2):
    """Cells around each vertex as (vtoe, vtoe_pointer): vertex v touches
    vtoe[vtoe_pointer[v]:vtoe_pointer[v + 1]] (geometry/utils.py:97-130).
    Rows list their cells in ascending order; vertices without cells get
    empty rows."""
    t = np.asarray(entities)
    n = len(vertices)
    v = t.reshape(-1)
    order = np.argsort(v, kind="stable")
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(v, minlength=n), out=ptr[1:])
    return (order // t.shape[1]).astype(np.int64), ptr


def do_any_overlap(vertices, entities, dim=2):
    """Pairs (ie, ele) of cells sharing a vertex where the centroid of ie lies
    inside ele (geometry/utils.py:745-817), on the GPU with the reference's
    FP64 arithmetic.  A pair is listed once per shared vertex, as the
    reference's loop lists it; the order is by ie, vertex slot, ele."""
    p = np.ascontiguousarray(vertices, dtype=np.float64)
    t = np.asarray(entities)
    if dim not in (2, 3) or p.ndim != 2 or p.shape[1] != dim or t.shape[1:] != (dim + 1,):
        raise ValueError("vertices must be (n, dim) and entities (m, dim + 1)")
    if len(t) == 0:
        return []
    X = torch.from_numpy(p).to(D.device())
    T = _cells_dev(t)
    ws = N.c_sz(0)
    N.call("dm_overlap_workspace_size", dim, len(p), len(t), ws)
    w = D.workspace(ws.value)
    cap = max(1024, len(t) // 8)
    for _ in range(2):
        out = D.empty((cap, 2), torch.int32)
        k = N.c_i64(0)
        try:
            N.call(
                "dm_overlap_pairs", dim, D.ptr(X), len(p), D.ptr(T), len(t), D.ptr(out), cap, k,
                D.ptr(w), w.numel(), D.stream_ptr(),
            )
            break
        except N.NativeError as e:
            if e.code != N.DM_ERR_CAPACITY:
                raise
            cap = k.value
    pairs = out[: k.value].cpu().numpy()
    return [(int(a), int(b)) for a, b in pairs]


def is_manifold(vertices, entities, dim=2):
    """True when every boundary vertex has exactly two boundary edges
    (geometry/utils.py:634-654)."""
    bedges = get_boundary_edges(entities, dim=dim)
    if bedges.size != np.asarray(vertices)[np.unique(bedges), :].size:
        print("Mesh has a non-manifold boundary...", flush=True)
        return False
    return True


def get_winded_boundary_edges(entities):
    """Boundary edges of a 2D mesh ordered by walking the boundary from the
    first edge (geometry/utils.py:329-361)."""
    bedges = get_boundary_edges(entities)
    if len(bedges) == 0:
        return bedges
    # edges incident to each vertex, then a walk that always takes the
    # first unvisited edge at the current vertex
    flat = bedges.reshape(-1)
    order = np.argsort(flat, kind="stable")
    ptr = np.searchsorted(flat[order], np.arange(flat.max() + 2))
    visited = np.zeros(len(bedges), dtype=bool)
    ordering = [0]
    visited[0] = True
    v_next = bedges[0, 1]
    while True:
        rows = order[ptr[v_next]:ptr[v_next + 1]] // 2
        cand = [r for r in np.sort(rows) if not visited[r]]
        if not cand:
            break
        r = cand[0]
        ordering.append(r)
        visited[r] = True
        e = bedges[r]
        v_next = e[1] if e[0] == v_next else e[0]
    return bedges[ordering, :]


def linter(vertices, entities, dim=2, min_qual=0.10):
    """Delete the lower-quality cell of every overlapping pair, clean the
    mesh, and (2D) delete poor boundary cells (geometry/utils.py:820-872)."""
    print("Performing mesh linting...", flush=True)
    vertices = np.asarray(vertices, dtype=float)
    entities = np.asarray(entities)
    qual = simp_qual(vertices, entities)
    pairs = np.array(do_any_overlap(vertices, entities, dim=dim), dtype=np.int64).reshape(-1, 2)
    # the lower quality of each pair; a tie goes to the first of the pair
    delete = np.unique(np.where(qual[pairs[:, 1]] < qual[pairs[:, 0]], pairs[:, 1], pairs[:, 0]))
    print("Deleting " + str(len(delete)) + " overlapped entities", flush=True)
    entities = np.delete(entities, delete, axis=0)
    vertices, entities, _ = fix_mesh(vertices, entities, dim=dim, delete_unused=True)
    if dim == 2:
        vertices, entities = delete_boundary_entities(vertices, entities, min_qual=min_qual)
        _ = is_manifold(vertices, entities)
    qual = simp_qual(vertices, entities)
    print(
        "There are " + str(len(vertices)) + " vertices and " + str(len(entities))
        + " elements in the mesh",
        flush=True,
    )
    print("The minimum element quality is " + str(np.amin(qual)), flush=True)
    return vertices, entities


def cell_quality(vertices, entities):
    """Per-cell dim * inradius / circumradius and, for tetrahedra, the
    minimum sine of the dihedral angles normalised to the regular
    tetrahedron (the measures the reference's benchmark reports take from
    meshplex, benchmarks/helpers.py).  Returns (quality, min_sin or None)."""
    p = np.ascontiguousarray(vertices, dtype=np.float64)
    t = np.asarray(entities)
    dim = p.shape[1]
    if dim not in (2, 3) or t.shape[1:] != (dim + 1,):
        raise ValueError("vertices must be (n, 2|3) and entities (m, dim + 1)")
    q = D.empty((len(t),), torch.float64)
    s = D.empty((len(t),), torch.float64) if dim == 3 else None
    if len(t):
        X = torch.from_numpy(p).to(D.device())
        N.call("dm_cell_quality", dim, D.ptr(X), D.ptr(_cells_dev(t)), len(t), D.ptr(q),
               D.ptr(s) if s is not None else None, D.stream_ptr())
    return q.cpu().numpy(), (s.cpu().numpy() if s is not None else None)


def quality_stats(vertices, entities):
    """The statistics of the reference's benchmark reports
    (benchmarks/helpers.py:10-109): quality min/avg/max with a 40-bin
    histogram on [0, 1]; in 3D also the minimum dihedral angle per cell,
    arcsin(2 sqrt(2) / 3 * q_min_sin) in degrees, with min/mean/max/std and a
    72-bin histogram on [0, 180]."""
    q, s = cell_quality(vertices, entities)
    out = {
        "num_verts": len(vertices), "num_cells": len(entities),
        "min_quality": float(np.min(q)), "avg_quality": float(np.average(q)),
        "max_quality": float(np.max(q)),
        "quality_hist": np.histogram(q, bins=np.linspace(0.0, 1.0, num=41, endpoint=True)),
    }
    if s is not None:
        ang = 180 * np.arcsin(np.minimum(2 * np.sqrt(2) / 3 * s, 1.0)) / np.pi
        out.update(
            min_dihedral=float(np.min(ang)), avg_dihedral=float(np.mean(ang)),
            max_dihedral=float(np.max(ang)), std_dihedral=float(np.std(ang)),
            dihedral_hist=np.histogram(ang, bins=np.linspace(0.0, 180.0, num=73, endpoint=True)),
        )
    return out
