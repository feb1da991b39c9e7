"""GPU Delaunay (dm_delaunay) against the oracle.

Generic inputs: identical to Qhull after canonical ordering.  Exactly
degenerate lattices: a valid triangulation of the convex hull whose cells
are positively oriented and whose circumspheres are empty under the
symbolic perturbation (checked with the host exact predicates)."""
import numpy as np
import pytest
import torch
from scipy.spatial import ConvexHull, cKDTree

from oracle import delaunay_check as dc
from seismicmesh_gb300 import _native as N
from seismicmesh_gb300.generation.mesh_generator import _Engine
from seismicmesh_gb300.generation.utils import create_staggered_grid

pytestmark = pytest.mark.gpu


def triangulate(p):
    eng = _Engine(p.shape[1], p, 0, grid=False)
    nc = eng.triangulate()
    return eng.cells[:nc].cpu().numpy(), eng.counters_host()


@pytest.mark.parametrize("dim,n", [(2, 10), (2, 300), (2, 20000), (3, 12), (3, 300), (3, 20000)])
def test_random_points_match_qhull(cuda, dim, n):
    rng = np.random.default_rng(dim * 1000 + n)
    p = rng.random((n, dim)).astype(np.float32).astype(np.float64)
    cells, c = triangulate(p)
    assert c[N.CNT_FLAGS] == 0
    dc.assert_same_triangulation(p, cells)


@pytest.mark.parametrize("dim", [2, 3])
def test_clustered_points_match_qhull(cuda, dim):
    """strongly non-uniform density (exercises the exhaustive level)"""
    rng = np.random.default_rng(11)
    a = rng.normal(0, 0.01, (3000, dim))
    b = rng.uniform(-1, 1, (2000, dim))
    p = np.vstack([a, b]).astype(np.float32).astype(np.float64)
    cells, c = triangulate(p)
    assert c[N.CNT_FLAGS] == 0
    dc.assert_same_triangulation(p, cells)


def _check_valid(p, cells, dim, max_checks=4000):
    L = N.lib()
    p32 = p.astype(np.float32)
    fp = lambda a: np.ascontiguousarray(a, np.float32).ctypes.data_as(N._FP)  # noqa: E731
    for c in cells:
        s = L.dm_orient3(*[fp(p32[i]) for i in c]) if dim == 3 else L.dm_orient2(*[fp(p32[i]) for i in c])
        assert s > 0
    d = p[cells[:, 1:]] - p[cells[:, :1]]
    vol = np.abs(np.linalg.det(d)).sum() / (6 if dim == 3 else 2)
    assert abs(vol - ConvexHull(p).volume) < 1e-9 * max(1.0, vol)
    tree = cKDTree(p)
    checked = 0
    for c in cells[:max_checks]:
        P = p[c]
        A = 2 * (P[1:] - P[0])
        b = (P[1:] ** 2).sum(1) - (P[0] ** 2).sum()
        cen = np.linalg.solve(A, b)
        r = np.linalg.norm(P[0] - cen)
        for j in tree.query_ball_point(cen, r * 1.001 + 1e-9):
            if j in c:
                continue
            checked += 1
            if dim == 3:
                s = L.dm_insphere_sos(*[fp(p32[i]) for i in c], fp(p32[j]))
            else:
                s = L.dm_incircle_sos(*[fp(p32[i]) for i in c], fp(p32[j]))
            assert s > 0, (c, j)
    return checked


@pytest.mark.parametrize("dim,h", [(2, 0.25), (2, 0.05), (3, 0.5), (3, 0.25)])
def test_degenerate_lattice_is_valid_perturbed_delaunay(cuda, dim, h):
    p = create_staggered_grid(h, dim, np.array([[-1.0, 1.0]] * dim)).astype(np.float32).astype(np.float64)
    cells, c = triangulate(p)
    assert c[N.CNT_FLAGS] == 0
    _check_valid(p, cells, dim)


def test_duplicate_points_are_merged_like_cgal(cuda):
    rng = np.random.default_rng(3)
    p = rng.random((500, 3)).astype(np.float32).astype(np.float64)
    q = np.vstack([p, p[:20]])
    eng = _Engine(3, q, 0, grid=False)
    nc = eng.triangulate()
    assert eng.n == 500
    dc.assert_same_triangulation(eng.P[:, :3].double().cpu().numpy(), eng.cells[:nc].cpu().numpy())


def _face_queries(P, faces, mode, grid=False):
    import ctypes

    import torch

    from seismicmesh_gb300 import _device as D
    from seismicmesh_gb300 import _native as N
    from seismicmesh_gb300.generation.mesh_generator import _Engine

    L = N.lib()
    f = L.dmdbg_face_query_mode
    f.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_size_t,
                  ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]
    eng = _Engine(3, P, 0, grid=grid)
    eng.triangulate()  # builds the grid in the workspace
    Fd = torch.from_numpy(np.ascontiguousarray(faces, dtype=np.int32)).to(D.device())
    out = torch.empty(len(faces), dtype=torch.int32, device=D.device())
    assert f(3, eng.P.data_ptr(), eng.n, eng.ws_dt.data_ptr(), eng.ws_dt.numel(), Fd.data_ptr(),
             len(faces), out.data_ptr(), None, mode) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy(), eng


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["lattice", "near_lattice", "rounded_lattice", "grid_near_lattice"])
def test_face_queries_match_exhaustive_half_space_scan(cuda, kind):
    """Region-bounded gift-wrap queries return the same point as a scan of
    the whole positive half-space, on faces of (near-)degenerate lattices
    where needle faces and huge circumspheres occur."""
    rng = np.random.default_rng(5)
    g = np.arange(-1.0, 1.0 + 1e-9, 0.1)
    X = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    X[:, 0] += 0.05 * (np.round(X[:, 1] / 0.1) % 2)  # staggered rows
    X = X[np.linalg.norm(X, axis=1) < 1.0]
    if kind == "near_lattice":
        X = X + 1e-6 * rng.standard_normal(X.shape)
    elif kind == "rounded_lattice":
        X = X * (1 + 1e-7 * rng.standard_normal(len(X)))[:, None]
    elif kind == "grid_near_lattice":
        from seismicmesh_gb300.generation.mesh_generator import position_grid_exponent, snap_to_grid

        X = X + 1e-6 * rng.standard_normal(X.shape)
        X = snap_to_grid(X, position_grid_exponent(X))
    grid = kind.startswith("grid")
    P = X.astype(np.float32).astype(np.float64)
    eng_cells = None
    from seismicmesh_gb300.generation.mesh_generator import _Engine

    e = _Engine(3, P, 0, grid=grid)
    nc = e.triangulate()
    eng_cells = e.cells[:nc].cpu().numpy()
    sel = eng_cells[rng.choice(len(eng_cells), min(len(eng_cells), 3000), replace=False)]
    faces = []
    for c in sel:
        for i in range(4):
            o = [c[j] for j in range(4) if j != i]
            for (u, v) in ((o[0], o[1]), (o[1], o[2]), (o[2], o[0]), (o[1], o[0]), (o[2], o[1]), (o[0], o[2])):
                faces.append((c[i], u, v))
    faces = np.array(faces)
    want, _ = _face_queries(P, faces, 1, grid)
    # mode 0: scans of every block; mode 2: hull scans through the hull
    # candidates that level 1 flagged
    for mode in (0, 2):
        got, _ = _face_queries(P, faces, mode, grid)
        bad = np.nonzero(got != want)[0]
        assert len(bad) == 0, (mode, len(bad), faces[bad[:5]].tolist(), got[bad[:5]].tolist(),
                               want[bad[:5]].tolist())
    assert (want < 0).sum() > 100  # hull faces are among the queries


@pytest.mark.gpu
@pytest.mark.parametrize("dim,n", [(2, 20000), (3, 20000)])
def test_grid_aligned_points_match_qhull(cuda, dim, n):
    """Points on a common power-of-two grid (as DistMesh keeps them) take the
    fixed-point path for every predicate; the triangulation is Qhull's."""
    from seismicmesh_gb300.generation.mesh_generator import _Engine, position_grid_exponent, snap_to_grid

    rng = np.random.default_rng(17 + dim)
    p = rng.uniform(-1, 1, (n, dim))
    p = snap_to_grid(p, position_grid_exponent(p))
    eng = _Engine(dim, p, 0, grid=True)
    assert np.array_equal(eng.P[:, :dim].cpu().numpy().astype(np.float64), p)
    nc = eng.triangulate()
    dc.assert_same_triangulation(p, eng.cells[:nc].cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["random", "hub"])
def test_adjacency_rows_match_unique_edges(cuda, case):
    """dm_adjacency rows are the sorted unique neighbours from the cells
    (_get_edges + unique_edges of the reference); a hub vertex with more
    neighbours than the row stride widens the rows instead of dropping
    neighbours."""
    rng = np.random.default_rng(23)
    if case == "random":
        p = rng.uniform(-1, 1, (5000, 3))
    else:
        # 80 neighbours: 156 star cells, within the star capacity (192 cells)
        s = rng.standard_normal((80, 3))
        p = np.vstack([[0.0, 0.0, 0.0], s / np.linalg.norm(s, axis=1)[:, None]])
    p = p.astype(np.float32).astype(np.float64)
    eng = _Engine(3, p, 0, grid=False)
    nc = eng.triangulate()
    eng.kept[:nc] = eng.cells[:nc]
    eng.counters[N.CNT_KEPT] = nc
    eng.build_adjacency()
    cells = eng.cells[:nc].cpu().numpy()
    e = np.concatenate([cells[:, [i, j]] for i in range(4) for j in range(i + 1, 4)])
    e = np.unique(np.sort(e, axis=1), axis=0)
    nbr = [[] for _ in range(len(p))]
    for a, b in e:
        nbr[a].append(b)
        nbr[b].append(a)
    deg = eng.deg.cpu().numpy()
    adj = eng.adj.cpu().numpy()
    for v in range(len(p)):
        assert deg[v] == len(nbr[v]), (v, deg[v], len(nbr[v]))
        assert np.array_equal(adj[v, : deg[v]], np.sort(nbr[v])), v
    assert int(eng.counters[N.CNT_EDGES].item()) == len(e)
    if case == "hub":
        assert deg[0] == 80 and eng.adj_cap >= 80


@pytest.mark.gpu
def test_device_predicates_match_host_exact_predicates(cuda):
    """The floating-point exact stages on the device (FP32 filter, FP64
    filter, expansion arithmetic, symbolic perturbation) give the host's
    signs on near-degenerate and exactly degenerate 5-point tuples."""
    import ctypes

    L = N.lib()
    f = L.dmdbg_predicates
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    rng = np.random.default_rng(29)
    pts = []
    # cospherical points (on a sphere up to float rounding), a jittered
    # lattice and an exact lattice with a non-representable offset
    s = rng.standard_normal((400, 3))
    pts.append(0.3 + 0.7 * s / np.linalg.norm(s, axis=1)[:, None])
    g = np.stack(np.meshgrid(*[np.arange(4) * 0.1] * 3, indexing="ij"), -1).reshape(-1, 3)
    pts.append(0.2 + g + 1e-7 * rng.standard_normal(g.shape))
    pts.append(1e-9 + g)
    P = np.concatenate(pts).astype(np.float32)
    n = len(P)
    lat0 = n - len(g)  # the exact lattice block: coplanar and cospherical tuples
    tup = np.concatenate([rng.integers(0, n, (3000, 5)), rng.integers(lat0, n, (3000, 5))]).astype(np.int32)
    tup = tup[np.array([len(set(t)) == 5 for t in tup])]
    P4 = np.zeros((n, 4), np.float32)
    P4[:, :3] = P
    Pd = torch.from_numpy(P4).cuda()
    Td = torch.from_numpy(tup).cuda()
    fp = N.fptr
    o_host = np.array([L.dm_orient3(*[fp(np.ascontiguousarray(P[i])) for i in t[:4]]) for t in tup])
    for kind in (0, 3, 4):
        out = torch.empty(len(tup), dtype=torch.int32, device="cuda")
        assert f(Pd.data_ptr(), Td.data_ptr(), len(tup), kind, out.data_ptr(), None) == 0
        np.testing.assert_array_equal(out.cpu().numpy(), o_host)
    nz = o_host != 0
    s_host = np.array([L.dm_insphere_sos(*[fp(np.ascontiguousarray(P[i])) for i in t]) for t in tup[nz]])
    out = torch.empty(int(nz.sum()), dtype=torch.int32, device="cuda")
    Tn = torch.from_numpy(np.ascontiguousarray(tup[nz])).cuda()
    assert f(Pd.data_ptr(), Tn.data_ptr(), int(nz.sum()), 1, out.data_ptr(), None) == 0
    np.testing.assert_array_equal(out.cpu().numpy(), s_host)
    assert (o_host == 0).sum() > 50  # exact degeneracies were exercised


@pytest.mark.gpu
@pytest.mark.parametrize("dim,m", [(3, 600), (2, 400)])
def test_very_large_star_is_completed(cuda, dim, m):
    """A vertex whose star outgrows the shared-memory star (192 link
    triangles) is finished by the level-3 kernel; the triangulation is Qhull's."""
    rng = np.random.default_rng(31 + dim)
    s = rng.standard_normal((m, dim))
    p = np.vstack([np.zeros(dim), s / np.linalg.norm(s, axis=1)[:, None]])
    p = p.astype(np.float32).astype(np.float64)
    eng = _Engine(dim, p, 0, grid=False)
    nc = eng.triangulate()
    cells = eng.cells[:nc].cpu().numpy()
    assert (cells == 0).any(1).sum() >= m
    dc.assert_same_triangulation(p, cells)
