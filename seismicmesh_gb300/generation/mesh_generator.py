"""DistMesh driver on the GPU: generate_mesh and sliver_removal.

Drop-in for generation/mesh_generator.py of the reference (same arguments,
keyword whitelist, defaults, messages and return types).  The points live on
the device as FP32 (float[n][4] in 3D, float[n][2] in 2D) for the whole
loop; each iteration is the kernel sequence

  dm_delaunay -> dm_filter_cells -> dm_adjacency -> dm_bar_sums ->
  dm_update_points (forces, update, Newton projection)

replacing, respectively, the CGAL rebuild + get_topology (465-469),
_remove_triangles_outside (734-738), _get_edges/unique_edges (680-688),
the L0 normalisation of _compute_forces (691-712) and the force scatter,
position update and _project_points_back_newton (497-506, 762-784).
Vertex indices never change (CGAL renumbers; the reference therefore
recomputes ifix by nearest search at 471-475, which here is the identity).
"""
import math
import time
import warnings

import numpy as np
import torch

from .. import _device as D
from .. import _native as N
from .. import geometry
from ..sizing.size_function import SizeFunction
from . import utils as mutils

__all__ = ["sliver_removal", "generate_mesh"]

ADJ_CAP = {2: 32, 3: 64}


def silence(func):
    def wrapper(*args, **kwargs):
        return None

    return wrapper


def talk(func):
    def wrapper(*args, **kwargs):
        func(*args, **kwargs)

    return wrapper


def _select_verbosity(opts):
    if opts["verbose"] == 0:
        return silence, silence
    elif opts["verbose"] == 1:
        return talk, silence
    elif opts["verbose"] > 1:
        return talk, talk
    else:
        raise ValueError("Unknown verbosity level")


# ---------------------------------------------------------------------------
# domain / sizing adapters
class _Domain:
    """A geometry object (device SDF program) or a host callable."""

    def __init__(self, obj):
        self.obj = obj
        self.is_program = hasattr(obj, "device_program")
        # distances from a separate batched device evaluation (Isosurface,
        # NeuralSDF): no inline program, no host round trip
        self.is_batched = hasattr(obj, "batched_eval")

    def __call__(self, x):
        if self.is_program or self.is_batched:
            return self.obj.eval(x)
        return np.asarray(self.obj(x), dtype=float)

    def program(self):
        if not self.is_program:
            raise NotImplementedError(
                "host-callable domains are evaluated on the host for the cell filter"
            )
        return self.obj.device_program()


class _Sizing:
    """Scalar, gridded (device) or host-callable mesh size function."""

    def __init__(self, edge_length, dim):
        self.dim = dim
        self.host = None
        self.grid = None
        self.const = None
        fh = edge_length.eval if isinstance(edge_length, SizeFunction) else edge_length
        if np.isscalar(edge_length):
            self.const = float(edge_length)
        elif hasattr(fh, "device_grid"):
            self.grid = fh
        elif isinstance(edge_length, SizeFunction) and hasattr(edge_length.cell_size, "device_grid"):
            self.grid = edge_length.cell_size
        else:
            self.host = fh
        self.struct = N.Sizing()
        self.struct.dim = dim
        if self.const is not None:
            self.struct.kind = N.SIZING_CONST
            self.struct.h = self.const
        elif self.grid is not None:
            self.grid.fill_struct(self.struct)
        else:
            self.struct.kind = N.SIZING_SLOTS

    def __call__(self, x):
        x = np.asarray(x)
        if self.const is not None:
            return np.full(len(x), self.const)
        if self.grid is not None:
            return self.grid(x)
        return np.asarray(self.host(x), dtype=float)


# ---------------------------------------------------------------------------
def position_grid_exponent(p):
    """Exponent e of the position grid 2^e of a run: 24 bits below the
    largest coordinate magnitude (with 25% headroom), i.e. the resolution a
    float32 has at that magnitude.  Points on one such grid let the Delaunay
    kernels decide every predicate in fixed-point integer arithmetic."""
    p = np.asarray(p, dtype=float)
    E = float(np.abs(p).max()) * 1.25 if p.size else 1.0
    if not np.isfinite(E) or E <= 0:
        return N.DM_NO_GRID
    return math.frexp(E)[1] - 1 - 24


def snap_to_grid(p, e):
    """p rounded to multiples of 2^e (float64, exactly representable in float32)."""
    if e == N.DM_NO_GRID:
        return np.asarray(p, dtype=float)
    q = math.ldexp(1.0, e)
    return np.rint(np.asarray(p, dtype=float) / q) * q


def _fd_gradients(fd, p, d, deps):
    """one-sided finite-difference gradient of a host SDF and its squared
    norm floored at deps (generation/mesh_generator.py:773-780)"""
    dim = p.shape[1]
    grads = []
    for i in range(dim):
        q = p.copy()
        q[:, i] += deps
        grads.append((fd(q) - d) / deps)
    g2 = sum(g**2 for g in grads)
    return np.vstack(grads), np.where(g2 < deps, deps, g2)


def _project_points_back_host(p, fd, deps, hmin, idx):
    """_project_points_back_newton (generation/mesh_generator.py:762-784) for
    host-callable domains: one Newton step for points outside level idx"""
    d = fd(p)
    ix = d > 0.0 if idx == 0 else np.logical_and(d > 0.0, d < hmin / 1.5)
    if ix.any():
        g, g2 = _fd_gradients(fd, p[ix], d[ix], deps)
        p[ix] -= (d[ix] * g / g2).T
    return p


MAX_ADJ_CAP = 4096


class _Engine:
    """Device state of one meshing run.  With grid=True the points live on the
    position grid of the run (snapped here, kept there by the update
    kernels); grid=False keeps the caller's float32 points unchanged."""

    def __init__(self, dim, p_host, nfix, grid=True):
        self.dim = dim
        self.nfix = nfix
        p_host = np.asarray(p_host, dtype=float)
        self.grid_exp = position_grid_exponent(p_host) if grid else N.DM_NO_GRID
        if grid:
            p_host = snap_to_grid(p_host, self.grid_exp)
        self.set_points(D.to_points(p_host, dim))
        self.counters = D.zeros((N.NCOUNTERS,), torch.int64)
        self.adj_cap = ADJ_CAP[dim]

    def set_points(self, P):
        self.P = P
        self.n = P.shape[0]
        self.P2 = torch.empty_like(P)
        nv = self.dim + 1
        self.cap_cells = (7 if self.dim == 3 else 2) * self.n + 1024
        self.cells = D.empty((self.cap_cells, nv), torch.int32)
        self.kept = D.empty((self.cap_cells, nv), torch.int32)
        ws = N.c_sz(0)
        N.call("dm_delaunay_workspace_size", self.dim, self.n, ws)
        self.ws_dt = D.workspace(ws.value)
        self.adj = None
        self.ws_adj = None
        nblk = N.c_int(0)
        N.call("dm_bar_blocks", self.n, nblk)
        self.nblk = nblk.value
        self.partials = D.empty((2 * self.nblk + 3,), torch.float64)
        self.maxf = D.empty((self.nblk + 1,), torch.float32)

    def counters_host(self):
        return self.counters.cpu().numpy()

    def triangulate(self):
        """Delaunay of the current points; merges exact duplicates like CGAL."""
        for _ in range(8):
            N.call(
                "dm_delaunay", self.dim, D.ptr(self.P), self.n, D.ptr(self.cells),
                self.cap_cells, D.ptr(self.counters), D.ptr(self.ws_dt),
                self.ws_dt.numel(), D.stream_ptr(),
            )
            c = self.counters_host()
            flags = int(c[N.CNT_FLAGS])
            if flags & N.FLAG_DUPLICATES:
                self._merge_duplicates()
                continue
            if flags & N.FLAG_CELL_OVERFLOW:
                self.cap_cells = int(c[N.CNT_CELLS]) + 1024
                nv = self.dim + 1
                self.cells = D.empty((self.cap_cells, nv), torch.int32)
                self.kept = D.empty((self.cap_cells, nv), torch.int32)
                continue
            bad = flags & (N.FLAG_STAR_OVERFLOW | N.FLAG_SEED_FAILED | N.FLAG_EXACT_OVERFLOW | N.FLAG_NONFINITE)
            if bad:
                raise N.NativeError("dm_delaunay", N.DM_ERR_DEGENERATE, f"flags {flags:#x}")
            return int(c[N.CNT_CELLS])
        raise RuntimeError("triangulation did not stabilise")

    def _merge_duplicates(self):
        # CGAL keeps one vertex per location; so do we (first occurrence).
        p = self.P[:, : self.dim].cpu().numpy()
        _, first = np.unique(p, axis=0, return_index=True)
        keep = np.sort(first)
        removed_fixed = np.sum(keep < self.nfix)
        self.nfix = int(removed_fixed)
        self.set_points(self.P[torch.from_numpy(keep).to(self.P.device)].contiguous())

    def filter(self, domain, geps):
        if domain.is_batched:
            # centroids, then their distances in one batched evaluation
            nc = int(self.counters[N.CNT_CELLS].item())
            cen = D.empty((max(nc, 1), self.dim), torch.float32)
            N.call(
                "dm_cell_centroids", self.dim, D.ptr(self.P), D.ptr(self.cells), self.cap_cells,
                D.ptr(self.counters), D.ptr(cen), D.stream_ptr(),
            )
            d = D.empty((max(nc, 1),), torch.float32)
            domain.obj.batched_eval(cen, self.dim, nc, d, mode="cells")
            N.call(
                "dm_filter_cells_by_value", self.dim, D.ptr(self.cells), nc, D.ptr(d), geps,
                D.ptr(self.kept), D.ptr(self.counters), D.stream_ptr(),
            )
            return int(self.counters[N.CNT_KEPT].item())
        if domain.is_program:
            N.call(
                "dm_filter_cells", self.dim, D.ptr(self.P), D.ptr(self.cells), self.cap_cells,
                domain.program().struct, geps, D.ptr(self.kept), D.ptr(self.counters),
                None, 0, D.stream_ptr(),
            )
            return int(self.counters[N.CNT_KEPT].item())
        # host-callable domain: centroids on the device, distance on the host
        nc = int(self.counters[N.CNT_CELLS].item())
        cen = D.empty((max(nc, 1), self.dim), torch.float32)
        N.call(
            "dm_cell_centroids", self.dim, D.ptr(self.P), D.ptr(self.cells), self.cap_cells,
            D.ptr(self.counters), D.ptr(cen), D.stream_ptr(),
        )
        d = domain(cen[:nc].double().cpu().numpy())
        keep = torch.from_numpy(np.nonzero(d < -geps)[0]).to(self.P.device)
        k = keep.numel()
        self.kept[:k] = self.cells[:nc][keep]
        self.counters[N.CNT_KEPT] = k
        return k

    def adjacency_async(self):
        """dm_adjacency on the current stream, no host synchronisation"""
        if self.adj is None or self.adj.shape != (self.n, self.adj_cap):
            self.adj = D.empty((self.n, self.adj_cap), torch.int32)
            self.deg = D.empty((self.n,), torch.int32)
        ws = N.c_sz(0)
        N.call("dm_adjacency_workspace_size", self.dim, self.n, self.cap_cells, ws)
        if self.ws_adj is None or self.ws_adj.numel() < ws.value:
            self.ws_adj = D.workspace(ws.value)
        N.call(
            "dm_adjacency", self.dim, self.n, D.ptr(self.kept), self.cap_cells, N.CNT_KEPT,
            D.ptr(self.adj), self.adj_cap, D.ptr(self.deg), D.ptr(self.counters),
            D.ptr(self.ws_adj), self.ws_adj.numel(), D.stream_ptr(),
        )

    def build_adjacency(self):
        """Adjacency rows; widens the rows when a vertex has more neighbours
        than the row stride."""
        while True:
            self.adjacency_async()
            c = self.counters_host()
            flags = int(c[N.CNT_FLAGS])
            if not flags & N.FLAG_ADJ_OVERFLOW:
                return
            self.counters[N.CNT_FLAGS] = flags & ~N.FLAG_ADJ_OVERFLOW
            need = max(int(c[N.CNT_MAXDEG]), self.adj_cap + 1)
            cap = 1 << (need - 1).bit_length()
            rows = 4 * self.n * cap
            free, _ = torch.cuda.mem_get_info()
            if cap > MAX_ADJ_CAP or rows > free // 2:
                # a vertex adjacent to thousands of others: no DistMesh
                # iteration of a sound triangulation has one
                raise N.NativeError(
                    "dm_adjacency", N.DM_ERR_CAPACITY,
                    f"a vertex has {need} neighbours (rows are limited to {MAX_ADJ_CAP}; "
                    f"{cap} for {self.n} vertices would need {rows / 2**30:.1f} GiB)")
            self.adj_cap = cap

    def slot_sizes(self, sizing):
        """per adjacency slot h(midpoint) for host-callable sizing functions"""
        mid = D.empty((self.n, self.adj_cap, self.dim), torch.float32)
        N.call(
            "dm_slot_midpoints", self.dim, D.ptr(self.P), self.n, D.ptr(self.adj),
            self.adj_cap, D.ptr(self.deg), D.ptr(mid), D.stream_ptr(),
        )
        deg = self.deg.cpu().numpy()
        mask = np.arange(self.adj_cap)[None, :] < deg[:, None]
        m = mid.cpu().numpy()[mask]
        h = np.zeros((self.n, self.adj_cap), dtype=np.float32)
        if len(m):
            h[mask] = np.asarray(sizing(m.astype(float)), dtype=np.float32).reshape(-1)
        self._slot_h = torch.from_numpy(h).to(self.P.device)
        sizing.struct.slot_h = self._slot_h.data_ptr()

    def step(self, sizing, levels, L0mult, delta_t, h0, deps):
        if sizing.host is not None:
            self.slot_sizes(sizing)
        N.call(
            "dm_bar_sums", self.dim, D.ptr(self.P), self.n, D.ptr(self.adj), self.adj_cap,
            D.ptr(self.deg), sizing.struct, D.ptr(self.partials), D.stream_ptr(),
        )
        lv = (N.SdfProgram * max(1, len(levels)))()
        for i, L in enumerate(levels):
            lv[i] = L.program().struct
        N.call(
            "dm_update_points", self.dim, D.ptr(self.P), D.ptr(self.P2), self.n,
            D.ptr(self.adj), self.adj_cap, D.ptr(self.deg), sizing.struct,
            D.ptr(self.partials), L0mult, delta_t, self.nfix, lv, len(levels), h0,
            deps, D.ptr(self.maxf), self.grid_exp, D.stream_ptr(),
        )
        self.P, self.P2 = self.P2, self.P

    def max_movement(self, delta_t):
        return delta_t * float(self.maxf[self.nblk].item())

    def boundary_vertices(self, count_index):
        ws = N.c_sz(0)
        N.call("dm_boundary_workspace_size", self.dim, self.n, self.cap_cells, ws)
        w = D.workspace(ws.value)
        flags = D.empty((self.n,), torch.int32)
        N.call(
            "dm_boundary", self.dim, self.n, D.ptr(self.kept), self.cap_cells, count_index,
            D.ptr(flags), None, 0, D.ptr(self.counters), D.ptr(w), w.numel(), D.stream_ptr(),
        )
        return torch.nonzero(flags).reshape(-1).to(torch.int32)

    def compact(self):
        """fix_mesh(delete_unused=True) on the kept cells"""
        ws = N.c_sz(0)
        N.call("dm_compact_workspace_size", self.n, ws)
        w = D.workspace(ws.value)
        nout = N.c_i64(0)
        N.call(
            "dm_compact_vertices", self.dim, D.ptr(self.P), D.ptr(self.P2), self.n,
            D.ptr(self.kept), self.cap_cells, N.CNT_KEPT, D.ptr(self.counters), nout,
            D.ptr(w), w.numel(), D.stream_ptr(),
        )
        nk = int(self.counters[N.CNT_KEPT].item())
        P = self.P2[: nout.value].clone()
        kept = self.kept[:nk].clone()
        self.set_points(P)
        self.kept[:nk] = kept
        self.counters[N.CNT_KEPT] = nk
        return nk

    def project_batched(self, domain):
        """_project_points_back_newton with batched device distances: points
        with d > 0 move by -d grad (the exact SDF's unit gradient)"""
        d = D.empty((self.n,), torch.float32)
        g = D.empty((self.n, 4), torch.float32)
        W = self.P.shape[1]
        domain.obj.batched_eval(self.P, W, self.n, d, g, mode="points")
        N.call("dm_project_by_value", self.dim, D.ptr(self.P), self.n, D.ptr(d), D.ptr(g),
               self.grid_exp, D.stream_ptr())

    def project_host(self, levels, deps, hmin):
        """Newton projection on the host, for runs with a host-callable level
        (the slow path: positions make one round trip per iteration)"""
        p = D.from_points(self.P, self.dim)
        for idx, lv in enumerate(levels):
            p = _project_points_back_host(p, lv, deps, hmin, idx)
        if self.grid_exp != N.DM_NO_GRID:
            p = snap_to_grid(p, self.grid_exp)
        self.P.copy_(D.to_points(p, self.dim))

    def improve_level_set(self, domain, deps):
        if domain.is_batched:
            # _improve_level_set_newton with exact distances and gradients at
            # the boundary vertices: 5 damped steps p -= alpha d grad
            bid = self.boundary_vertices(N.CNT_KEPT)
            m = bid.numel()
            if m == 0:
                return
            d = D.empty((self.n,), torch.float32)
            g = D.empty((self.n, 4), torch.float32)
            cnt = torch.tensor([m], dtype=torch.int64, device=self.P.device)
            W = self.P.shape[1]
            alpha = 1.0
            for it in range(5):
                domain.obj.batched_eval(self.P, W, self.n, d, g, idx=bid, count=cnt)
                N.call("dm_newton_by_value", self.dim, D.ptr(self.P), D.ptr(bid), m, D.ptr(d),
                       D.ptr(g), alpha, self.grid_exp, D.stream_ptr())
                alpha /= it + 1
            return
        if not domain.is_program:
            # _improve_level_set_newton (generation/mesh_generator.py:741-759)
            # with the host callable
            bid = self.boundary_vertices(N.CNT_KEPT).long().cpu().numpy()
            if len(bid) == 0:
                return
            p = D.from_points(self.P, self.dim)
            alpha = 1.0
            for it in range(5):
                d = domain(p[bid])
                g, g2 = _fd_gradients(domain, p[bid], d, deps)
                p[bid] -= alpha * (d * g / g2).T
                alpha /= it + 1
            if self.grid_exp != N.DM_NO_GRID:
                p = snap_to_grid(p, self.grid_exp)
            self.P.copy_(D.to_points(p, self.dim))
            return
        bid = self.boundary_vertices(N.CNT_KEPT)
        if bid.numel():
            N.call(
                "dm_improve_level_set", self.dim, D.ptr(self.P), D.ptr(bid), bid.numel(),
                domain.program().struct, deps, D.stream_ptr(),
            )

    def refilter_kept(self, domain, geps):
        """_remove_triangles_outside on the kept set (final clean-up)"""
        nk = int(self.counters[N.CNT_KEPT].item())
        self.cells[:nk] = self.kept[:nk]
        self.counters[N.CNT_CELLS] = nk
        return self.filter(domain, geps)

    def boundary_delete_mask(self, min_qual):
        """cells touching a boundary vertex whose quality is < min_qual
        (geometry/utils.py:456-459), as a device bool mask over the kept cells"""
        nk = int(self.counters[N.CNT_KEPT].item())
        qual = D.empty((nk,), torch.float64)
        N.call("dm_simplex_metrics", self.dim, D.ptr(self.P), D.ptr(self.kept), nk,
               None, D.ptr(qual), D.stream_ptr())
        bflag = D.zeros((self.n,), torch.int32)
        bflag[self.boundary_vertices(N.CNT_KEPT).long()] = 1
        t = self.kept[:nk].long()
        touches = bflag[t].sum(1) > 0
        return touches & (qual < min_qual)

    def delete_boundary_entities(self, min_qual, verbose):
        """geometry.delete_boundary_entities (geometry/utils.py:440-469):
        drop cells touching a boundary vertex whose quality is < min_qual"""
        nk = int(self.counters[N.CNT_KEPT].item())
        if nk == 0:
            return
        delete = self.boundary_delete_mask(min_qual)
        if verbose:
            print("Deleting " + str(int(delete.sum().item())) + " poor quality boundary entities...", flush=True)
        keep = self.kept[:nk][~delete].clone()
        self.kept[: keep.shape[0]] = keep
        self.counters[N.CNT_KEPT] = keep.shape[0]
        self.compact()

    def laplacian_smooth(self):
        """geometry.laplacian2_fixed_point (geometry/utils.py:494-547)"""
        from ..geometry import utils as gu

        gu._laplacian_device(self)

    def load_mesh(self, p, t):
        """replace points and kept cells by a host mesh (p exact in float32:
        it came from this engine's points)"""
        self.set_points(D.to_points(p, self.dim))
        nk = len(t)
        if nk:
            self.kept[:nk] = torch.from_numpy(np.ascontiguousarray(t, dtype=np.int32)).to(D.device())
        self.counters[N.CNT_KEPT] = nk

    def result(self):
        nk = int(self.counters[N.CNT_KEPT].item())
        p = D.from_points(self.P, self.dim)
        t = self.kept[:nk].cpu().numpy().astype(np.int32)
        return p, t


# ---------------------------------------------------------------------------
def generate_mesh(domain, edge_length, comm=None, **kwargs):  # noqa: C901
    r"""Generate a 2D/3D mesh using callbacks to a sizing function `edge_length`
    and signed distance function `domain` (same keywords and defaults as the
    reference generate_mesh, generation/mesh_generator.py:291-529).

    :return: points (numpy.ndarray[float x dim]), cells (numpy.ndarray[int32 x (dim+1)])
    """
    _check_comm(comm)
    gen_opts = {
        "verbose": 1,
        "max_iter": 50,
        "seed": 0,
        "perform_checks": False,
        "pfix": None,
        "axis": 1,
        "points": None,
        "delta_t": 0.30,
        "geps_mult": 0.1,
        "subdomains": None,
        "mesh_improvement": True,
        "r0m_is_h0": False,
    }
    gen_opts.update(kwargs)
    _parse_kwargs(kwargs)

    verbosity1, verbosity2 = _select_verbosity(gen_opts)

    @verbosity1
    def print_msg1(msg):
        print(msg, flush=True)

    @verbosity2
    def print_msg2(msg):
        print(msg, flush=True)

    run = _Run(domain, edge_length, gen_opts, print_msg1)
    count = 0
    while count < run.max_iter - 1:
        start = time.time()
        run.iterate(count, print_msg2)
        count += 1
        print_msg2("     Elapsed wall-clock time %f : " % (time.time() - start))
    run.finish(print_msg1)
    return run.eng.result()


class _Run:
    """One generate_mesh problem (generation/mesh_generator.py:291-529): the
    set-up, one DistMesh iteration (checked: duplicates, capacities and row
    widths handled on the host), the same iteration as a host-synchronisation
    free launch sequence for CUDA-graph capture, and the termination."""

    def __init__(self, domain, edge_length, gen_opts, print_msg1=lambda m: None):
        self.opts = gen_opts
        fd, bbox0, corners = _unpack_domain(domain, gen_opts)
        fh, bbox1, hmin, lsf = _unpack_sizing(edge_length)

        bbox = bbox0 if bbox1 is None else _minmax(bbox0, bbox1)
        if not isinstance(bbox, tuple):
            raise ValueError("`bbox` must be a tuple")
        dim = int(len(bbox) / 2)

        if not np.isscalar(edge_length) and dim == 3:
            corners = None

        if bbox0 != bbox1 and bbox1 is not None:
            fd = _Domain(geometry.Rectangle(bbox) if dim == 2 else geometry.Cube(bbox))

        bbox = np.array(bbox).reshape(-1, 2)
        h0 = hmin if hmin is not None else gen_opts["h0"]
        if h0 < 0:
            raise ValueError("`h0` must be > 0")

        self.dim, self.fd, self.h0 = dim, fd, h0
        self.L0mult = 1 + 0.4 / 2 ** (dim - 1)
        self.delta_t = gen_opts["delta_t"]
        self.geps = gen_opts["geps_mult"] * h0
        self.deps = np.sqrt(np.finfo(np.double).eps) * h0

        self.sizing = _Sizing(edge_length, dim)

        pfix, nfix = _unpack_pfix(dim, gen_opts)
        if corners is not None:
            corners = corners[fd(corners) > -1000 * self.deps]
            pfix = np.append(pfix, corners, axis=0)
            nfix = len(pfix)
        print_msg1(f"Constraining {nfix} fixed points...")

        p = _initialize_points(dim, self.geps, bbox, self.sizing, fd, h0, gen_opts, pfix)

        if gen_opts["max_iter"] < 0:
            raise ValueError("`max_iter` must be > 0")
        self.max_iter = gen_opts["max_iter"]
        N_pts = p.shape[0]
        assert N_pts > 0, "No vertices to mesh with!"
        print_msg1("Commencing mesh generation with %d vertices on rank %d." % (N_pts, 0))

        levels = [fd]
        if gen_opts["subdomains"] is not None:
            for sub in gen_opts["subdomains"]:
                sfd, _, _ = _unpack_domain(sub, gen_opts)
                levels.append(sfd)
        self.levels = levels
        self.batched = fd.is_batched
        if self.batched and len(levels) > 1:
            raise NotImplementedError("subdomains are not supported with a batched-SDF domain")
        # a host-callable level moves the projection to the host (slow path)
        self.host_levels = not self.batched and not all(lv.is_program for lv in levels)
        if self.host_levels:
            print_msg1("Host-callable domain: the Newton projection runs on the host")
        self.eng = _Engine(dim, p, nfix)
        self._lv = None

    @property
    def capturable(self):
        """the iteration can run as one host-synchronisation free sequence"""
        return (not self.batched and not self.host_levels and self.sizing.host is None
                and self.fd.is_program)

    def iterate(self, count, print_msg2=lambda m: None):
        eng = self.eng
        eng.triangulate()
        eng.filter(self.fd, self.geps)
        eng.build_adjacency()
        eng.step(self.sizing, [] if (self.host_levels or self.batched) else self.levels,
                 self.L0mult, self.delta_t, self.h0, self.deps)
        if self.batched:
            eng.project_batched(self.fd)
        elif self.host_levels:
            eng.project_host(self.levels, self.deps, self.h0)
        maxdp = eng.max_movement(self.delta_t)
        print_msg2(
            "Iteration #%d, max movement is %f, there are %d vertices and %d cells"
            % (count + 1, maxdp, eng.n, int(eng.counters[N.CNT_KEPT].item()))
        )
        assert maxdp < 1000 * self.h0, "max movement indicates there's a convergence problem"

    def iterate_async(self, flags_out):
        """the checked iteration's kernels on the current stream, with no host
        synchronisation: points are read from P and the result copied back
        into P, so a captured graph replays on fixed buffers.  The device
        flags of the iteration are OR-ed into flags_out (int64[1]); a set
        flag means the result must be discarded and the iteration redone
        with iterate()."""
        eng = self.eng
        st = D.stream_ptr()
        if self._lv is None:
            self._lv = (N.SdfProgram * len(self.levels))()
            for i, L in enumerate(self.levels):
                self._lv[i] = L.program().struct
        N.call("dm_delaunay", self.dim, D.ptr(eng.P), eng.n, D.ptr(eng.cells), eng.cap_cells,
               D.ptr(eng.counters), D.ptr(eng.ws_dt), eng.ws_dt.numel(), st)
        N.call("dm_filter_cells", self.dim, D.ptr(eng.P), D.ptr(eng.cells), eng.cap_cells,
               self.fd.program().struct, self.geps, D.ptr(eng.kept), D.ptr(eng.counters), None,
               0, st)
        eng.adjacency_async()
        N.call("dm_bar_sums", self.dim, D.ptr(eng.P), eng.n, D.ptr(eng.adj), eng.adj_cap,
               D.ptr(eng.deg), self.sizing.struct, D.ptr(eng.partials), st)
        N.call("dm_update_points", self.dim, D.ptr(eng.P), D.ptr(eng.P2), eng.n, D.ptr(eng.adj),
               eng.adj_cap, D.ptr(eng.deg), self.sizing.struct, D.ptr(eng.partials), self.L0mult,
               self.delta_t, eng.nfix, self._lv, len(self.levels), self.h0, self.deps,
               D.ptr(eng.maxf), eng.grid_exp, st)
        eng.P.copy_(eng.P2)
        torch.bitwise_or(flags_out, eng.counters[N.CNT_FLAGS:N.CNT_FLAGS + 1], out=flags_out)

    def finish(self, print_msg1=lambda m: None):
        eng = self.eng
        eng.triangulate()
        eng.filter(self.fd, self.geps)
        print_msg1("Termination reached...maximum number of iterations reached.")
        _termination(eng, self.fd, self.opts, self.h0, self.deps)


def _termination(eng, fd, opts, h0, deps, sliver=False):
    """_termination + _improve_level_set_newton + final filter
    (generation/mesh_generator.py:485-494, 655-677, 741-759)."""
    if eng.dim == 2:
        eng.compact()
        eng.delete_boundary_entities(0.15, opts["verbose"])
        if opts["subdomains"] is None and opts["mesh_improvement"]:
            eng.laplacian_smooth()
    eng.compact()
    if opts.get("perform_checks"):
        # geometry.linter, as the reference's _termination does when asked
        # (generation/mesh_generator.py:672-673)
        p, t = eng.result()
        p, t = geometry.linter(p, t, dim=eng.dim)
        eng.load_mesh(p, t)
    if sliver:
        return
    eng.improve_level_set(fd, deps)
    eng.refilter_kept(fd, h0 * 0.001)


def _calc_dihedral_angles(p, t, min_dh_bound, max_dh_bound):
    dh = geometry.calc_dihedral_angles(p, t)
    out = np.argwhere((dh[:, 0] < min_dh_bound) | (dh[:, 0] > max_dh_bound))
    ele = np.floor(out / 6).astype("int")
    return np.unique(ele, return_index=True)


def sliver_removal(points, domain, edge_length, comm=None, **kwargs):  # noqa: C901
    r"""Improve an existing 3D mesh by removing slivers (reference
    generation/mesh_generator.py:59-288): retriangulate, flag cells with a
    dihedral angle outside [min, max], push vertex 0 of each flagged cell
    along the gradient of its circumradius, adapt the step."""
    _check_comm(comm)
    sliver_opts = {
        "verbose": 1,
        "max_iter": 50,
        "perform_checks": False,
        "axis": 1,
        "min_dh_angle_bound": 10.0,
        "max_dh_angle_bound": 180.0,
        "points": None,
        "delta_t": 0.30,
        "geps_mult": 0.1,
        "subdomains": [],
        "gamma": 1.0,
        "preserve": False,
    }
    sliver_opts.update(kwargs)
    _parse_kwargs(kwargs)
    verbosity1, verbosity2 = _select_verbosity(sliver_opts)

    @verbosity1
    def print_msg1(msg):
        print(msg, flush=True)

    @verbosity2
    def print_msg2(msg):
        print(msg, flush=True)

    dim = points.shape[1]
    if dim == 2:
        raise Exception("Mesh improvement currently on works in 3D")

    fd, bbox0, _ = _unpack_domain(domain, sliver_opts)
    fh, bbox1, hmin, _ = _unpack_sizing(edge_length)
    bbox = bbox0 if bbox1 is None else _minmax(bbox0, bbox1)
    if bbox0 != bbox1 and bbox1 is not None:
        fd = _Domain(geometry.Cube(bbox))
    if not isinstance(bbox, tuple):
        raise ValueError("`bbox` must be a tuple")
    h0 = hmin if hmin is not None else sliver_opts["h0"]
    if h0 < 0:
        raise ValueError("`h0` must be > 0")
    if sliver_opts["max_iter"] < 0:
        raise ValueError("`max_iter` must be > 0")
    max_iter = sliver_opts["max_iter"]
    print_msg1(f"Will attempt {max_iter} iterations to bound the dihedral angles...")
    geps = sliver_opts["geps_mult"] * h0
    deps = np.sqrt(np.finfo(np.double).eps) * h0
    min_dh_bound = sliver_opts["min_dh_angle_bound"] * math.pi / 180
    max_dh_bound = sliver_opts["max_dh_angle_bound"] * math.pi / 180
    print_msg1(f"Enforcing a min. dihedral bound of: {min_dh_bound * 180 / math.pi} degrees...")
    print_msg1(f"Enforcing a max. dihedral bound of: {max_dh_bound * 180 / math.pi} degrees...")
    print_msg1("Commencing sliver removal with %d vertices on rank %d." % (len(points), 0))

    eng = _Engine(3, np.asarray(points), 0)
    flags = None
    ws = N.c_sz(0)
    count = 0
    step = 0.10
    gamma = sliver_opts["gamma"]
    num_old_bad = np.inf
    while True:
        start = time.time()
        eng.triangulate()
        eng.filter(fd, geps)
        if flags is None or flags.numel() < eng.cap_cells:
            flags = D.empty((eng.cap_cells,), torch.int32)
        N.call(
            "dm_dihedral_flags", D.ptr(eng.P), D.ptr(eng.kept), eng.cap_cells, N.CNT_KEPT,
            min_dh_bound, max_dh_bound, D.ptr(flags), D.ptr(eng.counters), D.stream_ptr(),
        )
        num_bad = int(eng.counters[N.CNT_BAD].item())
        if count == max_iter - 1:
            print_msg1(
                "FAILURE: Termination...maximum number of iterations reached. Try increasing max_iter when generating the mesh",
            )
            _termination(eng, fd, sliver_opts, h0, deps, sliver=True)
            break
        print_msg1(f"On rank: 0. There are {num_bad} slivers...")
        if num_bad == 0:
            print_msg1(f"Termination reached in {count} iterations...no slivers detected!")
            eng.compact()
            return eng.result()
        if num_bad < num_old_bad:
            step /= gamma
        elif num_bad > num_old_bad:
            step *= gamma
        else:
            step /= 0.8
        N.call("dm_sliver_workspace_size", eng.n, ws)
        w = D.workspace(ws.value)
        N.call(
            "dm_sliver_perturb", D.ptr(eng.P), eng.n, D.ptr(eng.kept), eng.cap_cells,
            N.CNT_KEPT, D.ptr(flags), step * h0, eng.grid_exp, D.ptr(w), w.numel(),
            D.ptr(eng.counters), D.stream_ptr(),
        )
        if sliver_opts["preserve"]:
            eng.improve_level_set(fd, deps)
        count += 1
        num_old_bad = num_bad
        print_msg2("     Elapsed wall-clock time %f : " % (time.time() - start))
    return eng.result()


# ---------------------------------------------------------------------------
def _check_comm(comm):
    if comm is not None and getattr(comm, "size", 1) > 1:
        raise NotImplementedError(
            "the GPU engine meshes one domain per GPU; MPI slab decomposition is not supported"
        )


def _minmax(bbox0, bbox1):
    d = []
    for i, (a, b) in enumerate(zip(bbox0, bbox1)):
        d.append(max(a, b) if i % 2 else min(a, b))
    return tuple(d)


def _check_bbox(bbox):
    if bbox is not None:
        for b in bbox:
            if isinstance(b, int):
                raise ValueError("bbox must contain all floats")


def _unpack_sizing(edge_length):
    bbox = None
    hmin = None
    lsf = False
    if isinstance(edge_length, SizeFunction):
        bbox = edge_length.bbox
        fh = edge_length.eval
        hmin = edge_length.hmin
        lsf = True
    elif callable(edge_length):
        fh = edge_length
    elif np.isscalar(edge_length):

        def fh(x):
            if type(x) == tuple:
                return np.zeros_like(x[0]) + edge_length
            return np.array([edge_length] * len(x))

        hmin = edge_length
        lsf = True
    else:
        raise ValueError(
            "`edge_length` must either be a function, a `edge_length` object, or a scalar"
        )
    _check_bbox(bbox)
    return fh, bbox, hmin, lsf


_GEOMETRY_TYPES = None


def _unpack_domain(domain, opts):
    global _GEOMETRY_TYPES
    if _GEOMETRY_TYPES is None:
        _GEOMETRY_TYPES = (
            geometry.Ball, geometry.Rectangle, geometry.Disk, geometry.Cube,
            geometry.Cylinder, geometry.Torus, geometry.Prism, geometry.Union,
            geometry.Intersection, geometry.Difference, geometry.Repeat, geometry.GridSDF,
        )
    corners = None
    if isinstance(domain, _GEOMETRY_TYPES):
        bbox = domain.bbox
        fd = _Domain(domain)
        corners = domain.corners
    elif hasattr(domain, "batched_eval"):
        bbox = tuple(domain.bbox)
        fd = _Domain(domain)
    elif callable(domain):
        bbox = opts["bbox"]
        fd = _Domain(domain)
    else:
        raise ValueError("`domain` must be a function or a :class:`geometry` object")
    _check_bbox(bbox)
    return fd, bbox, corners


def _parse_kwargs(kwargs):
    allowed = {
        "verbose", "max_iter", "seed", "perform_checks", "pfix", "axis", "points",
        "domain", "edge_length", "bbox", "min_dh_angle_bound", "max_dh_angle_bound",
        "delta_t", "h0", "geps_mult", "subdomains", "gamma", "preserve",
        "mesh_improvement", "r0m_is_h0",
    }
    for key in kwargs:
        if key not in allowed:
            raise ValueError("Option %s with parameter %s not recognized " % (key, kwargs[key]))


def _unpack_pfix(dim, opts):
    if opts["pfix"] is not None:
        pfix = np.array(opts["pfix"], dtype="d")
        return pfix, len(pfix)
    return np.empty((0, dim)), 0


def _initialize_points(dim, geps, bbox, sizing, fd, h0, opts, pfix):
    """_initialize_points / _generate_initial_points (808-864) for one rank:
    staggered lattice, SDF rejection, seeded decimation rand < r0m^d / r0^d."""
    if opts["points"] is not None:
        return np.asarray(opts["points"], dtype=float)
    p = mutils.create_staggered_grid(h0, dim, bbox)
    p = p[fd(p) < geps]
    r0 = sizing(p)
    if opts["r0m_is_h0"]:
        if dim == 2 and 1.1 * h0 < r0.min():
            r0m = 1.1 * h0
        elif dim == 3 and 1.1 * h0 < r0.min():
            r0m = 1.1 * h0
            warnings.warn("Warning: r0m_is_h0 option not test for 3D meshes.")
        else:
            r0m = h0
    else:
        r0m = r0.min()
    np.random.seed(opts["seed"])
    return np.vstack((pfix, p[np.random.rand(p.shape[0]) < r0m**dim / r0**dim]))
