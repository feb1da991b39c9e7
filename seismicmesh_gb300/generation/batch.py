"""Many independent meshing problems stepped together on one GPU.

The reference meshes one domain per call (generate_mesh,
generation/mesh_generator.py:291-529).  `generate_meshes` takes a list of
problems of uneven sizes, sets each up exactly as generate_mesh does, and
runs their DistMesh iterations together:

* the first `checked` iterations per problem take the checked path (exact
  duplicates of the initial lattice merged, cell capacity and adjacency row
  width settled);
* every later iteration of all capturable problems (SDF-program domains,
  device sizing) is one CUDA graph launch: the problems' launch sequences
  are captured on several streams, the largest problems first, each stream
  taking the next problem when it has the least work;
* the number of streams is tuned on the first graph iterations: each
  candidate is captured and timed on one real iteration (CUDA events), and
  the fastest is kept for the rest;
* a problem whose device flags were raised in a graph iteration
  (duplicates, capacity, row width) gets its positions back from the copy the
  graph made at the start of the iteration and redoes it on the checked
  path;
* termination runs per problem, as in generate_mesh.

Every kernel and every iteration is the one generate_mesh runs, so each
problem's mesh is the one generate_mesh returns for it.
"""
import time

import numpy as np
import torch

from .. import _device as D
from .. import _native as N
from .mesh_generator import _parse_kwargs, _Run

__all__ = ["generate_meshes"]


def _assign(sizes, nstreams):
    """largest first, each to the stream with the least work so far"""
    load = [0] * nstreams
    out = {}
    for i in sorted(range(len(sizes)), key=lambda k: -sizes[k]):
        s = int(np.argmin(load))
        out[i] = s
        load[s] += sizes[i]
    return out


def _buffers(r):
    """the device buffers a captured iteration of run r refers to"""
    e = r.eng
    return (e.n, e.cap_cells, e.adj_cap, e.P.data_ptr(), e.P2.data_ptr(), e.cells.data_ptr(),
            e.kept.data_ptr(), e.adj.data_ptr(), e.deg.data_ptr(), e.ws_dt.data_ptr(),
            e.ws_adj.data_ptr(), e.partials.data_ptr(), e.maxf.data_ptr(),
            e.counters.data_ptr())


class _Graph:
    def __init__(self, runs, idx, flags, saved, nstreams):
        self.nstreams = nstreams
        self.graph = torch.cuda.CUDAGraph()
        streams = [torch.cuda.Stream() for _ in range(nstreams)]
        assign = _assign([runs[i].eng.n for i in idx], nstreams)
        torch.cuda.synchronize()
        with torch.cuda.graph(self.graph):
            cur = torch.cuda.current_stream()
            for st in streams:
                st.wait_stream(cur)
            for k, i in enumerate(idx):
                with torch.cuda.stream(streams[assign[k]]):
                    saved[i].copy_(runs[i].eng.P)
                    runs[i].iterate_async(flags[i:i + 1])
            for st in streams:
                cur.wait_stream(st)
        torch.cuda.synchronize()


def generate_meshes(problems, candidates=(4, 8, 16, 32), checked=3, stats=None, **kwargs):
    """Mesh every (domain, edge_length) of `problems` with the keyword
    options of generate_mesh (shared by all), stepping them together.
    Returns the list of (points, cells) in the order of `problems` (None for
    a problem whose checked iterations raised, as generate_mesh would; its
    error is in stats["failed"]); `stats` (a dict, optional) receives the
    tuning record and timings."""
    gen_opts = {
        "verbose": 0, "max_iter": 50, "seed": 0, "perform_checks": False, "pfix": None,
        "axis": 1, "points": None, "delta_t": 0.30, "geps_mult": 0.1, "subdomains": None,
        "mesh_improvement": True, "r0m_is_h0": False,
    }
    gen_opts.update(kwargs)
    _parse_kwargs(kwargs)
    stats = {} if stats is None else stats
    t0 = time.perf_counter()
    runs = [_Run(dom, h, dict(gen_opts)) for dom, h in problems]
    torch.cuda.synchronize()
    stats["setup_s"] = time.perf_counter() - t0
    n_iter = gen_opts["max_iter"] - 1
    first = min(checked, n_iter)
    t1 = time.perf_counter()
    failed = {}
    for count in range(first):
        for i, r in enumerate(runs):
            if i in failed:
                continue
            try:
                r.iterate(count)
            except (N.NativeError, AssertionError) as e:
                # a problem generate_mesh itself would fail on: reported, not
                # meshed, and the batch goes on
                failed[i] = repr(e)[:300]
    torch.cuda.synchronize()
    stats["checked_s"] = time.perf_counter() - t1
    stats["failed"] = failed
    keep = [i for i in range(len(runs)) if i not in failed]
    stats["points"] = [runs[i].eng.n for i in keep]
    idx = [i for i in keep if runs[i].capturable]
    flags = D.zeros((len(runs),), torch.int64)
    saved = {i: torch.empty_like(runs[i].eng.P) for i in idx}
    graphs = {}
    tuning = []
    best = None
    redone = 0
    graph_ms = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t2 = time.perf_counter()
    for count in range(first, n_iter):
        if best is None and len(tuning) < len(candidates):
            ns = candidates[len(tuning)]
        else:
            if best is None:
                best = min(tuning, key=lambda r: r[1])[0]
            ns = best
        if idx and ns not in graphs:
            graphs[ns] = _Graph(runs, idx, flags, saved, ns)
        flags.zero_()
        if idx:
            ev0.record()
            graphs[ns].graph.replay()
            ev1.record()
        for i in keep:
            if i not in saved:
                runs[i].iterate(count)
        torch.cuda.synchronize()
        if idx:
            ms = ev0.elapsed_time(ev1)
            graph_ms.append(ms)
            if best is None and len(tuning) < len(candidates):
                tuning.append((ns, ms))
        bad = torch.nonzero(flags).reshape(-1).tolist()
        for i in bad:
            before = _buffers(runs[i])
            runs[i].eng.P.copy_(saved[i])
            runs[i].eng.counters[N.CNT_FLAGS] = 0
            runs[i].iterate(count)
            redone += 1
            if _buffers(runs[i]) != before:
                # the checked path reallocated (merged duplicates, more cell
                # capacity, wider rows): the graphs point at freed buffers
                graphs.clear()
                saved[i] = torch.empty_like(runs[i].eng.P)
    torch.cuda.synchronize()
    stats["graph_iterations_s"] = time.perf_counter() - t2
    stats["tuning"] = [{"streams": ns, "ms": ms} for ns, ms in tuning]
    stats["streams"] = best if best is not None else (tuning[-1][0] if tuning else None)
    stats["graph_ms"] = graph_ms
    stats["redone"] = redone
    stats["captured_problems"] = len(idx)
    t3 = time.perf_counter()
    out = []
    for i, r in enumerate(runs):
        if i in failed:
            out.append(None)
            continue
        r.finish()
        out.append(r.eng.result())
    stats["termination_s"] = time.perf_counter() - t3
    return out
