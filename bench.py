"""Benchmark: DistMesh point-iterations/s and time-to-mesh on one GB300.

Workload: 3D unit ball (Ball((0,0,0), 1)), constant edge length h = 0.02,
526,727 initial vertices, max_iter 50, seed 0, then sliver_removal with a
10 degree minimum dihedral angle.

  step    one DistMesh iteration on the device-resident point set:
          dm_delaunay -> dm_filter_cells -> dm_adjacency -> dm_bar_sums ->
          dm_update_points.  The first W (warm-up) iterations start from the
          initial lattice; the K timed iterations follow.  Each step is timed
          with CUDA events on the launching stream; a 256 MB buffer is written
          between steps so L2 (129 MB) holds none of the step's inputs.
  value   point-iterations/s = n_points * K / sum(step times).
  e2e     the same metric through the public API from host data:
          generate_mesh(Ball, 0.02) + sliver_removal, host numpy in, host
          numpy out; e2e value = n_points * (max_iter - 1) / wall time of
          generate_mesh; time_to_mesh_s includes sliver_removal.

--impl reference times the reference's CPU loop (the oracle's float64 numpy
restatement; CGAL and MPI are not available, so the triangulation is the
faster of the two stubs: the oracle's exact-predicate C++ Delaunay
(oracle/cdt3.cpp) when it builds, else Qhull) on the same workload: the
h = 0.02 ball, one DistMesh iteration per step.
With torchrun (N > 1) every rank meshes its own replica; value is the sum
over ranks (timed with a barrier and the max over ranks).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

H = 0.02
METRIC = "point-iterations/s (3D unit ball, h=0.02, DistMesh iterations)"


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x, world, backend):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, world, max_ms):
    """whole-job rate of `world` replicas that each processed
    `units_per_rank` units, timed by the slowest rank (max_ms)"""
    return world * units_per_rank / (max_ms / 1000.0)


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region"""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        cmd = [
            "nvidia-smi", f"--id={self.index}",
            "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
            "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
            "clocks_event_reasons.sw_power_cap",
            "--format=csv,noheader,nounits", "-lms", "200",
        ]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 3 + k and r[3 + k].lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": mx,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def measured_peaks_all():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "kind": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "kind": "fallback"}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def host_info():
    """core count and CPU model of this host"""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k = line.split(":")[0].strip().lower()
                if k in ("model name", "cpu part", "processor name"):
                    model = line.split(":", 1)[1].strip()
                    if k == "model name":
                        break
    except OSError:
        pass
    try:
        lscpu = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in lscpu.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"nproc": os.cpu_count(), "cpu_model": model}


def cpu_triangulator():
    """the faster triangulation stub of the oracle's loop: the C++
    exact-predicate Delaunay (1.7-3x Qhull on the h = 0.02 ball's iterations,
    2.7x on its initial lattice) when it builds here, else Qhull; returns
    (function, description)"""
    from oracle import cdt
    from oracle import distmesh_np as O

    if not cdt.available():
        return None, "Qhull (the C++ triangulator did not build here)"
    fallbacks = []

    def tri(p):
        try:
            return cdt.delaunay(p)
        except RuntimeError as e:  # reported in the line, never expected
            fallbacks.append(str(e))
            return O.delaunay(p)

    class Name:
        def __str__(self):
            extra = f"; Qhull on {len(fallbacks)} iterations it failed" if fallbacks else ""
            return "the oracle's exact-predicate C++ Delaunay (oracle/cdt3.cpp)" + extra

    return tri, Name()


def cpu_sample(steps, warmup, h=H):
    """the oracle's restatement of the reference loop (float64 numpy, with
    the faster triangulation stub) on the unit ball at edge length h:
    `warmup` untimed iterations from the initial lattice, then `steps` timed
    ones; returns (points, seconds, per-step seconds, triangulator)"""
    from oracle import distmesh_np as O
    from oracle import sdf_np as S

    tri, tri_name = cpu_triangulator()

    fd = S.ball(0.0, 0.0, 0.0, 1.0)
    fh = lambda x: np.full(len(x), h)  # noqa: E731
    bbox = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    p = O.initial_points(fd, fh, h, bbox, 0.1 * h, 3)
    for _ in range(warmup):
        p, _, _ = O.one_iteration(p, fd, fh, h, tri=tri)
    per = []
    for _ in range(steps):
        t0 = time.perf_counter()
        p, _, _ = O.one_iteration(p, fd, fh, h, tri=tri)
        per.append(time.perf_counter() - t0)
    return len(p), sum(per), per, tri_name


def run_reference(args, world, rank):
    """The reference's CPU loop on this arm's workload: the h = 0.02 unit ball
    (526,727 points), one DistMesh iteration per step, W untimed warm-up
    iterations from the initial lattice, then K timed.  The reference package
    itself cannot be installed on this machine (CGAL, Boost, GMP/MPFR and
    mpi4py are absent), so its loop runs as the oracle's float64 numpy
    restatement with the faster triangulation stub in CGAL's place; serial,
    as the reference's serial mode is (its MPI mode is not runnable here)."""
    if rank != 0:
        return
    n, dt, per, tri_name = cpu_sample(args.steps, args.warmup)
    value = n * args.steps / dt
    info = host_info()
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "point-iterations/s",
        "impl": "reference",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * dt / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (initial lattice of the unit ball, seeded decimation)",
        "config": {
            "workload": "3D unit ball, h=0.02, DistMesh iterations after 'warmup' iterations from "
                        "the initial lattice",
            "n_points": n,
            "parallelism": "serial (1 core)",
        },
        "host": info,
        "phases_ms": {"step_ms_min": 1000 * min(per), "step_ms_max": 1000 * max(per)},
        "cpu_baseline": {
            "value": value, "unit": "point-iterations/s", "cores": 1, "kind": "port",
            "sample": f"{args.steps} DistMesh iterations of the h=0.02 unit ball ({n} points) after "
                      f"{args.warmup} warm-up iterations: float64 numpy restatement of the reference "
                      f"loop, triangulated by {tri_name} (CGAL not installable), serial; "
                      f"host {info['nproc']} cores, {info['cpu_model']}",
        },
        "e2e": {"value": value, "unit": "point-iterations/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args, world, rank, local):
    import ctypes

    import torch

    from seismicmesh_gb300 import _build

    _build.build_library()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import seismicmesh_gb300 as sm
    from seismicmesh_gb300 import _device as D
    from seismicmesh_gb300 import _native as N
    from seismicmesh_gb300.generation import mesh_generator as MG

    L = N.lib()
    L.dmprof_read.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_int32)]
    L.dmprof_launches.restype = ctypes.c_int64

    ball = sm.Ball([0.0, 0.0, 0.0], 1.0)
    fd = MG._Domain(ball)
    sizing = MG._Sizing(H, 3)
    opts = {"points": None, "r0m_is_h0": False, "seed": 0}
    p0 = MG._initialize_points(3, 0.1 * H, np.array([[-1.0, 1.0]] * 3), sizing, fd, H, opts, np.empty((0, 3)))
    n = len(p0)
    L0mult = 1 + 0.4 / 2 ** 2
    deps = float(np.sqrt(np.finfo(float).eps) * H)
    eng = MG._Engine(3, p0, 0)
    levels = [fd]
    lv = (N.SdfProgram * 1)()
    lv[0] = fd.program().struct
    prog = fd.program().struct
    stream = D.stream_ptr()

    sticky = torch.zeros(1, dtype=torch.int64, device="cuda")

    def iteration_async():
        stream = D.stream_ptr()  # the current stream (a capture stream inside a graph)
        N.call("dm_delaunay", 3, D.ptr(eng.P), eng.n, D.ptr(eng.cells), eng.cap_cells,
               D.ptr(eng.counters), D.ptr(eng.ws_dt), eng.ws_dt.numel(), stream)
        N.call("dm_filter_cells", 3, D.ptr(eng.P), D.ptr(eng.cells), eng.cap_cells, prog,
               0.1 * H, D.ptr(eng.kept), D.ptr(eng.counters), None, 0, stream)
        eng.adjacency_async()
        N.call("dm_bar_sums", 3, D.ptr(eng.P), eng.n, D.ptr(eng.adj), eng.adj_cap,
               D.ptr(eng.deg), sizing.struct, D.ptr(eng.partials), stream)
        N.call("dm_update_points", 3, D.ptr(eng.P), D.ptr(eng.P2), eng.n, D.ptr(eng.adj),
               eng.adj_cap, D.ptr(eng.deg), sizing.struct, D.ptr(eng.partials), L0mult, 0.30,
               0, lv, 1, H, deps, D.ptr(eng.maxf), eng.grid_exp, stream)
        eng.P, eng.P2 = eng.P2, eng.P
        # flags of every timed iteration (dm_delaunay clears the counters)
        torch.bitwise_or(sticky, eng.counters[N.CNT_FLAGS:N.CNT_FLAGS + 1], out=sticky)

    # warm-up: the checked path (duplicates / capacity handled)
    for _ in range(args.warmup):
        eng.triangulate()
        eng.filter(fd, 0.1 * H)
        eng.build_adjacency()
        eng.step(sizing, levels, L0mult, 0.30, H, deps)
    torch.cuda.synchronize()
    # one DistMesh iteration as a CUDA graph: positions are copied back in
    # place so every replay sees the same buffers.  Captured with the star
    # kernels' event marks as event-record nodes (timed at every replay).
    graph = None
    try:
        def iteration_inplace():
            iteration_async()
            eng.P, eng.P2 = eng.P2, eng.P
            eng.P.copy_(eng.P2)

        s0 = torch.cuda.Stream()
        s0.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s0):
            iteration_inplace()  # warm the capture stream
        torch.cuda.current_stream().wait_stream(s0)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        L.dmprof_enable(1)  # the captured marks are entry 0 of the event table
        launches_c0 = L.dmprof_launches()
        with torch.cuda.graph(graph):
            iteration_inplace()
        launches_per_step = L.dmprof_launches() - launches_c0
    except Exception as exc:  # plain stream launches if capture is not possible
        print(f"CUDA graph capture failed ({exc}); timing stream launches", file=sys.stderr)
        graph = None
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = L.dmprof_launches()
    barrier(world)
    torch.cuda.synchronize()
    l1_total = l2_total = 0.0
    l_calls = 0
    ms1, ms2, calls = ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.fill_(float(k))
            if graph is None:
                L.dmprof_enable(1)
            ev[k][0].record()
            if graph is not None:
                graph.replay()
            else:
                iteration_async()
            ev[k][1].record()
            # star-kernel times of this step (outside the step's events)
            torch.cuda.synchronize()
            L.dmprof_read(ms1, ms2, calls)
            l1_total += ms1.value
            l2_total += ms2.value
            l_calls += calls.value
        torch.cuda.synchronize()
    L.dmprof_enable(0)
    barrier(world)
    launches = (launches_per_step * args.steps if graph is not None
                else L.dmprof_launches() - launches0)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    c = eng.counters_host()
    flags = int(sticky.item())
    if flags:
        raise RuntimeError(f"device flags {flags:#x} during the timed iterations")
    n_cells = int(c[N.CNT_CELLS])
    max_ms = reduce_max(total_ms, world, "nccl")
    value = replica_rate(n * args.steps, world, max_ms)

    # roofline of the dominant work, the star kernels of dm_delaunay (levels 1
    # and 2 together build one triangulation; 98 % of the device time):
    # algorithmic bytes per triangulation = points read (16 B each) + cells
    # written (16 B each) + candidate grid reads (4 B per point for the sorted
    # ids and 8 B per cell range), i.e. 16 n + 16 T + 4 n + 8 n_cells_grid
    # ~ 16 T + 28 n
    l1_ms = l1_total / max(l_calls, 1)
    l2_ms = l2_total / max(l_calls, 1)
    alg_bytes = 16 * n_cells + 28 * n
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / ((l1_ms + l2_ms) / 1000.0) / 1e9
    it_roof = iteration_roofline(n, n_cells, int(c[N.CNT_EDGES]), max_ms / args.steps, peak)

    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pts, cells = sm.generate_mesh(ball, H, verbose=0)
        t1 = time.perf_counter()
        pts2, cells2 = sm.sliver_removal(pts, ball, H, verbose=0)
        t2 = time.perf_counter()
        gen_s, sliver_s = t1 - t0, t2 - t1
        gen_max_s = reduce_max(gen_s, world, "nccl")
        e2e = {
            "value": replica_rate(n * 49, world, 1000.0 * gen_max_s),
            "unit": "point-iterations/s",
            "h2d_bytes_per_step": int(n * 16 / 49),
            "d2h_bytes_per_step": int((pts.nbytes + cells.nbytes) / 49),
            "time_to_mesh_s": gen_s + sliver_s,
            "generate_mesh_s": gen_s,
            "sliver_removal_s": sliver_s,
            "final_points": int(len(pts2)),
            "final_cells": int(len(cells2)),
        }
        # final quality from the library's own dihedral kernel
        dh = np.degrees(sm.geometry.calc_dihedral_angles(pts2, cells2)).reshape(-1, 6).min(1)
        e2e["min_dihedral_deg"] = float(dh.min())
        e2e["mean_min_dihedral_deg"] = float(dh.mean())

    salt = None
    if not args.no_salt:
        salt = salt_bench(measured_peaks_all())
    layered = None
    if not args.no_layered:
        layered = layered_bench()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ncpu, dt, _, tri_name = cpu_sample(1, 0)
        info = host_info()
        cpu = {
            "value": ncpu / dt, "unit": "point-iterations/s", "cores": 1, "kind": "port",
            "sample": f"1 DistMesh iteration of the h=0.02 unit ball ({ncpu} points) from the initial "
                      "lattice: float64 numpy restatement of the reference loop, triangulated by "
                      f"{tri_name}, serial; host {info['nproc']} cores, {info['cpu_model']}",
        }
    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "point-iterations/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": max_ms / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 (positions on a 2^-24-relative grid, forces); exact 64/128/192-bit integer predicates",
            "data": "synthetic (initial lattice of the unit ball, seeded decimation)",
            "config": {
                "workload": "3D unit ball, h=0.02, DistMesh iterations after 'warmup' iterations from the initial lattice",
                "n_points": n,
                "n_cells": n_cells,
                "l2": "256 MB buffer written between timed steps",
                "parallelism": f"replicas x{world}",
            },
            "roofline": {
                "bound": "hbm",
                "kernel": "k_star3_l1 + k_star3_l2 (vertex-star Delaunay, levels 1 and 2)",
                "achieved": achieved,
                "peak": peak,
                "peak_kind": peak_kind,
                "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": measured_traffic(),
                "alg_bytes_per_launch": alg_bytes,
                "avg_launch_ms": l1_ms + l2_ms,
                "level1_ms": l1_ms,
                "level2_ms": l2_ms,
            },
            "roofline_iteration": it_roof,
            "delaunay": {"stars_per_s": n / ((l1_ms + l2_ms) / 1000.0),
                         "level1_ms": l1_ms, "level2_ms": l2_ms},
            "phases_ms": {"step_ms_min": min(step_ms), "step_ms_max": max(step_ms)},
            "gpu_launches": int(launches),
            "clocks": clocks.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
            "neural_vs_exact": salt,
            "layered_2d": layered,
        }
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
SALT = {"hmin": 50.0, "wl": 10, "freq": 6.0, "grade": 0.15}
MLP_FLOPS_PER_QUERY = 2 * 128 * (64 + 3 * 128) + 2 * 128  # the four MMA layers + output dot


def salt_bench(peaks):
    """The synthetic 3D salt body (676 x 676 x 210 velocity grid at 20 m;
    its salt isosurface is the domain): time-to-mesh with the exact
    isosurface SDF and with the neural SDF (exact inside the band and for the
    final projection), both generate_mesh + sliver_removal at equal final
    quality; plus the MLP tensor-core inference throughput against the bf16
    peak and the exact SDF's query throughput."""
    import contextlib

    import torch

    import seismicmesh_gb300 as sm
    from seismicmesh_gb300 import synthetic as S

    def tick():
        torch.cuda.synchronize()
        return time.perf_counter()

    out = {"workload": "synthetic 3D salt body: velocity grid 210 x 676 x 676 (20 m nominal), "
                       "salt = 0.5 level set of 8 seeded Gaussian bumps; sizing wl=10 at 6 Hz, "
                       "hmin=50 m, grade 0.15; domain = the salt body"}
    with contextlib.redirect_stdout(sys.stderr):
        t0 = tick()
        vp, B, bbox = S.salt_model_3d()
        t1 = tick()
        ef = sm.get_sizing_function_from_segy(None, bbox, velocity_data=vp, nz=vp.shape[0],
                                              nx=vp.shape[1], ny=vp.shape[2], **SALT)
        t2 = tick()
        iso = sm.Isosurface(B, bbox, 0.5)
        t3 = tick()
        out.update(model_s=t1 - t0, sizing_s=t2 - t1, iso_build_s=t3 - t2, triangles=iso.ntri)
        t4 = tick()
        nn = sm.NeuralSDF(iso, SALT["hmin"])
        t5 = tick()
        out["mlp"] = {k: v for k, v in nn.stats.items() if k != "loss_per_epoch"}
        out["mlp"]["build_s"] = t5 - t4
        out["mlp"]["final_loss"] = nn.stats["loss_per_epoch"][-1]
        for name, dom in (("exact", iso), ("neural", nn)):
            ta = tick()
            p, c = sm.generate_mesh(dom, ef, verbose=0)
            tb = tick()
            p2, c2 = sm.sliver_removal(p, dom, ef, verbose=0)
            tc = tick()
            st = sm.geometry.quality_stats(p2, c2)
            out[name] = {
                "time_to_mesh_s": tc - ta, "generate_mesh_s": tb - ta, "sliver_removal_s": tc - tb,
                "point_iterations_per_s": len(p) * 49 / (tb - ta),
                "n_points": int(len(p2)), "n_cells": int(len(c2)),
                "min_dihedral_deg": st["min_dihedral"], "mean_min_dihedral_deg": st["avg_dihedral"],
                "mean_quality": st["avg_quality"], "min_quality": st["min_quality"],
            }
        out["speedup_time_to_mesh"] = out["exact"]["time_to_mesh_s"] / out["neural"]["time_to_mesh_s"]
        out["speedup_incl_training"] = out["exact"]["time_to_mesh_s"] / (
            out["neural"]["time_to_mesh_s"] + out["mlp"]["build_s"])
        # query throughput on 4M points uniform in the box
        n = 1 << 22
        g = torch.Generator(device="cuda")
        g.manual_seed(3)
        lo = torch.tensor(bbox[0::2], dtype=torch.float32, device="cuda")
        hi = torch.tensor(bbox[1::2], dtype=torch.float32, device="cuda")
        X = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        X[:, :3] = lo + (hi - lo) * torch.rand((n, 3), generator=g, device="cuda")
        d = torch.empty(n, dtype=torch.float32, device="cuda")
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

        def timed(fn, reps):
            fn()
            torch.cuda.synchronize()
            ev[0].record()
            for _ in range(reps):
                fn()
            ev[1].record()
            torch.cuda.synchronize()
            return ev[0].elapsed_time(ev[1]) / reps

        ms_mlp = timed(lambda: nn.mlp_eval_device(X, 4, n, d), 10)
        m1 = 1 << 20
        ms_exact = timed(lambda: iso.batched_eval(X, 4, m1, d), 1)
        ms_neural = timed(lambda: nn.batched_eval(X, 4, m1, d), 3)
        achieved = MLP_FLOPS_PER_QUERY * n / (ms_mlp / 1000.0) / 1e12
        out["mlp_roofline"] = {
            "bound": "tensor", "kernel": "k_mlp_infer_tc (tcgen05 BF16, FP32 accumulation in TMEM)",
            "achieved": achieved, "peak": peaks["bf16_tflops"], "peak_kind": peaks["kind"],
            "unit": "TFLOP/s", "frac": achieved / peaks["bf16_tflops"],
            "flops_per_query": MLP_FLOPS_PER_QUERY, "queries_per_launch": n,
            "avg_launch_ms": ms_mlp, "traffic": None,
        }
        out["sdf_queries_per_s"] = {
            "uniform_points": m1, "exact": m1 / (ms_exact / 1000.0),
            "neural_with_exact_band": m1 / (ms_neural / 1000.0),
            "network_only": n / (ms_mlp / 1000.0),
            "exact_fraction_in_band": int(nn._count.item()) / m1,
        }
    return out


def layered_bench():
    """The synthetic 2D layered model (1911 x 5395 cells): sizing build and
    generate_mesh on its Rectangle, time-to-mesh and point-iterations/s.  The
    reference loop's own time on this input, measured in the build container
    (reference loop + Qhull, one x86 core), is carried from
    tests/golden/layered2d.json for context; it is not timed here."""
    import contextlib

    import torch

    import seismicmesh_gb300 as sm
    from seismicmesh_gb300 import synthetic

    def tick():
        torch.cuda.synchronize()
        return time.perf_counter()

    vp, bbox = synthetic.layered_model_2d(0)
    with contextlib.redirect_stdout(sys.stderr):
        t0 = tick()
        ef = sm.get_sizing_function_from_segy(None, bbox, velocity_data=vp, nz=vp.shape[0],
                                              nx=vp.shape[1], hmin=75.0, wl=10, freq=2.0,
                                              grade=0.15)
        t1 = tick()
        p, t = sm.generate_mesh(sm.Rectangle(bbox), ef, verbose=0)
        t2 = tick()
    q = sm.geometry.simp_qual(p, t)
    out = {"workload": "2D layered model 1911 x 5395 (synthetic, seed 0), wl=10 at 2 Hz, "
                       "hmin=75 m, grade 0.15, Rectangle(bbox), max_iter 50",
           "sizing_s": t1 - t0, "generate_mesh_s": t2 - t1, "time_to_mesh_s": t2 - t0,
           "point_iterations_per_s": len(p) * 49 / (t2 - t1),
           "n_points": int(len(p)), "n_cells": int(len(t)),
           "min_quality": float(q.min()), "mean_quality": float(q.mean())}
    gpath = os.path.join(ROOT, "tests", "golden", "layered2d.json")
    if os.path.exists(gpath):
        with open(gpath) as f:
            g = json.load(f)
        out["reference_build_container"] = {
            "time_to_mesh_s": g["sizing_s"] + g["generate_mesh_s"], "n_points": g["n_points"],
            "mean_quality": g["mean_quality"],
            "how": "reference loop + Qhull, 1 x86 core, measured when the golden was made"}
    return out


def batch_bench(half):
    """The batched workload: 256 independent CSG domains (the first 128 2D,
    the rest 3D; vertex counts log-uniform over 2e3-2e5) meshed together by
    generate_meshes; half selects the 2D or 3D half.  point-iterations/s
    over the graph-captured iterations: the batch's points times the graph
    iterations over their wall time."""
    import torch

    from seismicmesh_gb300 import synthetic
    from seismicmesh_gb300.generation.batch import generate_meshes

    probs = synthetic.batch_domains(256)
    probs = probs[:128] if half == "2d" else probs[128:] if half == "3d" else probs
    st = {}
    t0 = time.perf_counter()
    out = generate_meshes(probs, stats=st)
    torch.cuda.synchronize()
    total = time.perf_counter() - t0
    pts = np.array(st["points"])
    n_graph = len(st["graph_ms"])
    return {
        "workload": f"batched CSG domains ({half}): {len(probs)} problems, seeds 0..255",
        "problems": len(probs), "meshed": sum(o is not None for o in out),
        "failed": st["failed"], "points": int(pts.sum()), "min_points": int(pts.min()),
        "max_points": int(pts.max()), "total_s": total, "setup_s": st["setup_s"],
        "checked_iterations_s": st["checked_s"], "graph_iterations_s": st["graph_iterations_s"],
        "termination_s": st["termination_s"], "graph_iterations": n_graph,
        "graph_ms_median": float(np.median(st["graph_ms"])) if n_graph else None,
        "point_iterations_per_s": float(pts.sum() * n_graph / st["graph_iterations_s"])
        if n_graph else None,
        "tuning": st["tuning"], "streams": st["streams"], "redone": st["redone"],
    }


PROFILE_L1 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                          "k_star3_l1_ball_h002.md")
PROFILE_L2 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                          "k_star3_l2_ball_h002.md")


def iteration_roofline(n, n_cells, n_edges, ms_per_step, peak, dim=3):
    """Roofline of a whole DistMesh iteration with the compulsory bytes of its
    per-iteration arrays (scalar sizing, no grid bytes): the cell table read
    twice (edge build and centroid filter), the unique edges written and
    read once, and the positions/forces passes,
        B_iter = 2 * 4 (d + 1) T + 2 * 8 E + 6 * 4 d N."""
    b_iter = 2 * 4 * (dim + 1) * n_cells + 2 * 8 * n_edges + 6 * 4 * dim * n
    achieved = b_iter / (ms_per_step / 1000.0) / 1e9
    return {
        "bound": "hbm",
        "scope": "one DistMesh iteration (graph replay)",
        "alg_bytes_per_iteration": b_iter,
        "bytes_per_point_iteration": b_iter / n,
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
    }


def measured_traffic():
    """DRAM bytes (read + write) of one k_star3_l1 and one k_star3_l2 launch
    from the committed ncu summaries of this workload (the lines
    'dram_bytes_per_launch: N'), or None"""
    total = 0
    for path in (PROFILE_L1, PROFILE_L2):
        try:
            vals = [int(line.split(":")[1].strip().replace(",", "")) for line in open(path)
                    if line.strip().startswith("dram_bytes_per_launch:")]
        except OSError:
            return None
        if not vals:
            return None
        total += vals[0]
    return total


def ncu_case(args):
    """Profiling cases (no timing, no JSON line).

    ball: the bench workload (3D unit ball, h = 0.02) for args.warmup
          iterations, then one more full iteration (triangulation, filter,
          adjacency, bar sums, update): the launches an ncu capture selects.
    mlp:  the salt body's network trained briefly, then dm_mlp_eval on 2^22
          points uniform in the box, args.warmup + 1 times.
    salt: the salt body with its exact isosurface SDF (h0 = hmin = 50 m) for
          args.warmup DistMesh iterations, then one more triangulation."""
    import torch

    import seismicmesh_gb300 as sm
    from seismicmesh_gb300.generation import mesh_generator as MG

    if args.ncu_case == "mlp":
        import contextlib

        from seismicmesh_gb300 import synthetic as S

        with contextlib.redirect_stdout(sys.stderr):
            vp, B, bbox = S.salt_model_3d()
            iso = sm.Isosurface(B, bbox, 0.5)
            nn = sm.NeuralSDF(iso, SALT["hmin"], n_samples=1 << 20, epochs=2, n_val=1 << 14)
        n = 1 << 22
        g = torch.Generator(device="cuda")
        g.manual_seed(3)
        lo = torch.tensor(bbox[0::2], dtype=torch.float32, device="cuda")
        hi = torch.tensor(bbox[1::2], dtype=torch.float32, device="cuda")
        X = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        X[:, :3] = lo + (hi - lo) * torch.rand((n, 3), generator=g, device="cuda")
        d = torch.empty(n, dtype=torch.float32, device="cuda")
        for _ in range(args.warmup + 1):
            nn.mlp_eval_device(X, 4, n, d)
        torch.cuda.synchronize()
        print("ncu case done:", n, "points", flush=True)
        return
    if args.ncu_case == "salt":
        import contextlib

        from seismicmesh_gb300 import synthetic as S

        with contextlib.redirect_stdout(sys.stderr):
            vp, B, bbox = S.salt_model_3d()
            ef = sm.get_sizing_function_from_segy(None, bbox, velocity_data=vp, nz=vp.shape[0],
                                                  nx=vp.shape[1], ny=vp.shape[2], **SALT)
            iso = sm.Isosurface(B, bbox, 0.5)
        h0 = SALT["hmin"]
        fd = MG._Domain(iso)
        sizing = MG._Sizing(ef, 3)
        opts = {"points": None, "r0m_is_h0": False, "seed": 0}
        p0 = MG._initialize_points(3, 0.1 * h0, np.array(bbox).reshape(-1, 2), sizing, fd, h0, opts,
                                   np.empty((0, 3)))
        eng = MG._Engine(3, p0, 0)
        deps = float(np.sqrt(np.finfo(float).eps) * h0)
        for _ in range(args.warmup):
            eng.triangulate()
            eng.filter(fd, 0.1 * h0)
            eng.build_adjacency()
            eng.step(sizing, [], 1.1, 0.30, h0, deps)
            eng.project_batched(fd)
        eng.triangulate()
        torch.cuda.synchronize()
        print("ncu case done:", eng.n, "points", int(eng.counters_host()[0]), "cells", flush=True)
        return
    ball = sm.Ball([0.0, 0.0, 0.0], 1.0)
    fd = MG._Domain(ball)
    sizing = MG._Sizing(H, 3)
    opts = {"points": None, "r0m_is_h0": False, "seed": 0}
    p0 = MG._initialize_points(3, 0.1 * H, np.array([[-1.0, 1.0]] * 3), sizing, fd, H, opts, np.empty((0, 3)))
    eng = MG._Engine(3, p0, 0)
    deps = float(np.sqrt(np.finfo(float).eps) * H)
    for _ in range(args.warmup + 1):
        eng.triangulate()
        eng.filter(fd, 0.1 * H)
        eng.build_adjacency()
        eng.step(sizing, [fd], 1 + 0.4 / 2**2, 0.30, H, deps)
    torch.cuda.synchronize()
    print("ncu case done:", eng.n, "points", int(eng.counters_host()[0]), "cells")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-salt", action="store_true",
                    help="skip the salt-body workload (neural vs exact SDF)")
    ap.add_argument("--no-layered", action="store_true",
                    help="skip the 2D layered-model workload")
    ap.add_argument("--batch-only", choices=["2d", "3d", "all"], default=None,
                    help="run only the batched workload (256 CSG domains, or its 2D or 3D half) "
                         "and print its JSON object")
    ap.add_argument("--salt-only", action="store_true",
                    help="run only the salt-body workload and print its JSON object")
    ap.add_argument("--ncu-case", choices=["ball", "mlp", "salt"], default=None,
                    help="profiling case: ball (the bench workload for --warmup iterations, then "
                         "one more), mlp (tensor-core inference on 2^22 points) or salt (the salt "
                         "body, exact SDF, --warmup iterations, then one triangulation); no "
                         "timing, no JSON line")
    args = ap.parse_args()
    if args.ncu_case:
        ncu_case(args)
        return
    if args.salt_only:
        print(json.dumps(salt_bench(measured_peaks_all())), flush=True)
        return
    if args.batch_only:
        print(json.dumps(batch_bench(args.batch_only)), flush=True)
        return
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    world, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
