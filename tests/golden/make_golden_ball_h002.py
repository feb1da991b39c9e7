"""End metrics of the reference on the 3D unit ball at h = 0.02 (526,727
initial points, max_iter 50, seed 0, then sliver_removal with a 10 degree
bound), run through oracle/ref_harness.py in the build container:

    python tests/golden/make_golden_ball_h002.py           # about 30 min, 1 core
    python tests/golden/make_golden_ball_h002.py --jitter  # same, generic start
    python tests/golden/make_golden_ball_h002.py --cpp     # the C++ triangulator

Writes tests/golden/ball_h002.json (counts, dihedral and quality
statistics, volume, wall times).  With --jitter the run starts from the
same initial points moved by a seeded uniform jitter of +-1e-3 h (rounded
to float32; oracle/distmesh_np.py jittered_ball_points), where every
Delaunay triangulation of the run is unique, and writes
ball_h002_jitter.json.  With --cpp the 3D triangulations are the oracle's
exact-predicate C++ Delaunay (oracle/cdt3.cpp) instead of Qhull, and the run
writes ball_h002_cpp.json: the reference loop timed with the faster of the
two triangulation stubs, and a second exact-triangulation run whose ties are
broken differently from Qhull's.  The GPU tests compare the package's
generate_mesh + sliver_removal with these numbers.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import distmesh_np as O  # noqa: E402
from oracle import mesh_qa_np as QA  # noqa: E402
from oracle import ref_harness  # noqa: E402

SM = ref_harness.load()
from _fast_geometry import calc_dihedral_angles  # noqa: E402


def metrics(p, t):
    dh = np.degrees(np.asarray(calc_dihedral_angles(p, t)).reshape(-1, 6)).min(1)
    q, s = QA.cell_quality_vec(p, t)
    vol = float(np.abs(SM.geometry.simp_vol(p, t)).sum())
    return {
        "n_points": int(len(p)), "n_cells": int(len(t)),
        "min_dihedral_deg": float(dh.min()), "mean_min_dihedral_deg": float(dh.mean()),
        "min_quality": float(q.min()), "mean_quality": float(q.mean()),
        "mean_min_sin": float(s.mean()), "volume": vol,
    }


def main():
    h = 0.02
    jitter = "--jitter" in sys.argv
    cpp = "--cpp" in sys.argv
    if cpp:
        ref_harness.use_cpp_triangulator()
    ball = SM.Ball([0.0, 0.0, 0.0], 1.0)
    kw = {"points": O.jittered_ball_points(h)} if jitter else {}
    t0 = time.perf_counter()
    p, t = SM.generate_mesh(ball, h, max_iter=50, seed=0, verbose=0, **kw)
    t1 = time.perf_counter()
    m_gen = metrics(p, t)
    print("generate_mesh", t1 - t0, m_gen, flush=True)
    t2 = time.perf_counter()
    p2, t2c = SM.sliver_removal(p, ball, h, min_dh_angle_bound=10, verbose=0)
    t3 = time.perf_counter()
    m_sl = metrics(p2, t2c)
    print("sliver_removal", t3 - t2, m_sl, flush=True)
    out = {
        "workload": "3D unit ball, h=0.02, max_iter 50, seed 0, sliver_removal(min_dh_angle_bound=10)"
                    + (", initial points jittered by U(-1e-3 h, 1e-3 h), seed 0" if jitter else ""),
        "engine": "reference loop (SeismicMesh generation/mesh_generator.py) with "
                  + ("the oracle's exact-predicate C++ Delaunay (oracle/cdt3.cpp)" if cpp else "Qhull")
                  + " standing in for CGAL",
        "generate_mesh": m_gen, "sliver_removal": m_sl,
        "generate_mesh_s": t1 - t0, "sliver_removal_s": t3 - t2,
    }
    name = "ball_h002" + ("_jitter" if jitter else "") + ("_cpp" if cpp else "") + ".json"
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", name)


if __name__ == "__main__":
    main()
