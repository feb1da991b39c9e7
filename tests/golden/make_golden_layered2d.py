"""End metrics of the reference on the 2D synthetic layered velocity model
(1911 x 5395 cells, dz = 6.25 m, dx = 12.5 m; seismicmesh_gb300/synthetic.py
layered_model_2d, seed 0): sizing by wavelength at 10 points per wavelength
at 2 Hz, hmin 75 m, grade 0.15, on a Rectangle of the model's box;
generate_mesh with max_iter 50, seed 0.  Run through oracle/ref_harness.py
in the build container:

    python tests/golden/make_golden_layered2d.py

Writes tests/golden/layered2d.json (counts, quality statistics, area, the
size grid's range, wall times).
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_harness  # noqa: E402
from seismicmesh_gb300 import synthetic  # noqa: E402  (numpy only: the model's values)

SM = ref_harness.load()


def main():
    vp, bbox = synthetic.layered_model_2d(0)
    t0 = time.perf_counter()
    ef = SM.get_sizing_function_from_segy(None, bbox, velocity_data=vp, nz=vp.shape[0],
                                          nx=vp.shape[1], hmin=75.0, wl=10, freq=2.0, grade=0.15)
    t1 = time.perf_counter()
    rect = SM.Rectangle(bbox)
    p, t = SM.generate_mesh(rect, ef, max_iter=50, seed=0, verbose=0)
    t2 = time.perf_counter()
    q = SM.geometry.simp_qual(p, t)
    out = {
        "workload": "2D layered model 1911 x 5395 (synthetic, seed 0), wl=10 at 2 Hz, hmin=75, "
                    "grade=0.15, Rectangle(bbox), max_iter 50, seed 0",
        "engine": "reference loop (SeismicMesh generation/mesh_generator.py) with Qhull standing in for CGAL",
        "n_points": int(len(p)), "n_cells": int(len(t)),
        "min_quality": float(q.min()), "mean_quality": float(q.mean()),
        "quality_q001": float(np.quantile(q, 0.001)), "quality_q01": float(np.quantile(q, 0.01)),
        "area": float(np.abs(SM.geometry.simp_vol(p, t)).sum()),
        "size_min": float(np.min(ef.cell_size.values) if hasattr(ef.cell_size, "values") else 0.0),
        "sizing_s": t1 - t0, "generate_mesh_s": t2 - t1,
    }
    print(out, flush=True)
    with open(os.path.join(HERE, "layered2d.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
