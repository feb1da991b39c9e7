"""Host-side helpers of bench.py (no GPU needed)."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def test_iteration_roofline_bytes():
    import bench

    r = bench.iteration_roofline(n=526727, n_cells=3120000, n_edges=3650000, ms_per_step=80.0,
                                 peak=6785.5)
    # 2*16*T + 16*E + 72*N for the 3D ball: about 196 MB, 373 B per point-iteration
    assert r["alg_bytes_per_iteration"] == 32 * 3120000 + 16 * 3650000 + 72 * 526727
    assert 370 < r["bytes_per_point_iteration"] < 376
    assert r["achieved"] == pytest.approx(r["alg_bytes_per_iteration"] / 0.080 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6785.5)


def test_measured_traffic_reads_both_profiles():
    import bench

    t = bench.measured_traffic()
    assert t is not None and t > 0
