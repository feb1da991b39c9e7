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


def test_cpu_triangulator_falls_back_to_qhull_and_says_so(monkeypatch):
    """the CPU loop's stub: the C++ triangulator when it builds; an
    iteration on which it fails (planted here, on the CPU) is triangulated
    by Qhull and the sample text reports it"""
    import numpy as np

    import bench
    from oracle import cdt

    if not cdt.available():
        pytest.skip("no C++ compiler for oracle/cdt3.cpp")
    p = np.random.default_rng(1).random((300, 3))
    tri, name = bench.cpu_triangulator()
    assert "C++" in str(name) and "Qhull" not in str(name)
    assert len(tri(p)) > 0

    def broken(_):
        raise RuntimeError("cdt3_delaunay failed (planted)")

    monkeypatch.setattr(cdt, "delaunay", broken)
    t = tri(p)
    from scipy.spatial import Delaunay

    assert np.array_equal(np.sort(t, 1), np.sort(Delaunay(p).simplices, 1))
    assert "Qhull on 1 iterations" in str(name)


def test_batch_stream_assignment_is_largest_first_least_loaded():
    """generate_meshes captures the problems on S streams: the largest first,
    each to the stream with the least work so far (host logic, no GPU)"""
    from seismicmesh_gb300.generation.batch import _assign

    sizes = [5, 100, 30, 30, 70, 1]
    a = _assign(sizes, 3)
    assert sorted(a) == list(range(len(sizes)))
    load = [0, 0, 0]
    for i, s in enumerate(sizes):
        load[a[i]] += s
    assert sorted(load) == [66, 70, 100]  # 100 | 70 | 30 + 30 + 5 + 1
    assert a[1] != a[4]  # the two largest go to different streams
    assert _assign([7], 4) == {0: 0}
