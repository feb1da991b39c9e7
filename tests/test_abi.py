"""C-ABI checks that need no GPU: exports, host predicates, program encoding."""
import os
import random
import re
from fractions import Fraction as Fr

import numpy as np

from conftest import ROOT
from seismicmesh_gb300 import _native as N


def _declared():
    src = open(os.path.join(ROOT, "include", "dmgb.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(dm_\w+)\(", src, re.M)))


def test_library_loads_and_exports_every_declared_symbol():
    L = N.lib()
    names = _declared()
    assert len(names) >= 30
    for name in names:
        assert hasattr(L, name), name
        assert name in N.SIGNATURES, f"{name} has no ctypes signature"
    assert L.dm_abi_count() == len(names)
    assert L.dm_version() >= 10000


def test_diagnostic_header_matches_exports():
    """every dmdbg_* / dmprof_* export is declared in include/dmgb_diag.h and
    every declaration there is exported"""
    src = open(os.path.join(ROOT, "include", "dmgb_diag.h")).read()
    names = set(re.findall(r"^(?:int|int64_t)\s+(dm(?:dbg|prof)_\w+)\(", src, re.M))
    L = N.lib()
    assert len(names) >= 10
    for name in names:
        assert hasattr(L, name), name
    import subprocess

    from seismicmesh_gb300 import _build

    out = subprocess.run(["nm", "-D", "--defined-only", _build.library_path()], capture_output=True, text=True)
    if out.returncode == 0:
        exported = set(re.findall(r"\b(dm(?:dbg|prof)_\w+)\b", out.stdout))
        assert exported == names, exported ^ names


def test_unique_edges_rejects_negative_indices_before_device_work():
    import pytest

    from seismicmesh_gb300 import geometry

    with pytest.raises(ValueError, match="negative"):
        geometry.unique_edges(np.array([[0, 1], [-1, 2]], dtype=np.int32))


def test_error_reporting_on_bad_arguments():
    L = N.lib()
    nbytes = N.c_sz(0)
    assert L.dm_delaunay_workspace_size(3, 1000, nbytes) == N.DM_OK and nbytes.value > 0
    rc = L.dm_delaunay(4, None, 10, None, 0, None, None, 0, None)
    assert rc == N.DM_ERR_ARG
    assert b"dim" in L.dm_last_error()


def _F(x):
    return Fr(float(x))


def _det(M):
    if len(M) == 1:
        return M[0][0]
    return sum((-1) ** j * M[0][j] * _det([r[:j] + r[j + 1:] for r in M[1:]]) for j in range(len(M)) if M[0][j] != 0)


def _sgn(x):
    return (x > 0) - (x < 0)


def _insph_sos_ref(P):
    """sign of the lifted 5x5 determinant with lift perturbation eps^rank,
    rank by lexicographic order (largest first), in exact rationals"""
    a = P[0]
    rows = []
    for q in P[1:]:
        v = [_F(q[i]) - _F(a[i]) for i in range(3)]
        rows.append(v + [sum(x * x for x in v)])
    base = _det(rows)
    if base != 0:
        return _sgn(base)
    order = sorted(range(5), key=lambda i: tuple(float(x) for x in P[i]), reverse=True)
    eps = Fr(1, 10**40)
    delta = [0] * 5
    for r, i in enumerate(order):
        delta[i] = eps ** (r + 1)
    rows = []
    for k, q in enumerate(P[1:], 1):
        v = [_F(q[i]) - _F(a[i]) for i in range(3)]
        rows.append(v + [sum(x * x for x in v) + delta[k] - delta[0]])
    return _sgn(_det(rows))


def test_host_predicates_exact_against_rationals():
    L = N.lib()
    rng = random.Random(7)
    fp = N.fptr
    degenerate = 0
    for t in range(1500):
        if t % 3 == 0:
            P = [np.float32([rng.uniform(-1, 1) for _ in range(3)]) for _ in range(5)]
        elif t % 3 == 1:
            P = []
            for _ in range(5):
                v = np.array([rng.gauss(0, 1) for _ in range(3)])
                P.append(np.float32(0.3 + 0.02 * v / np.linalg.norm(v)))
        else:
            P = [np.float32([0.5 * rng.randint(-2, 2), 0.5 * rng.randint(-2, 2) + 0.25 * rng.randint(0, 1),
                             0.5 * rng.randint(-2, 2)]) for _ in range(5)]
        if len({tuple(p) for p in P}) < 5:
            continue
        o = _sgn(_det([[_F(q[i]) - _F(P[0][i]) for i in range(3)] for q in P[1:4]]))
        assert L.dm_orient3(*[fp(p) for p in P[:4]]) == o
        for k in (0, 1):  # exact and FP64-filtered stages alone
            assert L.dmdbg_host_pred(k, *[fp(p) for p in P[:4]], fp(P[4])) == o
        if o == 0:
            continue
        s = _insph_sos_ref(P)
        degenerate += 0
        assert L.dm_insphere_sos(*[fp(p) for p in P]) == s
    assert degenerate == 0


def test_fixed_point_predicates_match_expansion_predicates():
    """The integer (fixed-point) predicates used inside vertex stars give the
    same exact, symbolically perturbed signs as the expansion predicates."""
    import ctypes
    import math

    L = N.lib()
    fp = N.fptr
    f = L.dmdbg_fixed_pred
    f.argtypes = [ctypes.c_int, ctypes.c_int] + [N._FP] * 5
    rng = np.random.default_rng(11)
    checked = {0: 0, 1: 0, 2: 0, 3: 0}
    zeros = 0
    for t in range(3000):
        mode = t % 3
        if mode == 0:  # small lattice: coplanar and cospherical ties
            P = (0.3 + rng.integers(-3, 4, (5, 3)) * 0.0625).astype(np.float32)
        elif mode == 1:  # generic points near 0.5
            P = (0.5 + 0.05 * rng.standard_normal((5, 3))).astype(np.float32)
        else:  # rounded lattice: ties broken by float rounding
            P = (0.71 + rng.integers(-2, 3, (5, 3)) * 0.02).astype(np.float32)
        if len({tuple(q) for q in P}) < 5:
            continue
        rel = (P[1:] - P[0]).astype(np.float32)
        g = math.frexp(float(np.abs(rel).max()))[1] - 1 - 28
        o = L.dm_orient3(*[fp(q) for q in P[:4]])
        r = f(0, g, *[fp(q) for q in P])
        if r != -99:
            assert r == o
            checked[0] += 1
            zeros += o == 0
        if o != 0:
            r = f(1, g, *[fp(q) for q in P])
            if r != -99:
                assert r == L.dm_insphere_sos(*[fp(q) for q in P])
                checked[1] += 1
        Q = [np.ascontiguousarray(q[:2]) for q in P[:4]]
        o2 = L.dm_orient2(*[fp(q) for q in Q[:3]])
        r = f(2, g, *[fp(q) for q in Q], fp(Q[0]))
        if r != -99:
            assert r == o2
            checked[2] += 1
        if o2 != 0 and len({tuple(q) for q in Q}) == 4:
            r = f(3, g, *[fp(q) for q in Q], fp(Q[0]))
            if r != -99:
                assert r == L.dm_incircle_sos(*[fp(q) for q in Q])
                checked[3] += 1
    assert min(checked.values()) > 500, checked
    assert zeros > 20


def test_sdf_program_encoding():
    import seismicmesh_gb300 as sm

    d = sm.Difference([sm.Ball((0, 0, 0.5), 0.85), sm.Cube((-0.5, 0.5, -0.5, 0.5, -0.5, 0.5))], smoothness=0.2)
    prog = d.program()
    assert [op[0] for op in prog.ops] == [2, 4, 22]
    assert prog.ops[-1][2] == 2 and prog.params[prog.ops[-1][1]] == np.float32(0.2)
    r = sm.Rectangle((0.0, 1.0, 0.0, 1.0), rotate=[0.3, 0, 0], translate=[0.1, 0.2])
    op = r.program().ops[0]
    assert op[0] == 3 and op[3] == (1 | 2)  # translate + 2D rotation


def test_qa_entry_points_reject_bad_arguments():
    """argument checks of the mesh-QA entry points run before any device
    work: bad dimension, negative sizes, missing pointers, tiny workspace"""
    import ctypes

    L = N.lib()
    k = ctypes.c_int64(-1)
    assert L.dm_overlap_pairs(4, None, 10, None, 5, None, 0, ctypes.byref(k), None, 0, None) == N.DM_ERR_ARG
    assert b"dim" in L.dm_last_error()
    assert L.dm_overlap_pairs(2, None, 10, None, -1, None, 0, ctypes.byref(k), None, 0, None) == N.DM_ERR_ARG
    assert L.dm_overlap_pairs(3, None, 10, None, 5, None, 0, ctypes.byref(k), None, 0, None) == N.DM_ERR_ARG
    # no cells: nothing to do, no pairs
    assert L.dm_overlap_pairs(2, None, 0, None, 0, None, 0, ctypes.byref(k), None, 0, None) == N.DM_OK
    assert k.value == 0
    ws = N.c_sz(0)
    assert L.dm_overlap_workspace_size(3, 1000, 5000, ws) == N.DM_OK and ws.value > 0
    # a workspace below the size asked for is refused by name
    fake = ctypes.c_void_p(256)
    assert L.dm_overlap_pairs(3, fake, 1000, fake, 5000, fake, 10, ctypes.byref(k), fake, 16, None) \
        == N.DM_ERR_WORKSPACE
    assert b"workspace" in L.dm_last_error()
    assert L.dm_radius_edge_ratios(5, None, None, 3, None, None) == N.DM_ERR_ARG
    assert L.dm_radius_edge_ratios(2, None, None, 3, None, None) == N.DM_ERR_ARG
    assert L.dm_radius_edge_ratios(2, None, None, 0, None, None) == N.DM_OK
    assert L.dm_cell_quality(1, None, None, 3, None, None, None) == N.DM_ERR_ARG
    assert L.dm_cell_quality(3, None, None, 3, None, None, None) == N.DM_ERR_ARG
    assert L.dm_cell_quality(3, None, None, 0, None, None, None) == N.DM_OK


def test_qa_python_wrappers_check_shapes():
    import pytest

    from seismicmesh_gb300 import geometry as G

    with pytest.raises(ValueError):
        G.do_any_overlap(np.zeros((4, 2)), np.zeros((2, 4), dtype=int), dim=2)
    with pytest.raises(ValueError):
        G.calc_re_ratios(np.zeros((4, 2)), np.zeros((2, 3), dtype=int), dim=4)
    with pytest.raises(ValueError):
        G.cell_quality(np.zeros((4, 4)), np.zeros((2, 5), dtype=int))
    # empty meshes need no device
    assert G.do_any_overlap(np.zeros((0, 2)), np.zeros((0, 3), dtype=int), dim=2) == []
    assert len(G.calc_re_ratios(np.zeros((0, 3)), np.zeros((0, 4), dtype=int), dim=3)) == 0
