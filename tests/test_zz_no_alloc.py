"""dm_unique_edges_noalloc (static library scratch) against dm_unique_edges
(caller workspace) on the same inputs.  Results are integer pairs: compared
exactly (tolerance 0).  Kept in the last-collected file so that it also runs
after every other GPU test has used the device."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 1 << 17
MAX_M = 1 << 19


def _with_workspace(E, m, n):
    import torch

    from seismicmesh_gb300 import _device as D
    from seismicmesh_gb300 import _native as N

    out = D.empty((max(m, 1), 2), torch.int32)
    ws = N.c_sz(0)
    N.call("dm_unique_edges_workspace_size", n, m, ws)
    w = D.workspace(ws.value)
    nout = N.c_i64(0)
    N.call("dm_unique_edges", D.ptr(E), m, n, D.ptr(out), nout, D.ptr(w), w.numel(), D.stream_ptr())
    return out[: nout.value].cpu().numpy()


def _no_alloc(E, m, n):
    import torch

    from seismicmesh_gb300 import _device as D
    from seismicmesh_gb300 import _native as N

    out = D.empty((max(m, 1), 2), torch.int32)
    torch.cuda.synchronize()
    nout = N.c_i64(-1)
    N.call("dm_unique_edges_noalloc", D.ptr(E), m, n, D.ptr(out), nout, D.stream_ptr())
    return out[: nout.value].cpu().numpy()


def _edges(rng, n, m):
    import torch

    from seismicmesh_gb300 import _device as D

    e = rng.integers(0, n, (m, 2)).astype(np.int32)
    return e, torch.from_numpy(e).to(D.device())


def test_no_alloc_matches_workspace_entry_two_calls_in_a_row(cuda):
    from seismicmesh_gb300 import _device as D
    from seismicmesh_gb300 import _native as N

    # first call on the device (address lookup) with m = 0
    nout = N.c_i64(-1)
    N.call("dm_unique_edges_noalloc", None, 0, 0, None, nout, D.stream_ptr())
    assert nout.value == 0
    rng = np.random.default_rng(2024)
    # a large call, then a smaller one: stale scratch from the first call must
    # not leak into the second
    for n, m in ((20000, 300000), (700, 9000)):
        e, E = _edges(rng, n, m)
        got = _no_alloc(E, m, n)
        want = _with_workspace(E, m, n)
        assert got.dtype == want.dtype == np.int32
        np.testing.assert_array_equal(got, want)
        np.testing.assert_array_equal(got, np.unique(np.sort(e, axis=1), axis=0))


def test_no_alloc_at_the_limits_and_beyond(cuda):
    from seismicmesh_gb300 import _device as D
    from seismicmesh_gb300 import _native as N

    rng = np.random.default_rng(7)
    e, E = _edges(rng, MAX_N, MAX_M)
    np.testing.assert_array_equal(_no_alloc(E, MAX_M, MAX_N), _with_workspace(E, MAX_M, MAX_N))
    for n, m in ((MAX_N + 1, 10), (10, MAX_M + 1)):
        nout = N.c_i64(-1)
        rc = N.lib().dm_unique_edges_noalloc(D.ptr(E), m, n, D.ptr(E), ctypes.byref(nout), D.stream_ptr())
        assert rc == N.DM_ERR_CAPACITY
        msg = N.lib().dm_last_error().decode()
        assert "131072" in msg and "524288" in msg, msg
        assert nout.value == -1
