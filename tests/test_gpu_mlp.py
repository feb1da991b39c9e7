"""The MLP kernels against the float64 oracle (oracle/iso_np.py).

* dm_mlp_forward_backward: every gradient within 1e-4 of the largest
  gradient of its layer (FP32 sums over the batch against float64).
* dm_mlp_eval (tcgen05, BF16 operands, FP32 accumulation in tensor memory):
  against the oracle's forward with the same BF16 roundings, the median
  error within 1e-5 of the output scale and the largest within 5e-3 (a
  value on a rounding tie can round to the neighbouring BF16 value: one
  BF16 step is 2^-8 relative); within 2e-2 of the FP32 forward.
* A short training run lowers the loss, and the kernel's waits all ended in
  time (dm_mlp_eval_status).
"""
import numpy as np
import pytest
import torch

from oracle import iso_np as I
from seismicmesh_gb300 import _device as D
from seismicmesh_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _mlp(seed=0, sigma=2.0, scale=0.3):
    rng = np.random.default_rng(seed)
    m = N.Mlp()
    freq = rng.normal(0, sigma, size=96).astype(np.float32)
    for i, v in enumerate(freq):
        m.freq[i] = float(v)
    center = np.array([0.1, -0.2, 0.3], dtype=np.float32)
    for k in range(3):
        m.center[k] = float(center[k])
    m.inv_scale = 0.8
    m.out_scale = 2.0
    params = np.zeros(N.MLP_NPARAMS, dtype=np.float32)
    off = 0
    for fan in (64, 128, 128, 128):
        params[off:off + 128 * fan] = rng.normal(0, np.sqrt(2.0 / fan), 128 * fan)
        params[off + 128 * fan:off + 128 * fan + 128] = rng.normal(0, 0.05, 128)
        off += 128 * fan + 128
    params[off:off + 128] = rng.normal(0, scale, 128)
    params[off + 128] = 0.1
    P = torch.from_numpy(params).cuda()
    W = torch.empty(N.MLP_NBF16, dtype=torch.int16, device="cuda")
    m.params = P.data_ptr()
    m.wbf16 = W.data_ptr()
    N.call("dm_mlp_to_bf16", D.ptr(P), D.ptr(W), D.stream_ptr())
    return m, params, freq, center, (P, W)


def _points(n, seed=1):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 4), dtype=np.float32)
    x[:, :3] = rng.uniform(-1.2, 1.2, size=(n, 3))
    return x


def test_gradients_match_float64_oracle(cuda):
    m, params, freq, center, keep = _mlp()
    B = 256
    x = _points(B)
    t = np.random.default_rng(2).normal(0, 0.5, B).astype(np.float32)
    ws = N.c_sz(0)
    N.call("dm_mlp_train_workspace_size", B, ws)
    w = D.workspace(ws.value)
    g = torch.zeros(N.MLP_NPARAMS, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    X, T = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    N.call("dm_mlp_forward_backward", m, D.ptr(X), D.ptr(T), None, B, D.ptr(g), D.ptr(loss),
           D.ptr(w), w.numel(), D.stream_ptr())
    gr, lr = I.mlp_grad(params.astype(np.float64), x, t, freq, center, 0.8)
    gg = g.double().cpu().numpy()
    assert abs(float(loss.item()) - lr) <= 1e-5 * max(1.0, lr)
    bounds = [(I.OFF_W[l], I.OFF_W[l] + 128 * I.KDIM[l]) for l in range(4)]
    bounds += [(I.OFF_W[l] + 128 * I.KDIM[l], I.OFF_W[l] + 128 * I.KDIM[l] + 128) for l in range(4)]
    bounds += [(I.OFF_W5, I.OFF_W5 + 128), (I.OFF_B5, I.OFF_B5 + 1)]
    for a, b in bounds:
        scale = np.abs(gr[a:b]).max()
        assert np.abs(gg[a:b] - gr[a:b]).max() <= 1e-4 * scale + 1e-9, (a, b)


def test_tensor_core_inference_matches_bf16_oracle(cuda):
    m, params, freq, center, keep = _mlp(seed=3)
    for n in (1, 127, 128, 1000, 40000):
        x = _points(n, seed=n)
        X = torch.from_numpy(x).cuda()
        d = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        N.call("dm_mlp_eval", m, D.ptr(X), 4, n, D.ptr(d), D.stream_ptr())
        st = N.c_int(-1)
        N.call("dm_mlp_eval_status", st, D.stream_ptr())
        assert st.value == 0
        got = d.double().cpu().numpy()
        ref = 2.0 * I.mlp_forward_bf16(params.astype(np.float64), x, freq, center, 0.8)
        ref32 = 2.0 * I.mlp_forward(params.astype(np.float64), x, freq, center, 0.8)[0]
        scale = max(np.abs(ref32).max(), 1e-3)
        assert np.all(np.isfinite(got))
        err = np.abs(got - ref)
        assert np.median(err) <= 1e-5 * scale, (n, np.median(err), scale)
        assert err.max() <= 5e-3 * scale, (n, err.max(), scale)
        assert np.abs(got - ref32).max() <= 2e-2 * scale
    # a strided point array (float[n][3], the centroid layout)
    x3 = np.ascontiguousarray(_points(500, seed=9)[:, :3])
    d3 = torch.empty(500, dtype=torch.float32, device="cuda")
    N.call("dm_mlp_eval", m, D.ptr(torch.from_numpy(x3).cuda()), 3, 500, D.ptr(d3), D.stream_ptr())
    ref3 = 2.0 * I.mlp_forward_bf16(params.astype(np.float64), x3, freq, center, 0.8)
    assert np.abs(d3.double().cpu().numpy() - ref3).max() <= 5e-3 * max(np.abs(ref3).max(), 1e-3)


def test_fp32_eval_matches_oracle(cuda):
    m, params, freq, center, keep = _mlp(seed=5)
    n = 20000
    x = _points(n, seed=7)
    X = torch.from_numpy(x).cuda()
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    ws = N.c_sz(0)
    N.call("dm_mlp_train_workspace_size", 16384, ws)
    w = D.workspace(ws.value)
    N.call("dm_mlp_eval_fp32", m, D.ptr(X), 4, n, D.ptr(d), D.ptr(w), w.numel(), D.stream_ptr())
    ref = 2.0 * I.mlp_forward(params.astype(np.float64), x, freq, center, 0.8)[0]
    assert np.abs(d.double().cpu().numpy() - ref).max() <= 1e-4 * np.abs(ref).max()


def test_training_lowers_the_loss(cuda):
    """fit sin(3 x0) cos(2 x1) + x2 on random points for 300 Adam steps"""
    m, params, freq, center, keep = _mlp(seed=8, scale=0.01)
    P, W = keep
    B = 4096
    ws = N.c_sz(0)
    N.call("dm_mlp_train_workspace_size", B, ws)
    w = D.workspace(ws.value)
    g = torch.zeros(N.MLP_NPARAMS, dtype=torch.float32, device="cuda")
    m1, m2 = torch.zeros_like(g), torch.zeros_like(g)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    losses = []
    for step in range(1, 301):
        x = _points(B, seed=1000 + step)
        t = (np.sin(3 * x[:, 0]) * np.cos(2 * x[:, 1]) + x[:, 2]).astype(np.float32)
        X, T = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
        N.call("dm_mlp_forward_backward", m, D.ptr(X), D.ptr(T), None, B, D.ptr(g), D.ptr(loss),
               D.ptr(w), w.numel(), D.stream_ptr())
        N.call("dm_mlp_adam", D.ptr(P), D.ptr(g), D.ptr(m1), D.ptr(m2), N.MLP_NPARAMS, 1e-3,
               0.9, 0.999, 1e-8, step, D.stream_ptr())
        losses.append(float(loss.item()))
    assert np.mean(losses[-20:]) < 0.35 * np.mean(losses[:5]), (losses[:5], losses[-20:])
