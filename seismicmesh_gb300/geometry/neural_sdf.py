"""A learned stand-in for an expensive signed distance function.

`NeuralSDF` fits a Fourier-feature MLP (3 -> 64 features -> 128 x 4 -> 1,
ReLU) to an exact SDF (e.g. `Isosurface`) on samples the exact SDF labels,
training on the GPU with the library's own forward, backward and Adam
kernels (dm_mlp_forward_backward, dm_mlp_adam, FP32).  Inference runs on the
tensor cores (dm_mlp_eval: BF16 weights and activations, FP32 accumulation
in tensor memory).  Distances are clamped to +-clamp during training, so the
network answers "how far, up to clamp" and the sign.

The exact SDF decides near the boundary: wherever the network's
value lies within `band` = 2 hmin + margin * (largest error measured on
held-out samples) of the surface, and everywhere a point may lie outside
(where DistMesh projects it), the exact distance replaces it.  Decisions
the DistMesh loop takes far from the boundary (keep a cell, leave a point
alone) only need the sign, which the bound makes certain on the measured
samples.
"""
import math
import time

import numpy as np
import torch

from .. import _device as D
from .. import _native as N

__all__ = ["NeuralSDF"]


class NeuralSDF:
    """MLP fit of `exact` (an object with batched_eval / bbox) for meshes with
    minimum edge length hmin."""

    def __init__(self, exact, hmin, clamp=None, n_samples=4_000_000, batch=16384, epochs=60,
                 lr=5e-3, sigma=1.5, near_fraction=0.5, near_scale=None, weight_alpha=3.0,
                 seed=0, margin=1.5, n_val=1 << 18, samples=None, val_samples=None,
                 verbose=False):
        self.exact = exact
        self.dim = 3
        self.bbox = tuple(exact.bbox)
        self.corners = None
        self.hmin = float(hmin)
        self.clamp = float(clamp if clamp is not None else 20.0 * hmin)
        self.margin = float(margin)
        self.verbose = verbose
        lo = np.array(self.bbox[0::2], dtype=np.float64)
        hi = np.array(self.bbox[1::2], dtype=np.float64)
        self.lo, self.hi = lo, hi
        rng = np.random.default_rng(seed)
        self.gen = torch.Generator(device=D.device())
        self.gen.manual_seed(seed)
        m = N.Mlp()
        center = 0.5 * (lo + hi)
        for k in range(3):
            m.center[k] = float(center[k])
        m.inv_scale = float(1.0 / (0.5 * (hi - lo).max()))
        m.out_scale = self.clamp
        freq = rng.normal(0.0, sigma, size=(N.MLP_NFREQ, 3)).astype(np.float32)
        for i, v in enumerate(freq.ravel()):
            m.freq[i] = float(v)
        self.freq = freq
        self.params = torch.from_numpy(self._init_params(rng)).to(D.device())
        self.wbf16 = D.empty((N.MLP_NBF16,), torch.int16)
        m.params = self.params.data_ptr()
        m.wbf16 = self.wbf16.data_ptr()
        self.struct = m
        self.stats = {}
        self._idx = None
        self._count = D.zeros((1,), torch.int64)
        near_scale = near_scale if near_scale is not None else 8.0 * hmin
        t0 = time.perf_counter()
        if samples is None:
            samples = self.make_samples(n_samples, near_fraction, near_scale)
        torch.cuda.synchronize()
        self.stats["samples_s"] = time.perf_counter() - t0
        self.train(samples, batch, epochs, lr, weight_alpha)
        if val_samples is None:
            val_samples = self.make_samples(n_val, 0.5, near_scale)
        self.validate(val_samples)

    # ------------------------------------------------------------------
    @staticmethod
    def _init_params(rng):
        """He-normal weights for the ReLU layers, zero biases, a small output
        layer"""
        p = np.zeros(N.MLP_NPARAMS, dtype=np.float32)
        off = 0
        for fan_in in (64, 128, 128, 128):
            w = rng.normal(0.0, math.sqrt(2.0 / fan_in), size=(128, fan_in))
            p[off:off + w.size] = w.ravel()
            off += w.size + 128
        p[off:off + 128] = rng.normal(0.0, math.sqrt(1.0 / 128), size=128)
        return p

    def make_samples(self, n, near_fraction, near_scale):
        """n points (float[n][4]) : a share near the surface (a random point
        of a random triangle plus a Gaussian offset), the rest uniform in the
        box; and their exact distances"""
        dev = D.device()
        nn = int(n * near_fraction)
        lo = torch.tensor(self.lo, dtype=torch.float32, device=dev)
        hi = torch.tensor(self.hi, dtype=torch.float32, device=dev)
        X = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        X[nn:, :3] = lo + (hi - lo) * torch.rand((n - nn, 3), generator=self.gen, device=dev)
        tris = getattr(self.exact, "tris", None)
        ntri = getattr(self.exact, "ntri", 0)
        if nn and ntri:
            t = torch.randint(0, ntri, (nn,), generator=self.gen, device=dev)
            r1 = torch.rand((nn, 1), generator=self.gen, device=dev).sqrt()
            r2 = torch.rand((nn, 1), generator=self.gen, device=dev)
            a, b, c = tris[t, 0, :3], tris[t, 1, :3], tris[t, 2, :3]
            p = (1 - r1) * a + r1 * (1 - r2) * b + r1 * r2 * c
            p = p + near_scale * torch.randn((nn, 3), generator=self.gen, device=dev)
            X[:nn, :3] = torch.maximum(torch.minimum(p, hi), lo)
        elif nn:
            X[:nn, :3] = lo + (hi - lo) * torch.rand((nn, 3), generator=self.gen, device=dev)
        d = D.empty((n,), torch.float32)
        self.exact.batched_eval(X, 4, n, d)
        return X, d

    def train(self, samples, batch, epochs, lr, weight_alpha=0.0):
        """Adam on MSE against the clamped exact distances (in units of the
        clamp), optionally weighted by 1 + alpha exp(-|d| / (4 hmin))"""
        X, d = samples
        n_samples = len(d)
        t1 = time.perf_counter()
        target = torch.clamp(d, -self.clamp, self.clamp) / self.clamp
        weight = None
        if weight_alpha:
            weight = 1.0 + weight_alpha * torch.exp(-d.abs() / (4.0 * self.hmin))
        npar = N.MLP_NPARAMS
        grads = D.zeros((npar,), torch.float32)
        m1 = D.zeros((npar,), torch.float32)
        m2 = D.zeros((npar,), torch.float32)
        loss = D.zeros((1,), torch.float32)
        ws = N.c_sz(0)
        N.call("dm_mlp_train_workspace_size", batch, ws)
        w = D.workspace(ws.value)
        steps_per_epoch = n_samples // batch
        total = steps_per_epoch * epochs
        step = 0
        losses = []
        for ep in range(epochs):
            perm = torch.randperm(n_samples, generator=self.gen, device=D.device())
            for s in range(steps_per_epoch):
                sel = perm[s * batch:(s + 1) * batch]
                xb = X[sel]
                tb = target[sel]
                wb = weight[sel] if weight is not None else None
                N.call("dm_mlp_forward_backward", self.struct, D.ptr(xb), D.ptr(tb), D.ptr(wb),
                       batch, D.ptr(grads), D.ptr(loss), D.ptr(w), w.numel(), D.stream_ptr())
                step += 1
                # cosine decay to 1 % of lr
                lr_t = lr * (0.01 + 0.99 * 0.5 * (1 + math.cos(math.pi * step / total)))
                N.call("dm_mlp_adam", D.ptr(self.params), D.ptr(grads), D.ptr(m1), D.ptr(m2),
                       npar, lr_t, 0.9, 0.999, 1e-8, step, D.stream_ptr())
            losses.append(float(loss.item()))
            if self.verbose:
                print(f"epoch {ep}: loss {losses[-1]:.3e}", flush=True)
        N.call("dm_mlp_to_bf16", D.ptr(self.params), D.ptr(self.wbf16), D.stream_ptr())
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        self.stats.update(train_s=t2 - t1, steps=step, epochs=epochs, batch=batch,
                          n_samples=n_samples, loss_per_epoch=losses, lr=lr,
                          weight_alpha=weight_alpha)

    def validate(self, samples):
        """largest |network - clamp(exact)| on held-out samples, with the
        tensor-core inference; sets band (infinite when the network cannot
        separate anything from the band: every value is then exact)"""
        X, d = samples
        n = len(d)
        y = D.empty((n,), torch.float32)
        self.mlp_eval_device(X, 4, n, y)
        ref = torch.clamp(d, -self.clamp, self.clamp)
        err = (y - ref).abs()
        near = d.abs() < 2 * self.hmin
        self.max_error = float(err.max().item())
        self.band = 2 * self.hmin + self.margin * self.max_error
        if self.band >= self.clamp:
            self.band = float("inf")
        sign_ok = ((y > 0) == (d > 0)) | (d.abs() < self.band)
        self.stats.update(
            max_abs_error=self.max_error,
            rms_error=float(err.pow(2).mean().sqrt().item()),
            max_abs_error_near=float(err[near].max().item()) if bool(near.any()) else 0.0,
            band=self.band, n_val=n, clamp=self.clamp,
            sign_agreement_outside_band=float(sign_ok.float().mean().item()),
        )

    # ------------------------------------------------------------------
    def mlp_eval_device(self, pts, stride, n, d):
        """network value (tensor cores) of float[n][stride] device points"""
        if n:
            N.call("dm_mlp_eval", self.struct, D.ptr(pts), stride, n, D.ptr(d), D.stream_ptr())

    def mlp_eval_fp32_device(self, pts, stride, n, d):
        """network value with the FP32 training arithmetic"""
        ws = N.c_sz(0)
        N.call("dm_mlp_train_workspace_size", 16384, ws)
        w = D.workspace(ws.value)
        N.call("dm_mlp_eval_fp32", self.struct, D.ptr(pts), stride, n, D.ptr(d), D.ptr(w),
               w.numel(), D.stream_ptr())

    def batched_eval(self, pts, stride, n, d, grad=None, mode="cells", idx=None, count=None):
        """signed distances of device points: the network's value, replaced by
        the exact distance in the band (mode "cells": |value| < band) or
        wherever the point may be outside or near (mode "points":
        value > -band, the points DistMesh may project).  With idx the listed
        points are evaluated exactly."""
        if idx is not None:
            self.exact.batched_eval(pts, stride, n, d, grad, idx=idx, count=count)
            return
        if n == 0:
            return
        self.mlp_eval_device(pts, stride, n, d)
        if self._idx is None or self._idx.numel() < n:
            self._idx = D.empty((max(n, 1024),), torch.int32)
        hi = 3.0e38 if mode == "points" else self.band
        N.call("dm_select_band", D.ptr(d), n, -self.band, hi, D.ptr(self._idx), D.ptr(self._count),
               D.stream_ptr())
        self.exact.batched_eval(pts, stride, n, d, grad, idx=self._idx, count=self._count)

    def eval(self, x):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(-1, 3))
        n = len(x)
        P = torch.from_numpy(x).to(D.device())
        d = D.empty((max(n, 1),), torch.float32)
        self.batched_eval(P, 3, n, d, mode="cells")
        return d[:n].double().cpu().numpy()

    def eval_network(self, x, fp32=False):
        """the network alone (no exact band) at host points"""
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(-1, 3))
        n = len(x)
        P = torch.from_numpy(x).to(D.device())
        d = D.empty((max(n, 1),), torch.float32)
        if n:
            (self.mlp_eval_fp32_device if fp32 else self.mlp_eval_device)(P, 3, n, d)
        return d[:n].double().cpu().numpy()
