"""Device plumbing: CUDA device selection, streams and buffer helpers.

PyTorch only provides device memory and streams here; every computation on
these buffers is a libdmgb.so kernel.
"""
import ctypes

import numpy as np
import torch


def device():
    if not torch.cuda.is_available():
        raise RuntimeError(
            "seismicmesh_gb300 needs a CUDA GPU: its kernels have no CPU implementation"
        )
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    """void* of a device tensor (None -> NULL)"""
    if t is None:
        return ctypes.c_void_p(0)
    return ctypes.c_void_p(t.data_ptr())


def to_points(p, dim=None):
    """host (n, dim) array -> device float32 [n, 4] (3D) or [n, 2] (2D)"""
    p = np.asarray(p)
    dim = dim or p.shape[1]
    n = p.shape[0]
    width = 4 if dim == 3 else 2
    host = np.zeros((n, width), dtype=np.float32)
    host[:, :dim] = p[:, :dim]
    return torch.from_numpy(host).to(device())


def from_points(P, dim):
    return P[:, :dim].double().cpu().numpy()


def empty(shape, dtype):
    return torch.empty(shape, dtype=dtype, device=device())


def zeros(shape, dtype):
    return torch.zeros(shape, dtype=dtype, device=device())


def workspace(nbytes):
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device())


def sync():
    torch.cuda.current_stream().synchronize()
