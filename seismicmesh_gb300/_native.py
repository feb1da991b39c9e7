"""ctypes binding of libdmgb.so (C ABI in include/dmgb.h).

The CUDA library is the only compute path: if it cannot be loaded every
operation raises instead of falling back to the CPU.
"""
import ctypes
import os
import threading

from . import _build

_lock = threading.Lock()
_lib = None

c_int = ctypes.c_int32
c_i64 = ctypes.c_int64
c_f = ctypes.c_float
c_d = ctypes.c_double
c_p = ctypes.c_void_p
c_sz = ctypes.c_size_t

DM_OK = 0
DM_ERR_ARG = 1
DM_ERR_CUDA = 2
DM_ERR_CAPACITY = 3
DM_ERR_NOT_CONVERGED = 4
DM_ERR_DEGENERATE = 5
DM_ERR_WORKSPACE = 6
DM_NO_GRID = -1000

CNT_CELLS, CNT_ESCALATED, CNT_FLAGS, CNT_KEPT, CNT_EDGES, CNT_BAD, CNT_DUPS, CNT_AUX = range(8)
CNT_MAXDEG = 13
NCOUNTERS = 16

FLAG_CELL_OVERFLOW = 1
FLAG_STAR_OVERFLOW = 2
FLAG_SEED_FAILED = 4
FLAG_DUPLICATES = 8
FLAG_EXACT_OVERFLOW = 16
FLAG_ADJ_OVERFLOW = 32
FLAG_DIVERGED = 64
FLAG_NONFINITE = 128

SIZING_CONST, SIZING_GRID, SIZING_SLOTS = 0, 1, 2


class SdfProgram(ctypes.Structure):
    _fields_ = [("ops", c_p), ("params", c_p), ("n_ops", c_int), ("dim", c_int)]


class Sizing(ctypes.Structure):
    _fields_ = [
        ("kind", c_int),
        ("dim", c_int),
        ("h", c_f),
        ("grid", c_p),
        ("n", c_int * 3),
        ("lo", c_f * 3),
        ("hi", c_f * 3),
        ("slot_h", c_p),
    ]


class Iso(ctypes.Structure):
    """dm_iso: isosurface SDF of a gridded field (device pointers)"""
    _fields_ = [
        ("field", c_p),
        ("level", c_f),
        ("n", c_int * 3),
        ("origin", c_f * 3),
        ("h", c_f * 3),
        ("tris", c_p),
        ("ntri", c_i64),
        ("bstart", c_p),
        ("btri", c_p),
        ("bring", c_p),
        ("nb", c_int * 3),
        ("bsize", c_f * 3),
        ("rho", c_f),
        ("cf", c_int),
        ("ncb", c_int * 3),
        ("cocc", c_p),
        ("cring", c_p),
    ]


MLP_NFREQ = 32
MLP_NPARAMS = 128 * 64 + 128 + 3 * (128 * 128 + 128) + 128 + 1
MLP_NBF16 = 128 * 64 + 3 * 128 * 128


class Mlp(ctypes.Structure):
    """dm_mlp: Fourier-feature MLP SDF (params / wbf16 are device pointers)"""
    _fields_ = [
        ("freq", c_f * (MLP_NFREQ * 3)),
        ("center", c_f * 3),
        ("inv_scale", c_f),
        ("out_scale", c_f),
        ("params", c_p),
        ("wbf16", c_p),
    ]


_FP = ctypes.POINTER(c_f)

# name -> (restype, argtypes)
SIGNATURES = {
    "dm_version": (c_int, []),
    "dm_last_error": (ctypes.c_char_p, []),
    "dm_abi_count": (c_int, []),
    "dm_orient2": (c_int, [_FP, _FP, _FP]),
    "dm_orient3": (c_int, [_FP, _FP, _FP, _FP]),
    "dm_incircle_sos": (c_int, [_FP, _FP, _FP, _FP]),
    "dm_insphere_sos": (c_int, [_FP, _FP, _FP, _FP, _FP]),
    "dm_delaunay_workspace_size": (c_int, [c_int, c_i64, ctypes.POINTER(c_sz)]),
    "dm_delaunay": (c_int, [c_int, c_p, c_i64, c_p, c_i64, c_p, c_p, c_sz, c_p]),
    "dm_filter_cells_workspace_size": (c_int, [c_i64, ctypes.POINTER(c_sz)]),
    "dm_filter_cells": (
        c_int,
        [c_int, c_p, c_p, c_i64, ctypes.POINTER(SdfProgram), c_f, c_p, c_p, c_p, c_sz, c_p],
    ),
    "dm_cell_centroids": (c_int, [c_int, c_p, c_p, c_i64, c_p, c_p, c_p]),
    "dm_adjacency_workspace_size": (c_int, [c_int, c_i64, c_i64, ctypes.POINTER(c_sz)]),
    "dm_radius_edge_ratios": (c_int, [c_int, c_p, c_p, c_i64, c_p, c_p]),
    "dm_cell_quality": (c_int, [c_int, c_p, c_p, c_i64, c_p, c_p, c_p]),
    "dm_overlap_workspace_size": (c_int, [c_int, c_i64, c_i64, ctypes.POINTER(c_sz)]),
    "dm_overlap_pairs": (
        c_int,
        [c_int, c_p, c_i64, c_p, c_i64, c_p, c_i64, ctypes.POINTER(c_i64), c_p, c_sz, c_p],
    ),
    "dm_gradient_term_workspace_size": (c_int, [c_i64, ctypes.POINTER(c_sz)]),
    "dm_gradient_term": (
        c_int,
        [c_p, ctypes.POINTER(c_int), c_int, ctypes.POINTER(c_int), c_d, c_d, c_int, c_d, c_p,
         c_p, c_sz, c_p],
    ),
    "dm_adjacency": (c_int, [c_int, c_i64, c_p, c_i64, c_int, c_p, c_int, c_p, c_p, c_p, c_sz, c_p]),
    "dm_unique_edges_workspace_size": (c_int, [c_i64, c_i64, ctypes.POINTER(c_sz)]),
    "dm_unique_edges": (c_int, [c_p, c_i64, c_i64, c_p, ctypes.POINTER(c_i64), c_p, c_sz, c_p]),
    "dm_unique_edges_noalloc": (c_int, [c_p, c_i64, c_i64, c_p, ctypes.POINTER(c_i64), c_p]),
    "dm_bar_blocks": (c_int, [c_i64, ctypes.POINTER(c_int)]),
    "dm_bar_sums": (c_int, [c_int, c_p, c_i64, c_p, c_int, c_p, ctypes.POINTER(Sizing), c_p, c_p]),
    "dm_update_points": (
        c_int,
        [
            c_int, c_p, c_p, c_i64, c_p, c_int, c_p, ctypes.POINTER(Sizing), c_p,
            c_f, c_f, c_i64, ctypes.POINTER(SdfProgram), c_int, c_f, c_f, c_p, c_int, c_p,
        ],
    ),
    "dm_slot_midpoints": (c_int, [c_int, c_p, c_i64, c_p, c_int, c_p, c_p, c_p]),
    "dm_sdf_eval": (c_int, [ctypes.POINTER(SdfProgram), c_p, c_i64, c_int, c_p, c_p, c_p]),
    "dm_sizing_eval": (c_int, [ctypes.POINTER(Sizing), c_p, c_i64, c_int, c_p, c_p]),
    "dm_improve_level_set": (c_int, [c_int, c_p, c_p, c_i64, ctypes.POINTER(SdfProgram), c_f, c_p]),
    "dm_dihedral_angles": (c_int, [c_p, c_p, c_i64, c_p, c_p]),
    "dm_dihedral_angles_f64": (c_int, [c_p, c_p, c_i64, c_p, c_p]),
    "dm_circumsphere_grad": (c_int, [c_p, c_p, c_p, c_p, c_i64, c_p, c_p]),
    "dm_dihedral_flags": (c_int, [c_p, c_p, c_i64, c_int, c_f, c_f, c_p, c_p, c_p]),
    "dm_sliver_workspace_size": (c_int, [c_i64, ctypes.POINTER(c_sz)]),
    "dm_sliver_perturb": (c_int, [c_p, c_i64, c_p, c_i64, c_int, c_p, c_f, c_int, c_p, c_sz, c_p, c_p]),
    "dm_limgrad": (c_int, [ctypes.POINTER(c_int), c_d, c_d, c_int, c_p, c_p]),
    "dm_boundary_workspace_size": (c_int, [c_int, c_i64, c_i64, ctypes.POINTER(c_sz)]),
    "dm_boundary": (c_int, [c_int, c_i64, c_p, c_i64, c_int, c_p, c_p, c_i64, c_p, c_p, c_sz, c_p]),
    "dm_compact_workspace_size": (c_int, [c_i64, ctypes.POINTER(c_sz)]),
    "dm_compact_vertices": (
        c_int,
        [c_int, c_p, c_p, c_i64, c_p, c_i64, c_int, c_p, ctypes.POINTER(c_i64), c_p, c_sz, c_p],
    ),
    "dm_simplex_metrics": (c_int, [c_int, c_p, c_p, c_i64, c_p, c_p, c_p]),
    "dm_simplex_metrics_f64": (c_int, [c_int, c_p, c_p, c_i64, c_p, c_p, c_p]),
    "dm_size_from_velocity": (
        c_int,
        [c_p, c_i64, c_i64, c_p, c_d, c_d, c_d, c_d, c_d, c_d, c_d, c_d, c_d, c_d,
         c_int, c_p, ctypes.POINTER(c_int), c_p, c_sz, c_p],
    ),
    "dm_pad_grid": (
        c_int,
        [c_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_int),
         c_int, c_int, c_d, c_p, c_p],
    ),
    "dm_laplacian_workspace_size": (c_int, [c_i64, ctypes.POINTER(c_sz)]),
    "dm_iso_count": (c_int, [ctypes.POINTER(Iso), c_p, c_p, ctypes.POINTER(c_i64), c_p]),
    "dm_iso_emit": (c_int, [ctypes.POINTER(Iso), c_p, c_p, c_p]),
    "dm_iso_bucket_workspace_size": (c_int, [c_i64, c_i64, ctypes.POINTER(c_sz)]),
    "dm_iso_bucket": (c_int, [ctypes.POINTER(Iso), c_p, c_p, c_p, c_p, c_p, c_sz, c_p]),
    "dm_iso_eval": (c_int, [ctypes.POINTER(Iso), c_p, c_int, c_i64, c_p, c_p, c_p, c_p, c_p]),
    "dm_filter_cells_by_value": (c_int, [c_int, c_p, c_i64, c_p, c_f, c_p, c_p, c_p]),
    "dm_project_by_value": (c_int, [c_int, c_p, c_i64, c_p, c_p, c_int, c_p]),
    "dm_select_band": (c_int, [c_p, c_i64, c_f, c_f, c_p, c_p, c_p]),
    "dm_newton_by_value": (c_int, [c_int, c_p, c_p, c_i64, c_p, c_p, c_f, c_int, c_p]),
    "dm_mlp_train_workspace_size": (c_int, [c_i64, ctypes.POINTER(c_sz)]),
    "dm_mlp_forward_backward": (
        c_int, [ctypes.POINTER(Mlp), c_p, c_p, c_p, c_i64, c_p, c_p, c_p, c_sz, c_p]),
    "dm_mlp_adam": (c_int, [c_p, c_p, c_p, c_p, c_i64, c_f, c_f, c_f, c_f, c_int, c_p]),
    "dm_mlp_to_bf16": (c_int, [c_p, c_p, c_p]),
    "dm_mlp_eval_fp32": (c_int, [ctypes.POINTER(Mlp), c_p, c_int, c_i64, c_p, c_p, c_sz, c_p]),
    "dm_mlp_eval": (c_int, [ctypes.POINTER(Mlp), c_p, c_int, c_i64, c_p, c_p]),
    "dm_mlp_eval_status": (c_int, [ctypes.POINTER(c_int), c_p]),
    "dm_laplacian_smooth": (
        c_int,
        [c_p, c_i64, c_p, c_int, c_p, c_p, c_int, c_d, ctypes.POINTER(c_int), c_p, c_sz, c_p],
    ),
}


class NativeError(RuntimeError):
    def __init__(self, name, code, msg):
        super().__init__(f"{name} failed with status {code}: {msg}")
        self.code = code


def lib():
    """Load libdmgb.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.library_path()
        if not os.path.exists(path):
            _build.build_library()
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def call(name, *args):
    """Call an entry point and raise NativeError on a non-zero status."""
    L = lib()
    rc = getattr(L, name)(*args)
    if rc != DM_OK:
        msg = L.dm_last_error()
        raise NativeError(name, rc, msg.decode() if msg else "")
    return rc


def fptr(arr):
    """float* for a host numpy float32 array"""
    return arr.ctypes.data_as(_FP)
