"""Mesh size functions from seismic velocity models, built on the GPU.

Drop-in for sizing/mesh_size_function.py of the reference:
get_sizing_function_from_segy (34-239) with the same keyword options and
defaults, read_velocity_model (590-606) and its binary / SEG-Y readers, and
write_velocity_model (242-335).  read_velocity_model_to_device streams a raw
binary model from disk into a device grid; get_sizing_function_from_segy
takes that path for binary files and accepts device tensors as
velocity_data.
The size grid is computed by dm_size_from_velocity (wavelength sizing,
clamp, Courant bound), dm_limgrad (gradation limiting) and dm_pad_grid
(domain pad); the resulting SizeFunction evaluates with dm_sizing_eval
(linear, extrapolating interpolation like RegularGridInterpolator with
bounds_error=False, fill_value=None).
"""
import os
import warnings

import numpy as np
import torch

from .. import _device as D
from .. import _native as N
from .size_function import SizeFunction

__all__ = [
    "get_sizing_function_from_segy",
    "write_velocity_model",
    "plot_sizing_function",
    "read_velocity_model",
    "read_velocity_model_to_device",
    "GridSizing",
]


class GridSizing:
    """Device-resident size grid with linear interpolation on the GPU.

    ``values`` (n0, n1[, n2]) on axes linspace(bbox[2k], bbox[2k+1], n_k);
    query columns are in the same axis order as the grid.
    """

    device_grid = True

    def __init__(self, values, bbox):
        v = np.asarray(values)
        self.dim = v.ndim
        self.shape = v.shape
        self.bbox = tuple(float(b) for b in bbox)
        self.values = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).to(D.device())
        self.grid = np.asarray(values)

    @classmethod
    def from_device(cls, values_dev, bbox):
        obj = cls.__new__(cls)
        obj.dim = values_dev.dim()
        obj.shape = tuple(values_dev.shape)
        obj.bbox = tuple(float(b) for b in bbox)
        obj.values = values_dev.float().contiguous()
        obj.grid = None
        return obj

    def fill_struct(self, s):
        s.kind = N.SIZING_GRID
        s.dim = self.dim
        s.grid = self.values.data_ptr()
        for k in range(3):
            s.n[k] = self.shape[k] if k < self.dim else 1
            s.lo[k] = self.bbox[2 * k] if k < self.dim else 0.0
            s.hi[k] = self.bbox[2 * k + 1] if k < self.dim else 1.0

    def __call__(self, x):
        if isinstance(x, tuple):
            x = np.column_stack([np.ravel(c) for c in x])
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(-1, self.dim))
        n = x.shape[0]
        s = N.Sizing()
        self.fill_struct(s)
        xd = torch.from_numpy(x).to(D.device())
        h = D.empty((n,), torch.float32)
        N.call("dm_sizing_eval", s, D.ptr(xd), n, self.dim, D.ptr(h), D.stream_ptr())
        return h.double().cpu().numpy()


def get_sizing_function_from_segy(filename, bbox, comm=None, **kwargs):
    r"""Build a mesh size function from a seismic velocity model (same
    keywords as the reference: velocity_data, vp_water, hmin, hmax, wl, freq,
    grad, grade, stencil_size, space_order, dt, cr_max, pad_style,
    domain_pad, units, nz, nx, ny, byte_order, axes_order, axes_order_sort,
    dtype).  Returns a SizeFunction whose grid lives on the GPU."""
    sz_opts = {
        "velocity_data": None,
        "vp_water": 1500.0,
        "hmin": 150.0,
        "hmax": 10000.0,
        "wl": 0,
        "freq": 2.0,
        "grad": 0.0,
        "grade": 0.0,
        "stencil_size": 10.0,
        "space_order": 1,
        "dt": 0.0,
        "cr_max": 1.0,
        "pad_style": "edge",
        "domain_pad": 0.0,
        "units": "m-s",
        "nz": None,
        "nx": None,
        "ny": None,
        "byte_order": "byte_order",
        "axes_order": (0, 1, 2),
        "axes_order_sort": "F",
        "dtype": "float32",
    }
    if comm is not None and getattr(comm, "size", 1) > 1:
        raise NotImplementedError("the GPU engine builds sizing functions on one GPU")
    sz_opts.update(kwargs)
    vp = sz_opts["velocity_data"]
    nz, nx, ny = sz_opts["nz"], sz_opts["nx"], sz_opts["ny"]
    owned = False  # vp is a device grid this call made (no defensive copy)
    if vp is None:
        reader = read_velocity_model if filename.endswith(".segy") else read_velocity_model_to_device
        vp, nz, nx, ny = reader(
            filename,
            nz=nz,
            nx=nx,
            ny=ny,
            byte_order=sz_opts["byte_order"],
            axes_order=sz_opts["axes_order"],
            axes_order_sort=sz_opts["axes_order_sort"],
            dtype=sz_opts["dtype"],
        )
        owned = isinstance(vp, torch.Tensor)
    scale = 1.0
    if sz_opts["units"] == "km-s":
        print("Converting from km-s to m-s...", flush=True)
        scale = 1000.0
    elif sz_opts["units"] == "ft-s":
        print("Converting from ft-s to m-s...", flush=True)
        scale = 0.30

    if len(bbox) == 4:
        dim = 2
    elif len(bbox) == 6:
        dim = 3
    else:
        raise ValueError("Dimension not supported")

    allowed = {
        "hmin", "hmax", "wl", "freq", "cr_max", "dt", "space_order", "grad", "grade",
        "stencil_size", "pad_style", "domain_pad", "units", "nz", "nx", "ny",
        "byte_order", "axes_order", "axes_order_sort", "dtype", "velocity_data", "vp_water",
    }
    for key in kwargs:
        if key not in allowed:
            raise ValueError("Option %s with parameter %s not recognized " % (key, kwargs[key]))

    if isinstance(vp, torch.Tensor):
        # a grid already in memory, on the device or not: used as FP64 on
        # the device (copied unless this call read it)
        vp_host = None
        vpd = vp.detach().to(device=D.device(), dtype=torch.float64, copy=not owned).contiguous()
    else:
        vp_host = np.ascontiguousarray(np.asarray(vp, dtype=np.float64))
        vpd = torch.from_numpy(vp_host).to(D.device())
    shape = tuple(vpd.shape)
    cell = torch.empty_like(vpd)
    if sz_opts["wl"] < 0:
        raise ValueError("Parameter `wl` must be set > 0")
    if sz_opts["freq"] < 0.0:
        raise ValueError("Parameter `freq` must be set > 0.0")
    if sz_opts["grad"] < 0:
        raise ValueError("Parameter grad must be > 0")
    if sz_opts["wl"] > 0:
        print(
            f"Mesh sizes will be built to resolve an estimate of wavelength of a "
            f"{sz_opts['freq']}  hz wavelet with {sz_opts['wl']} vertices",
            flush=True,
        )
    gterm = None
    if sz_opts["grad"] > 0:
        # _gradient_sizing (sizing/mesh_size_function.py:428-448) on the device
        print("Refining mesh sizes near sharp velocity gradients...")
        st = sz_opts["stencil_size"]
        window = [int(st)] * dim if np.isscalar(st) else [int(w) for w in st]
        # water replacement as the reference decides it (any vp < 1e-3 in a
        # row other than the first, sizing/mesh_size_function.py:154-165)
        if vp_host is not None:
            replace = bool(np.any(vp_host[1:] * scale < 1e-3))
        else:
            replace = bool((vpd[1:] * scale < 1e-3).any().item())
        vw = float(sz_opts["vp_water"]) if sz_opts["vp_water"] is not None else 0.0
        if replace and (sz_opts["vp_water"] is None or vw < 1300 or vw > 1800):
            raise ValueError("vp_water is None or out of bounds. It should be >1300 and <1800 m/s")
        gterm = torch.empty_like(vpd)
        gsz = N.c_sz(0)
        N.call("dm_gradient_term_workspace_size", vpd.numel(), gsz)
        gws = D.workspace(gsz.value)
        N.call(
            "dm_gradient_term", D.ptr(vpd), (N.c_int * 3)(*(list(shape) + [1] * (3 - dim))), dim,
            (N.c_int * 3)(*(window + [1] * (3 - dim))), scale, vw, int(replace),
            float(sz_opts["grad"]), D.ptr(gterm), D.ptr(gws), gws.numel(), D.stream_ptr(),
        )
    if sz_opts["dt"] != 0.0 and sz_opts["cr_max"] != 0.0 and sz_opts["space_order"] != 0:
        if sz_opts["cr_max"] < 0:
            raise ValueError("Parameter `cr_max` must be > 0.0")
        if sz_opts["dt"] < 0:
            raise ValueError("Parameter `dt` must be > 0.0")
        if sz_opts["space_order"] < 1:
            raise ValueError("Parameter `space_order` must be >= 1 ")
        print(f"Enforcing timestep of {sz_opts['dt']} seconds...", flush=True)
    print(f"Enforcing minimum edge length of {sz_opts['hmin']}")
    print(f"Enforcing maximum edge length of {sz_opts['hmax']}")
    ws = D.workspace(256)
    replaced = N.c_int(0)
    N.call(
        "dm_size_from_velocity", D.ptr(vpd), vpd.numel(), shape[1] * (shape[2] if dim == 3 else 1),
        D.ptr(gterm), scale, float(sz_opts["vp_water"] or 0.0), float(sz_opts["wl"]),
        float(sz_opts["freq"]), float(sz_opts["grad"]), float(sz_opts["hmin"]),
        float(sz_opts["hmax"]), float(sz_opts["dt"]), float(sz_opts["cr_max"]),
        float(sz_opts["space_order"]), dim, D.ptr(cell), replaced, D.ptr(ws), ws.numel(),
        D.stream_ptr(),
    )
    grade = sz_opts["grade"]
    if grade == 0.0:
        warnings.warn("Mesh size gradient is deactiavted. This may compromise mesh quality")
    else:
        if grade < 0:
            raise ValueError("Parameter `grade` must be > 0.0")
        if grade > 1.0:
            warnings.warn("Parameter `grade` is set pretty high (> 1.0)!")
        print(f"Enforcing mesh size gradation of {grade} decimal percent...")
        elen = (bbox[1] - bbox[0]) / nz
        # a C-order (n0, n1[, n2]) array is the column-major array with the
        # axes reversed; the limiter is symmetric in the axes
        dims = (N.c_int * 3)(*(list(shape[::-1]) + [1] * (3 - dim)))
        N.call("dm_limgrad", dims, float(elen), float(grade), 10000, D.ptr(cell), D.stream_ptr())

    cell, vpd, bbox = _build_domain_pad(cell, vpd, bbox, sz_opts)
    fh = GridSizing.from_device(cell, bbox)
    return SizeFunction(bbox, fh, sz_opts["hmin"])


def _gradient_sizing(vp, grad, stencil_size):
    """Gradient sizing term of a velocity grid on the device (the reference's
    _gradient_sizing, sizing/mesh_size_function.py:428-448): grad / (v + 0.1)
    with v the normalised windowed variance of vp.  Returns 99999 for grad == 0."""
    if grad == 0.0:
        return 99999
    if grad < 0:
        raise ValueError("Parameter grad must be > 0")
    vp = np.ascontiguousarray(np.asarray(vp, dtype=np.float64))
    dim = vp.ndim
    window = [int(stencil_size)] * dim if np.isscalar(stencil_size) else [int(w) for w in stencil_size]
    vpd = torch.from_numpy(vp).to(D.device())
    g = torch.empty_like(vpd)
    gsz = N.c_sz(0)
    N.call("dm_gradient_term_workspace_size", vpd.numel(), gsz)
    ws = D.workspace(gsz.value)
    N.call(
        "dm_gradient_term", D.ptr(vpd), (N.c_int * 3)(*(list(vp.shape) + [1] * (3 - dim))), dim,
        (N.c_int * 3)(*(window + [1] * (3 - dim))), 1.0, 0.0, 0, float(grad), D.ptr(g),
        D.ptr(ws), ws.numel(), D.stream_ptr(),
    )
    return g.cpu().numpy()


def _get_dimensions(shape, bbox):
    dim = len(shape)
    return [(bbox[2 * k + 1] - bbox[2 * k]) / shape[k] for k in range(dim)]


def _build_domain_pad(cell, vp, bbox, opts):
    """domain extension (sizing/mesh_size_function.py:526-572) on the GPU"""
    dim = cell.dim()
    domain_pad = opts["domain_pad"]
    pad_style = opts["pad_style"]
    if domain_pad < 0:
        raise ValueError("Domain extension must be >= 0")
    if domain_pad <= 0:
        return cell, vp, bbox
    print(f"Including a {domain_pad} meter domain extension...")
    d = _get_dimensions(tuple(cell.shape), bbox)
    nn = [int(domain_pad / dk) for dk in d]
    if dim == 2:
        bbox = (bbox[0] - domain_pad, bbox[1], bbox[2] - domain_pad, bbox[3] + domain_pad)
        pre, post = [nn[0], nn[1]], [0, nn[1]]
    else:
        bbox = (
            bbox[0] - domain_pad, bbox[1], bbox[2] - domain_pad, bbox[3] + domain_pad,
            bbox[4] - domain_pad, bbox[5] + domain_pad,
        )
        pre, post = [nn[0], nn[1], nn[2]], [0, nn[1], nn[2]]
    print(f"Using the pad_style: {pad_style}")
    modes = {"edge": 0, "constant": 1, "linear_ramp": 2}
    if pad_style not in modes:
        raise ValueError(
            "pad style currently not supported. Try `linear_ramp`, `edge`, or `constant`"
        )

    def pad(a):
        cval = float(a.max().item())
        out_shape = [a.shape[k] + pre[k] + post[k] for k in range(dim)]
        out = D.empty(out_shape, torch.float64)
        n = (N.c_int * 3)(*list(a.shape))
        pr = (N.c_int * 3)(*pre)
        po = (N.c_int * 3)(*post)
        N.call("dm_pad_grid", D.ptr(a), n, pr, po, dim, modes[pad_style], cval, D.ptr(out), D.stream_ptr())
        return out

    return pad(cell), pad(vp), bbox


def read_velocity_model(
    filename, nz=None, nx=None, ny=None, byte_order=None, axes_order=None,
    axes_order_sort=None, dtype=None,
):
    """Read a velocity model (sizing/mesh_size_function.py:590-606)."""
    if filename.endswith(".segy"):
        return _read_segy(filename)
    return _read_bin(filename, nz, nx, ny, byte_order, axes_order, axes_order_sort, dtype)


def _read_bin(filename, nz, nx, ny, byte_order, axes_order, axes_order_sort, dtype):
    """Binary model with endianness, axis order and F/C order
    (sizing/mesh_size_function.py:609-630)."""
    axes, fdt = _bin_layout(nz, nx, ny, byte_order, axes_order, dtype)
    print(f"Reading binary file: {filename}")
    vp = np.fromfile(filename, dtype=fdt)
    vp = vp.reshape(*axes, order=axes_order_sort)
    vp = np.flipud(vp.transpose((*axes_order,)))
    return vp, nz, nx, ny


def _bin_layout(nz, nx, ny, byte_order, axes_order, dtype):
    """stored axis lengths and file dtype of a binary model, checked as
    _read_bin checks them"""
    if (nz is None) or (nx is None) or (ny is None):
        raise ValueError(
            "Please specify the number of grid points in each dimension (e.g., `nz`, `nx`, `ny`)..."
        )
    axes = [nz, nx, ny]
    stored = [axes[o] for o in np.argsort(axes_order)]
    if byte_order == "big":
        fdt = np.dtype(dtype).newbyteorder(">")
    elif byte_order == "little":
        fdt = np.dtype(dtype).newbyteorder("<")
    else:
        raise ValueError("Please specify byte_order as either: little or big.")
    return stored, fdt


def read_velocity_model_to_device(
    filename, nz=None, nx=None, ny=None, byte_order=None, axes_order=(0, 1, 2),
    axes_order_sort="F", dtype="float32", device=None, slab_bytes=1 << 26,
):
    """Stream a raw binary velocity model from disk into a device grid.

    Returns (vp, nz, nx, ny) like read_velocity_model, with vp a float64
    tensor on `device` (default: the current CUDA device) equal to the
    array _read_bin returns: the file is reshaped in axes_order_sort order
    to the stored axis lengths, transposed by axes_order and flipped along
    its first axis (sizing/mesh_size_function.py:609-630).

    The file is read in slabs of slab_bytes.  On a CUDA device two pinned
    host buffers alternate: a slab is read and converted to native byte
    order while the previous one is copied to the device on a side stream
    and widened to FP64 there.  The reshape, transposition and flip are
    index permutations applied on the device, so no host copy of the whole
    model is made.  The defaults of axes_order, axes_order_sort and dtype
    are those of get_sizing_function_from_segy; nz, nx, ny and byte_order
    are required, as for _read_bin."""
    axes_order = (0, 1, 2) if axes_order is None else tuple(axes_order)
    axes_order_sort = "F" if axes_order_sort is None else axes_order_sort
    dtype = "float32" if dtype is None else dtype
    stored, fdt = _bin_layout(nz, nx, ny, byte_order, axes_order, dtype)
    if axes_order_sort not in ("F", "C", "A"):
        raise ValueError("order must be one of 'C', 'F' or 'A'")
    dev = D.device() if device is None else torch.device(device)
    total = int(np.prod(stored))
    size = os.path.getsize(filename)
    if size != total * fdt.itemsize:
        raise ValueError(
            f"cannot reshape array of size {size // fdt.itemsize} into shape {tuple(stored)}"
        )
    print(f"Reading binary file: {filename}")
    native = fdt.newbyteorder("=")
    tdt = torch.from_numpy(np.zeros(1, dtype=native)).dtype
    out = torch.empty(total, dtype=torch.float64, device=dev)
    chunk = max(1, min(total, int(slab_bytes) // fdt.itemsize))
    cuda = dev.type == "cuda"
    host = [torch.empty(chunk, dtype=tdt, pin_memory=cuda) for _ in range(2)]
    if cuda:
        stage = [torch.empty(chunk, dtype=tdt, device=dev) for _ in range(2)]
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        done = [None, None]
    with open(filename, "rb") as fh:
        for k, start in enumerate(range(0, total, chunk)):
            m = min(chunk, total - start)
            b = k % 2
            if cuda and done[b] is not None:
                done[b].synchronize()  # the copy out of this pinned buffer has ended
            raw = np.fromfile(fh, dtype=fdt, count=m)
            if raw.size != m:
                raise ValueError(f"{filename}: file ended after {start + raw.size} values")
            host[b].numpy()[:m] = raw
            if cuda:
                with torch.cuda.stream(side):
                    stage[b][:m].copy_(host[b][:m], non_blocking=True)
                    out[start:start + m].copy_(stage[b][:m])
                    done[b] = torch.cuda.Event()
                    done[b].record(side)
            else:
                out[start:start + m].copy_(host[b][:m])
    if cuda:
        torch.cuda.current_stream(dev).wait_stream(side)
    if axes_order_sort == "F":
        # column-major: the C-order view of the reversed lengths, axes reversed
        vp = out.view(*stored[::-1]).permute(2, 1, 0)
    else:
        vp = out.view(*stored)
    vp = vp.permute(*axes_order).flip(0).contiguous()
    return vp, nz, nx, ny


def _ibm_to_ieee(words):
    """IBM System/360 single precision (SEG-Y format code 1) to float64:
    sign bit, 7-bit base-16 exponent biased by 64, 24-bit fraction."""
    w = words.astype(np.uint32)
    sign = np.where(w >> 31, -1.0, 1.0)
    expo = ((w >> 24) & 0x7F).astype(np.int64) - 64
    frac = (w & 0x00FFFFFF).astype(np.float64) / float(1 << 24)
    return sign * frac * np.power(16.0, expo)


def _read_segy(filename):
    """SEG-Y reader (sizing/mesh_size_function.py:633-646) without segyio:
    3200-byte text header, 400-byte binary header (samples per trace at
    bytes 3221-3222, format code at 3225-3226), then traces of a 240-byte
    header plus samples.  Format codes 1 (IBM float) and 5 (IEEE float)."""
    raw = np.fromfile(filename, dtype=np.uint8)
    ns = int.from_bytes(raw[3220:3222].tobytes(), "big")
    fmt = int.from_bytes(raw[3224:3226].tobytes(), "big")
    if fmt not in (1, 5):
        raise NotImplementedError(f"SEG-Y sample format {fmt} is not supported")
    body = raw[3600:]
    tr_bytes = 240 + 4 * ns
    nx = len(body) // tr_bytes
    traces = body[: nx * tr_bytes].reshape(nx, tr_bytes)[:, 240:]
    words = traces.copy().view(">u4").reshape(nx, ns)
    if fmt == 1:
        vals = _ibm_to_ieee(words)
    else:
        vals = words.view(">f4").astype(np.float64)
    vp = np.ascontiguousarray(vals.T)
    if np.amin(vp) < 1000.0:
        warnings.warn("Velocity appear to be in km/s. Maybe pass `units` km-s key pair?")
    return np.flipud(vp), ns, nx, 0


def write_velocity_model(filename, ofname=None, comm=None, **kwargs):
    r"""Read a velocity model and write it as an HDF5 file
    (sizing/mesh_size_function.py:242-335).

    The model is read as read_velocity_model reads it (nz, nx, ny,
    byte_order, axes_order, axes_order_sort and dtype as there), padded when
    domain_pad > 0 (with bbox and pad_style, as the sizing call pads), and
    written to ofname + ".hdf5" (filename + ".hdf5" without ofname, with a
    warning) as the float32 dataset "velocity_model" with the attributes
    shape and units = "m/s".  With a communicator only rank 0 writes.
    Needs h5py."""
    try:
        import h5py
    except ImportError as e:
        raise ImportError("write_velocity_model needs h5py") from e
    opts = {
        "hmin": 150.0, "hmax": 10000.0, "wl": 0, "freq": 2.0, "grad": 0.0, "grade": 0.0,
        "stencil_size": 10.0, "space_order": 1, "dt": 0.0, "cr_max": 1.0, "pad_style": "edge",
        "domain_pad": 0.0, "units": "m-s", "nz": None, "nx": None, "ny": None,
        "byte_order": "byte_order", "axes_order": (0, 1, 2), "axes_order_sort": "F",
        "dtype": "float32",
    }
    opts.update(kwargs)
    if comm is not None and getattr(comm, "rank", 0) != 0:
        return
    if ofname is None:
        warnings.warn("No output filename specified, name will be `filename`")
        ofname = filename
    vp, nz, nx, ny = read_velocity_model(
        filename, nz=opts["nz"], nx=opts["nx"], ny=opts["ny"], byte_order=opts["byte_order"],
        axes_order=opts["axes_order"], axes_order_sort=opts["axes_order_sort"],
        dtype=opts["dtype"],
    )
    if opts["domain_pad"] > 0.0:
        print("Adding a domain pad to the velocity model...")
        vpd = torch.from_numpy(np.ascontiguousarray(vp, dtype=np.float64)).to(D.device())
        _, vpd, _ = _build_domain_pad(vpd, vpd, opts["bbox"], opts)
        vp = vpd.cpu().numpy()
    ofname += ".hdf5"
    print(f"Writing velocity model: {ofname}", flush=True)
    with h5py.File(ofname, "w") as f:
        f.create_dataset("velocity_model", data=vp, dtype="f")
        f.attrs["shape"] = vp.shape
        f.attrs["units"] = "m/s"


def plot_sizing_function(*args, **kwargs):
    raise NotImplementedError("plotting is not part of the GPU engine")
