"""Velocity model readers and writer (sizing/mesh_size_function.py:242-335,
590-646) on files written here: a SEG-Y rev 1 file with IBM float samples
holding the decoded reference fixture, raw binaries in both byte orders and
axis orders (read on the host and streamed into a tensor), and the HDF5
writer against a stand-in h5py module."""
import numpy as np
import pytest
import torch

from seismicmesh_gb300.sizing.mesh_size_function import _read_bin, _read_segy

from conftest import golden


def _to_ibm(v):
    """float64 -> IBM System/360 single (sign, base-16 exponent + 64, 24-bit
    fraction), truncating like the hardware format"""
    out = np.zeros(v.shape, dtype=np.uint32)
    for idx, x in np.ndenumerate(v):
        if x == 0:
            continue
        s = 0x80000000 if x < 0 else 0
        a = abs(float(x))
        e = 64
        while a >= 1.0:
            a /= 16.0
            e += 1
        while a < 1.0 / 16.0:
            a *= 16.0
            e -= 1
        out[idx] = s | (e << 24) | int(a * (1 << 24))
    return out


def test_segy_reader_roundtrip(tmp_path):
    vp = golden("velocity_fixtures.npz")["segy_vp"]
    nz, nx = vp.shape
    traces = np.flipud(vp).T  # trace k = column k before the flip
    words = _to_ibm(traces)
    hdr = bytearray(3600)
    hdr[3220:3222] = int(nz).to_bytes(2, "big")
    hdr[3224:3226] = (1).to_bytes(2, "big")
    body = b"".join(bytes(240) + words[k].astype(">u4").tobytes() for k in range(nx))
    f = tmp_path / "m.segy"
    f.write_bytes(bytes(hdr) + body)
    got, gnz, gnx, gny = _read_segy(str(f))
    assert (gnz, gnx, gny) == (nz, nx, 0)
    np.testing.assert_array_equal(got, vp)


def test_binary_reader_orders(tmp_path):
    rng = np.random.default_rng(3)
    nz, nx, ny = 5, 4, 3
    for order in ((0, 1, 2), (2, 0, 1), (1, 2, 0)):
        for bo, code in (("little", "<f4"), ("big", ">f4")):
            for sort in ("F", "C"):
                axes = [nz, nx, ny]
                stored = [axes[o] for o in np.argsort(order)]
                data = rng.random(stored).astype(np.float32)
                f = tmp_path / f"m_{bo}_{sort}.bin"
                data.reshape(-1, order=sort).astype(code).tofile(str(f))
                got, *_ = _read_bin(str(f), nz, nx, ny, bo, order, sort, "float32")
                want = np.flipud(data.transpose(order))
                np.testing.assert_array_equal(got, want)


def test_vtk_writer_roundtrip(tmp_path):
    from seismicmesh_gb300.io import read_vtk, write_vtk

    rng = np.random.default_rng(5)
    for dim, nv in ((2, 3), (3, 4)):
        p = rng.random((50, dim))
        t = rng.integers(0, 50, (80, nv))
        f = tmp_path / f"m{dim}.vtk"
        write_vtk(str(f), p, t, cell_data={"q": rng.random(80)})
        pp, tt = read_vtk(str(f))
        np.testing.assert_array_equal(pp[:, :dim], p)
        np.testing.assert_array_equal(tt, t)
        assert f.read_bytes().startswith(b"# vtk DataFile Version 3.0")


def test_gmsh22_writer_roundtrip(tmp_path):
    from seismicmesh_gb300.io import read_gmsh22, write_mesh

    rng = np.random.default_rng(6)
    for dim, nv in ((2, 3), (3, 4)):
        p = rng.random((40, dim))
        t = rng.integers(0, 40, (70, nv))
        f = tmp_path / f"m{dim}.msh"
        write_mesh(str(f), p, t)
        pp, tt = read_gmsh22(str(f))
        np.testing.assert_array_equal(pp[:, :dim], p)
        np.testing.assert_array_equal(tt, t)


def test_ibm_float_known_answers():
    """IBM System/360 single-precision words with known values, written from
    the format's definition (sign bit, 7-bit excess-64 base-16 exponent,
    24-bit fraction): decoded independently of this file's encoder"""
    from seismicmesh_gb300.sizing.mesh_size_function import _ibm_to_ieee

    words = np.array([
        0x00000000,  # 0
        0x41100000,  # 16^1 * 1/16 = 1.0
        0xC1100000,  # -1.0
        0x42640000,  # 16^2 * 0x64/256 = 100.0
        0xC276A000,  # -(16^2 * 0x76A000/2^24) = -118.625
        0x43A98000,  # 16^3 * 0xA98000/2^24 = 2712.0 (a velocity)
        0x40800000,  # 16^0 * 0.5 = 0.5
        0x3F200000,  # 16^-1 * 0.125 = 0.0078125
    ], dtype=">u4")
    want = np.array([0.0, 1.0, -1.0, 100.0, -118.625, 2712.0, 0.5, 0.0078125])
    got = np.asarray(_ibm_to_ieee(words), dtype=np.float64).ravel()
    np.testing.assert_array_equal(got, want)


def test_streamed_binary_reader_matches_host_reader(tmp_path):
    """read_velocity_model_to_device (slabs through staging buffers, layout
    applied as tensor permutations) equals _read_bin exactly, for every axis
    order, both byte orders, F and C order, both dtypes and slabs that split
    the file unevenly"""
    import itertools

    from seismicmesh_gb300.sizing.mesh_size_function import read_velocity_model_to_device

    rng = np.random.default_rng(4)
    nz, nx, ny = 7, 5, 3
    for order in itertools.permutations((0, 1, 2)):
        for bo, end in (("little", "<"), ("big", ">")):
            for sort in ("F", "C"):
                for dt in ("float32", "float64"):
                    axes = [nz, nx, ny]
                    stored = [axes[o] for o in np.argsort(order)]
                    data = rng.random(stored).astype(dt)
                    f = tmp_path / f"m_{''.join(map(str, order))}_{bo}_{sort}_{dt}.bin"
                    data.reshape(-1, order=sort).astype(end + np.dtype(dt).str[1:]).tofile(str(f))
                    want, *_ = _read_bin(str(f), nz, nx, ny, bo, order, sort, dt)
                    for slab in (7 * np.dtype(dt).itemsize, 1 << 20):
                        got, gnz, gnx, gny = read_velocity_model_to_device(
                            str(f), nz, nx, ny, bo, order, sort, dt, device="cpu", slab_bytes=slab)
                        assert (gnz, gnx, gny) == (nz, nx, ny)
                        assert got.dtype == torch.float64 and got.is_contiguous()
                        np.testing.assert_array_equal(got.numpy(), want.astype(np.float64))


def test_streamed_binary_reader_checks_its_input(tmp_path):
    from seismicmesh_gb300.sizing.mesh_size_function import read_velocity_model_to_device

    f = tmp_path / "short.bin"
    np.zeros(59, dtype="<f4").tofile(str(f))
    with pytest.raises(ValueError, match="cannot reshape"):
        read_velocity_model_to_device(str(f), 5, 4, 3, "little", (0, 1, 2), "F", "float32", device="cpu")
    with pytest.raises(ValueError, match="byte_order"):
        read_velocity_model_to_device(str(f), 5, 4, 3, "middle", (0, 1, 2), "F", "float32", device="cpu")
    with pytest.raises(ValueError, match="number of grid points"):
        read_velocity_model_to_device(str(f), 5, None, 3, "little", (0, 1, 2), "F", "float32",
                                      device="cpu")


class _H5File:
    """stand-in for h5py.File: records what is written"""
    written = {}

    def __init__(self, name, mode):
        self.name, self.mode, self.attrs = name, mode, {}

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        _H5File.written[self.name] = self
        return False

    def create_dataset(self, key, data, dtype):
        self.key, self.data, self.dtype = key, np.array(data), dtype


def test_write_velocity_model_writes_the_reference_layout(tmp_path, monkeypatch):
    """sizing/mesh_size_function.py:242-335: dataset "velocity_model" (float),
    attributes shape and units, file ofname + ".hdf5"; h5py is absent here, so
    a stand-in module records the calls"""
    import sys
    import types
    import warnings

    from seismicmesh_gb300.sizing.mesh_size_function import write_velocity_model

    monkeypatch.setitem(sys.modules, "h5py", types.SimpleNamespace(File=_H5File))
    _H5File.written.clear()
    rng = np.random.default_rng(5)
    data = rng.random((4, 3, 2)).astype(np.float32)
    f = tmp_path / "v.bin"
    data.reshape(-1, order="F").astype("<f4").tofile(str(f))
    kw = dict(nz=4, nx=3, ny=2, byte_order="little")
    write_velocity_model(str(f), ofname=str(tmp_path / "out"), **kw)
    rec = _H5File.written[str(tmp_path / "out") + ".hdf5"]
    want, *_ = _read_bin(str(f), 4, 3, 2, "little", (0, 1, 2), "F", "float32")
    assert rec.mode == "w" and rec.key == "velocity_model" and rec.dtype == "f"
    np.testing.assert_array_equal(rec.data, want)
    assert tuple(rec.attrs["shape"]) == want.shape and rec.attrs["units"] == "m/s"
    # no output name: the input's, with a warning; ranks other than 0 write nothing
    _H5File.written.clear()
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        write_velocity_model(str(f), **kw)
    assert any("No output filename" in str(x.message) for x in w)
    assert list(_H5File.written) == [str(f) + ".hdf5"]
    _H5File.written.clear()
    write_velocity_model(str(f), ofname=str(tmp_path / "r1"), comm=types.SimpleNamespace(rank=1), **kw)
    assert not _H5File.written


def test_write_velocity_model_needs_h5py(tmp_path, monkeypatch):
    import sys

    from seismicmesh_gb300.sizing.mesh_size_function import write_velocity_model

    monkeypatch.setitem(sys.modules, "h5py", None)
    with pytest.raises(ImportError, match="h5py"):
        write_velocity_model(str(tmp_path / "v.bin"), nz=1, nx=1, ny=1, byte_order="little")
