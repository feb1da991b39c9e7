"""Velocity model readers (sizing/mesh_size_function.py:590-646) on files
written here: a SEG-Y rev 1 file with IBM float samples holding the decoded
reference fixture, and raw binaries in both byte orders and axis orders."""
import numpy as np

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
