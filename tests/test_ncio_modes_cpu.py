"""The other pnet_out_chunk modes (common/mpi_parallel.f90:7481-8176) on a
single rank, from host arrays, read back with scipy's netCDF-3 reader.

The expected arrays restate each mode's single-rank behaviour: every edge
flag is set and the rank sits at position 1, so
- the staggered modes 2-4 write the block var(1:n+ia) of dimensions n+ia;
- the halo modes 6-8 write the right/top/sky strip at offset ih of a 2*ih
  dimension (the other strip is overwritten before the one write), and 9 the
  cells var(n-ih+1:n) at offset ih on every axis;
- the planes 10/13 (double), 11/12 (through single precision into double)
  and the lines 20-22 (float) are written only when (ia-1)/n == 0 for each
  fixed index; 35 writes the ground halo plane k = 1-ih without time; 30
  defines a float (t) variable and writes nothing.
"""
import numpy as np
import pytest

scipy_io = pytest.importorskip("scipy.io")

NP, MP, LP = 7, 6, 5
FILL = 9.9692099683868690e+36


def array(seed, ih, ia=(0, 0, 0), imem=0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    shape = tuple(n + a * imem + 2 * ih for n, a in zip((NP, MP, LP), ia))
    return np.asfortranarray(rng.uniform(-2.0, 2.0, shape).astype(dtype))


def out(lib, path, name, imode, a, ih, ia=(0, 0, 0), imem=0, ifrmd=0):
    fn = lib.mpdata_pnet_out_chunk_f64 if a.dtype == np.float64 else lib.mpdata_pnet_out_chunk_f32
    return fn(name.encode(), str(path).encode(), imode, ia[0], ia[1], ia[2], ifrmd, imem, a.ctypes.data, NP, MP,
              LP, ih, 0, None)


def read(path):
    with scipy_io.netcdf_file(str(path), "r", mmap=False) as f:
        return ({k: np.array(v.data) for k, v in f.variables.items()},
                {k: v.dimensions for k, v in f.variables.items()}, dict(f.dimensions))


def file_order(block):
    """(x,y,z) Fortran block -> the file's (z,y,x) order."""
    return np.ascontiguousarray(block.transpose(2, 1, 0))


@pytest.mark.parametrize("ia", [(1, 0, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1)])
@pytest.mark.parametrize("imode", [2, 3, 4])
def test_staggered_blocks(native_lib, tmp_path, imode, ia):
    ih = 1
    a = array(3, ih, ia, imem=1)
    p = tmp_path / "s.nc"
    assert out(native_lib, p, "u", imode, a, ih, ia, imem=1) == 0
    v, vd, dims = read(p)
    assert dims == {"x": NP + ia[0], "y": MP + ia[1], "z": LP + ia[2], "t": None}
    assert vd["u"] == ("t", "z", "y", "x") and v["u"].dtype == np.dtype(">f8")
    want = a[ih:ih + NP + ia[0], ih:ih + MP + ia[1], ih:ih + LP + ia[2]]
    np.testing.assert_array_equal(v["u"][0], file_order(want))


@pytest.mark.parametrize("ih", [1, 2])
def test_halo_strips(native_lib, tmp_path, ih):
    a = array(5, ih)
    n = (NP, MP, LP)
    for imode in (6, 7, 8):
        ax = imode - 6
        p = tmp_path / ("h%d.nc" % imode)
        assert out(native_lib, p, "hx", imode, a, ih) == 0
        assert out(native_lib, p, "hx", imode, a, ih, ifrmd=1) == 0
        v, vd, dims = read(p)
        want_dims = {"x": NP, "y": MP, "z": LP, "t": None}
        want_dims["xyz"[ax]] = 2 * ih
        assert dims == want_dims
        sl = [slice(ih, ih + NP), slice(ih, ih + MP), slice(ih, ih + LP)]
        sl[ax] = slice(ih + n[ax], ih + n[ax] + ih)          # the right/top/sky strip
        got = v["hx"]
        assert got.shape[0] == 2
        for t in range(2):
            g = got[t].transpose(2, 1, 0)                    # back to (x,y,z)
            lo = [slice(None)] * 3
            lo[ax] = slice(0, ih)
            hi = [slice(None)] * 3
            hi[ax] = slice(ih, 2 * ih)
            assert np.all(g[tuple(lo)] == FILL)              # never written on one rank
            np.testing.assert_array_equal(g[tuple(hi)], a[tuple(sl)])
    p = tmp_path / "h9.nc"
    assert out(native_lib, p, "c", 9, a, ih) == 0
    v, _, dims = read(p)
    assert dims == {"x": 2 * ih, "y": 2 * ih, "z": 2 * ih, "t": None}
    g = v["c"][0].transpose(2, 1, 0)
    want = a[NP:NP + ih, MP:MP + ih, LP:LP + ih]             # var(n-ih+1:n) on each axis
    np.testing.assert_array_equal(g[ih:, ih:, ih:], want)
    mask = np.ones(g.shape, bool)
    mask[ih:, ih:, ih:] = False
    assert np.all(g[mask] == FILL)


def test_halo_strip_in_existing_dimensions(native_lib, tmp_path):
    """A file whose x already has length np: the strip lands at offset ih of
    that dimension, the rest of the variable keeps fill values."""
    ih = 1
    a = array(7, ih)
    p = tmp_path / "e.nc"
    assert out(native_lib, p, "psi", 1, a, ih) == 0
    assert out(native_lib, p, "hx", 6, a, ih) == 0
    v, _, dims = read(p)
    assert dims["x"] == NP
    g = v["hx"][0].transpose(2, 1, 0)
    np.testing.assert_array_equal(g[ih:2 * ih], a[ih + NP:ih + NP + ih, ih:ih + MP, ih:ih + LP])
    assert np.all(g[:ih] == FILL) and np.all(g[2 * ih:] == FILL)


def test_planes_and_lines(native_lib, tmp_path):
    ih = 1
    a = array(9, ih)
    I, J, K = slice(ih, ih + NP), slice(ih, ih + MP), slice(ih, ih + LP)
    p = tmp_path / "pl.nc"
    cases = [
        # (name, imode, ia, dims, expected block in file order)
        ("xy3", 10, (0, 0, 3), ("t", "y", "x"), a[I, J, ih + 2].T),
        ("xy1", 13, (0, 0, 0), ("t", "y", "x"), a[I, J, ih].T),
        ("xz4", 11, (0, 4, 0), ("t", "z", "x"), a[I, ih + 3, K].astype(np.float32).astype(np.float64).T),
        ("yz2", 12, (2, 0, 0), ("t", "z", "y"), a[ih + 1, J, K].astype(np.float32).astype(np.float64).T),
        ("lz", 20, (2, 3, 0), ("t", "z"), a[ih + 1, ih + 2, K].astype(np.float32)),
        ("ly", 21, (2, 0, 4), ("t", "y"), a[ih + 1, J, ih + 3].astype(np.float32)),
        ("lx", 22, (0, 3, 5), ("t", "x"), a[I, ih + 2, ih + 4].astype(np.float32)),
    ]
    for name, imode, ia, _, _ in cases:
        assert out(native_lib, p, name, imode, a, ih, ia) == 0
    assert out(native_lib, p, "gnd", 35, a, ih) == 0
    assert out(native_lib, p, "pt", 30, a, ih) == 0
    v, vd, dims = read(p)
    for name, imode, ia, d, want in cases:
        assert vd[name] == d, name
        assert v[name].dtype == np.dtype(">f4" if imode >= 20 else ">f8"), name
        np.testing.assert_array_equal(v[name][0], want, err_msg=name)
    assert vd["gnd"] == ("y", "x") and v["gnd"].dtype == np.dtype(">f8")
    np.testing.assert_array_equal(v["gnd"], a[I, J, 0].T)    # the plane k = 1-ih
    assert vd["pt"] == ("t",) and v["pt"].dtype == np.dtype(">f4")


def test_planes_outside_the_rank_are_not_written(native_lib, tmp_path):
    """A fixed index with (ia-1)/n != 0 lies on another rank: the variable is
    defined and nothing is written (no record)."""
    ih = 1
    a = array(11, ih)
    p = tmp_path / "o.nc"
    assert out(native_lib, p, "xy", 10, a, ih, (0, 0, LP + 1)) == 0
    assert out(native_lib, p, "lz", 20, a, ih, (NP + 1, 2, 0)) == 0
    v, vd, dims = read(p)
    assert v["xy"].shape == (0, MP, NP) and v["lz"].shape == (0, LP)
    assert "z" not in vd["xy"] and dims["x"] == NP


def test_plane_frames(native_lib, tmp_path):
    ih = 1
    frames = [array(20 + t, ih) for t in range(3)]
    p = tmp_path / "f.nc"
    for t, a in enumerate(frames):
        assert out(native_lib, p, "xy", 10, a, ih, (0, 0, 2), ifrmd=t) == 0
    v, _, _ = read(p)
    for t, a in enumerate(frames):
        np.testing.assert_array_equal(v["xy"][t], a[ih:ih + NP, ih:ih + MP, ih + 1].T)


def test_mode_errors(native_lib, tmp_path):
    ih = 1
    a = array(30, ih)
    p = tmp_path / "x.nc"
    for imode in (5, 14, 23, 31, 36):
        assert out(native_lib, p, "x", imode, a, ih) == -7, imode
    # a staggered block larger than the array: (1, 0, 0) offsets with imem = 0
    # reach one cell past the halo only when ih = 0
    b = array(31, 0)
    assert out(native_lib, p, "s", 2, b, 0, (1, 0, 0)) == -1
    # a plane index outside the array's halo
    assert out(native_lib, p, "xy", 10, a, ih, (0, 0, -1)) == -1
