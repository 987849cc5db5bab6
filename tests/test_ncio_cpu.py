"""Field output in the netCDF classic 64-bit-offset format, the single-rank
path of pnet_out_chunk (common/mpi_parallel.f90:7481-8176), from host
arrays: every file is read back by scipy's independent netCDF-3 reader."""
import ctypes

import numpy as np
import pytest

scipy_io = pytest.importorskip("scipy.io")

NP, MP, LP, IH = 6, 5, 4, 1
FILL = 9.9692099683868690e+36


def field(seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.uniform(-2.0, 2.0, (NP + 2 * IH, MP + 2 * IH, LP + 2 * IH)).astype(dtype))


def interior(a):
    return a[IH:-IH, IH:-IH, IH:-IH]


def out(lib, name, path, imode, ifrmd, a):
    fn = lib.mpdata_pnet_out_chunk_f64 if a.dtype == np.float64 else lib.mpdata_pnet_out_chunk_f32
    return fn(name.encode(), str(path).encode(), imode, 0, 0, 0, ifrmd, 0, a.ctypes.data, NP, MP, LP, IH, 0, None)


def read(path):
    with scipy_io.netcdf_file(str(path), "r", mmap=False) as f:
        return {k: np.array(v.data) for k, v in f.variables.items()}, dict(f.dimensions), f.version_byte


def test_frames_and_variables_round_trip(native_lib, tmp_path):
    lib, p = native_lib, tmp_path / "tape.nc"
    psi = [field(s) for s in range(3)]
    th = [field(10 + s) for s in range(2)]
    assert out(lib, "psi", p, 1, 0, psi[0]) == 0
    assert out(lib, "th", p, 0, 0, th[0]) == 0     # a second variable rewrites the file
    assert out(lib, "psi", p, 1, 1, psi[1]) == 0
    assert out(lib, "th", p, 0, 1, th[1]) == 0
    assert out(lib, "psi", p, 1, 2, psi[2]) == 0    # th keeps the fill value at frame 3
    v, dims, ver = read(p)
    assert ver == 2 and dims == {"x": NP, "y": MP, "z": LP, "t": None}
    assert v["psi"].dtype == np.dtype(">f8") and v["psi"].shape == (3, LP, MP, NP)
    assert v["th"].dtype == np.dtype(">f4") and v["th"].shape == (3, LP, MP, NP)
    for t in range(3):
        np.testing.assert_array_equal(v["psi"][t], interior(psi[t]).transpose(2, 1, 0))
    for t in range(2):
        np.testing.assert_array_equal(v["th"][t], interior(th[t]).astype(np.float32).transpose(2, 1, 0))
    assert np.all(v["th"][2] == np.float32(FILL))


def test_variable_added_after_records_and_static_field(native_lib, tmp_path):
    lib, p = native_lib, tmp_path / "tape.nc"
    a = [field(20 + s) for s in range(3)]
    for t in range(3):
        assert out(lib, "u", p, 1, t, a[t]) == 0
    qv = field(30)
    assert out(lib, "qv", p, 1, 0, qv) == 0
    h = field(31, np.float32)
    assert out(lib, "h", p, 34, 0, h) == 0          # no time dimension
    v, dims, _ = read(p)
    for t in range(3):
        np.testing.assert_array_equal(v["u"][t], interior(a[t]).transpose(2, 1, 0))
    np.testing.assert_array_equal(v["qv"][0], interior(qv).transpose(2, 1, 0))
    assert np.all(v["qv"][1:] == FILL)
    assert v["h"].shape == (LP, MP, NP)
    np.testing.assert_array_equal(v["h"], interior(h).transpose(2, 1, 0))
    # a later frame beyond the last record: the frames in between hold fill values
    assert out(lib, "u", p, 1, 5, a[0]) == 0
    v, _, _ = read(p)
    assert v["u"].shape[0] == 6 and np.all(v["u"][3:5] == FILL) and np.all(v["qv"][3:] == FILL)
    np.testing.assert_array_equal(v["u"][5], interior(a[0]).transpose(2, 1, 0))


def test_read_back_into_interior(native_lib, tmp_path):
    lib, p = native_lib, tmp_path / "tape.nc"
    a, b = field(40), field(41)
    assert out(lib, "x", p, 1, 0, a) == 0
    assert out(lib, "x", p, 1, 1, b) == 0
    dst = field(42)
    halo = dst.copy()
    assert lib.mpdata_pnet_in_chunk_f64(b"x", str(p).encode(), 1, dst.ctypes.data, NP, MP, LP, IH, 0, None) == 0
    np.testing.assert_array_equal(interior(dst), interior(b))
    mask = np.ones(dst.shape, bool)
    mask[IH:-IH, IH:-IH, IH:-IH] = False
    np.testing.assert_array_equal(dst[mask], halo[mask])
    d32 = field(43, np.float32)
    assert lib.mpdata_pnet_in_chunk_f32(b"x", str(p).encode(), 0, d32.ctypes.data, NP, MP, LP, IH, 0, None) == 0
    np.testing.assert_array_equal(interior(d32), interior(a).astype(np.float32))


def test_errors(native_lib, tmp_path):
    lib, p = native_lib, tmp_path / "tape.nc"
    a = field(50)
    assert out(lib, "x", p, 5, 0, a) == -7          # not a pnet_out_chunk mode
    assert out(lib, "x", p, 1, 3, a) == -10         # frame > 0 of a variable never defined
    assert out(lib, "x", p, 1, 0, a) == 0
    # mode 0 into the double variable: the single-precision buffer converts to
    # double, as PnetCDF's put_vara_real does
    assert out(lib, "x", p, 0, 1, a) == 0
    v, _, _ = read(p)
    np.testing.assert_array_equal(v["x"][1], interior(a).astype(np.float32).astype(np.float64).transpose(2, 1, 0))
    assert out(lib, "x", p, 34, 1, a) == -1         # a static mode into the record variable
    assert lib.mpdata_pnet_in_chunk_f64(b"x", str(p).encode(), 4, a.ctypes.data, NP, MP, LP, IH, 0, None) == -10
    assert lib.mpdata_pnet_in_chunk_f64(b"x", str(tmp_path / "none.nc").encode(), 0, a.ctypes.data, NP, MP, LP,
                                        IH, 0, None) == -10
    bad = tmp_path / "bad.nc"
    bad.write_bytes(b"not a netcdf file")
    assert out(lib, "x", bad, 1, 0, a) == -10
