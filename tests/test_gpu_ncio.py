"""Field output from device arrays: the pack kernel (interior gather,
precision conversion, big-endian bytes on the GPU) must write the same file,
byte for byte, as the host path; and reading a frame back into a device
array restores its interior."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = (37, 29, 11)
IH = 1


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_device_file_equals_host_file(M, tmp_path, dtype):
    rng = np.random.default_rng(5)
    shp = tuple(n + 2 * IH for n in N)
    frames = [np.asfortranarray(rng.uniform(-3, 3, shp).astype(dtype)) for _ in range(3)]
    for where in ("host", "dev"):
        p = tmp_path / ("%s.nc" % where)
        for t, a in enumerate(frames):
            var = M.fortran_device(a) if where == "dev" else a
            M.pnet_out_chunk("psi", p, 1, t, var, *N, IH)
            M.pnet_out_chunk("psi_sp", p, 0, t, var, *N, IH)
        M.pnet_out_chunk("h", p, 34, 0, var, *N, IH)
    assert (tmp_path / "host.nc").read_bytes() == (tmp_path / "dev.nc").read_bytes()
    d = M.fortran_device(np.zeros(shp, dtype=dtype, order="F"))
    M.pnet_in_chunk("psi", tmp_path / "dev.nc", 1, d, *N, IH)
    got = M.to_numpy(d)
    np.testing.assert_array_equal(got[IH:-IH, IH:-IH, IH:-IH], frames[1][IH:-IH, IH:-IH, IH:-IH])
    assert np.all(got[0] == 0)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_device_file_equals_host_file_all_modes(M, tmp_path, dtype):
    """Every other mode (staggered block, halo strips and corners, planes,
    lines, the ground plane, the point variable) writes the same bytes from
    a device array as from the host."""
    rng = np.random.default_rng(9)
    ih, ia = 2, (1, 1, 1)
    stag = np.asfortranarray(rng.uniform(-3, 3, tuple(n + a + 2 * ih for n, a in zip(N, ia))).astype(dtype))
    psi = np.asfortranarray(rng.uniform(-3, 3, tuple(n + 2 * ih for n in N)).astype(dtype))
    calls = [("st", 4, ia, 1, stag)] + [("h%d" % m, m, (0, 0, 0), 0, psi) for m in (6, 7, 8, 9)] + [
        ("p10", 10, (0, 0, 5), 0, psi), ("p11", 11, (0, 7, 0), 0, psi), ("p12", 12, (9, 0, 0), 0, psi),
        ("p13", 13, (0, 0, 0), 0, psi), ("l20", 20, (3, 4, 0), 0, psi), ("l21", 21, (3, 0, 6), 0, psi),
        ("l22", 22, (0, 4, 6), 0, psi), ("g35", 35, (0, 0, 0), 0, psi), ("p30", 30, (0, 0, 0), 0, psi)]
    for where in ("host", "dev"):
        for name, imode, a, imem, arr in calls:
            p = tmp_path / ("%s_%s.nc" % (where, name))
            var = M.fortran_device(arr) if where == "dev" else arr
            for t in range(2):
                M.pnet_out_chunk(name, p, imode, t, var, *N, ih, ia1=a[0], ia2=a[1], ia3=a[2], imem=imem)
    for name, _, _, _, _ in calls:
        assert (tmp_path / ("host_%s.nc" % name)).read_bytes() == (tmp_path / ("dev_%s.nc" % name)).read_bytes(), name
