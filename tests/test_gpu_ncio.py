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
