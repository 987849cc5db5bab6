"""The no-allocation step (mpdata_step_noalloc_f64) against the workspace
step (mpdata_step_f64), through the C ABI, on two calls in a row.

Callers that cannot let the library allocate device memory use the
no-allocation entry point; it must give the same field as the regular one.
This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import _native, mpdata
    return native_lib, _native, mpdata, torch


@pytest.mark.parametrize("ibc,gauge,iord,nonos", [((1, 1, 1), 1, 3, 1), ((0, 0, 0), 0, 2, 1), ((1, 0, 0), 1, 2, 1),
                                                   ((1, 1, 1), 1, 1, 1), ((0, 1, 0), 1, 3, 0), ((1, 1, 1), 0, 2, 0)])
def test_noalloc_matches_workspace_step_twice(env, ibc, gauge, iord, nonos):
    lib, N, M, torch = env
    n, m, l = 32, 32, 32  # exactly the 32768-cell limit
    f = W.random_fields(n, m, l, ibc=ibc, seed=5 + iord + gauge)
    a = {k: M.fortran_device(getattr(f, k)) for k in ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}
    b = {k: v.clone() for k, v in a.items()}
    grid = N.MpdataGrid(n, m, l, 1, *ibc)
    opts = N.MpdataOpts(iord, nonos, gauge, 64, 0)
    ws = M.Workspace(n, m, l, 1, *ibc, iord=iord, nonos=nonos, gauge=gauge, precision=64)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        torch.cuda.synchronize()
        alloc0, free0 = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
        rc = lib.mpdata_step_noalloc_f64(grid, opts, b["x"].data_ptr(), b["u1"].data_ptr(), b["u2"].data_ptr(),
                                         b["u3"].data_ptr(), b["h"].data_ptr(), b["rhr"].data_ptr(),
                                         b["bcx"].data_ptr(), b["bcy"].data_ptr(), stream)
        assert rc == 0, lib.mpdata_strerror(rc)
        torch.cuda.synchronize()
        if call == 1:  # a warm call takes no device memory from torch's pool or the driver
            assert torch.cuda.memory_allocated() == alloc0
            assert torch.cuda.mem_get_info()[0] == free0
        ws.step(a["x"], a["u1"], a["u2"], a["u3"], a["h"], a["rhr"], a["bcx"], a["bcy"])
        torch.cuda.synchronize()
        got, ref = M.to_numpy(b["x"]), M.to_numpy(a["x"])
        # same arithmetic: equal bits; the bound is the parity tolerance of the suite
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), "call %d" % call
        np.testing.assert_array_equal(got, ref)
    ws.close()


def test_noalloc_rejects_grids_beyond_its_scratch(env):
    lib, N, M, torch = env
    grid = N.MpdataGrid(33, 32, 32, 1, 1, 1, 1)  # 33792 cells > 32768
    opts = N.MpdataOpts(2, 1, 1, 64, 0)
    dummy = ctypes.c_void_p(1)
    rc = lib.mpdata_step_noalloc_f64(grid, opts, dummy, dummy, dummy, dummy, dummy, dummy, None, None, None)
    assert rc == -8
    assert b"32768" in lib.mpdata_strerror(rc)
    # FP32 is not offered by this entry point
    rc = lib.mpdata_step_noalloc_f64(N.MpdataGrid(8, 8, 8, 1, 1, 1, 1), N.MpdataOpts(2, 1, 1, 32, 0),
                                     dummy, dummy, dummy, dummy, dummy, dummy, None, None, None)
    assert rc == -2
    # the fused predictor is reserved, as for a workspace
    rc = lib.mpdata_step_noalloc_f64(N.MpdataGrid(8, 8, 8, 1, 1, 1, 1), N.MpdataOpts(2, 1, 1, 64, 1),
                                     dummy, dummy, dummy, dummy, dummy, dummy, None, None, None)
    assert rc == -7
