"""FP64 compensated reductions (mass, error norms) against exactly rounded
host sums (math.fsum)."""
import math

import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_mass_matches_fsum(M, dtype):
    f = W.random_fields(45, 33, 21, ibc=(1, 1, 1), seed=3, dtype=dtype)
    # a wide dynamic range makes plain summation lose digits
    f.x[...] *= np.where(np.arange(f.x.size).reshape(f.x.shape, order="F") % 7 == 0, 1e8, 1.0).astype(dtype)
    x, h, rhr = (M.fortran_device(getattr(f, k)) for k in ("x", "h", "rhr"))
    xi = W.interior(f.x).astype(np.float64)
    hi = W.interior(f.h).astype(np.float64)
    ri = W.interior(f.rhr).astype(np.float64)
    exact = math.fsum((xi * hi).ravel())
    got = M.mass(x, h)
    assert abs(got - exact) <= 4e-16 * abs(exact)
    exact_r = math.fsum((xi * hi / ri).ravel())
    assert abs(M.mass(x, h, rhr) - exact_r) <= 4e-16 * abs(exact_r)


def test_error_norms_fp32_against_fp64(M):
    import torch
    f = W.random_fields(30, 20, 10, ibc=(1, 1, 1), seed=4)
    a64 = M.fortran_device(f.x)
    a32 = M.fortran_device(f.x.astype(np.float32))
    mx, l2, bmax, bl2 = M.error_norms(a32, a64)
    ai, bi = W.interior(f.x.astype(np.float32)).astype(np.float64), W.interior(f.x)
    d = (ai - bi).ravel()
    assert mx == pytest.approx(np.abs(d).max(), rel=0, abs=0)
    assert l2 == pytest.approx(math.sqrt(math.fsum(d * d)), rel=1e-14)
    assert bmax == np.abs(bi).max()
    assert bl2 == pytest.approx(math.sqrt(math.fsum(bi.ravel() ** 2)), rel=1e-14)
    torch.cuda.synchronize()
