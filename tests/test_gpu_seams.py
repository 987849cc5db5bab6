"""Full warps at a boundary.  A 96-wide grid puts whole warps at i = 1 and
i = np, and the boundary flags mix periodic seams and walls on every axis.  In
the FP64 gauge form such warps read the stored pair sums of xant (through the
xant halo maps: wrap or reflection) and of the pass velocities (through the
face maps).  The step and the batch must match the oracle bit for bit, the
adjoint to rounding (its atomic sums have no fixed order)."""
import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W
from tests.test_gpu_adjoint import gpu_adjoint_run, oracle_adjoint, problem, rel
from tests.test_gpu_batch import dev, oracle_steps

pytestmark = pytest.mark.gpu

N = (96, 12, 10)
IBCS = [(1, 1, 1), (1, 0, 1), (0, 1, 1), (1, 1, 0)]
IDS = ["periodic", "y_walls", "x_walls", "z_walls"]


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


def set_density(f, density):
    """unit: h = rhr = 1; one_cell_off: one cell of the i = np seam warp
    differs; random: the generator's densities."""
    if density == "random":
        return f
    f.h[...] = 1.0
    f.rhr[...] = 1.0
    if density == "one_cell_off":
        f.h[90, 5, 4] = 1.125
        f.rhr[90, 5, 4] = 0.875
    return f


@pytest.mark.parametrize("density", ["unit", "one_cell_off", "random"])
@pytest.mark.parametrize("iord", [2, 3])
@pytest.mark.parametrize("ibc", IBCS, ids=IDS)
def test_step_on_seams(M, oracle, ibc, iord, density):
    f = set_density(W.random_fields(*N, ibc=ibc, seed=71 + iord, courant=0.3), density)
    d = dev(M, f)
    ws = M.Workspace(*N, 1, *ibc, iord=iord, nonos=1, gauge=1, precision=64)
    for _ in range(3):
        ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], d["bcx"], d["bcy"])
    out = M.to_numpy(d["x"])
    ws.close()
    np.testing.assert_array_equal(out, oracle_steps(oracle, f, 1, iord, 3))


@pytest.mark.parametrize("iord", [2, 3])
@pytest.mark.parametrize("shape", [(32, 4), (16, 8)])
def test_batch_domains_on_seams(M, oracle, shape, iord):
    """Three gauge domains with their own velocities (both passes store the
    velocity pairs) and different boundary flags, in one batch."""
    doms = [((96, 12, 10), (1, 1, 1)), ((64, 8, 6), (1, 0, 1)), ((128, 10, 6), (0, 1, 1))]
    fs = [set_density(W.random_fields(*n, ibc=ibc, seed=81 + p, courant=0.3), "unit" if p != 1 else "random")
          for p, (n, ibc) in enumerate(doms)]
    probs = [dict(np=n[0], mp=n[1], lp=n[2], ibcx=ibc[0], ibcy=ibc[1], ibcz=ibc[2], gauge=1) for n, ibc in doms]
    b = M.Batch(probs, iord=iord)
    b.shape(*shape)
    ds = [dev(M, f) for f in fs]
    for p, d in enumerate(ds):
        b.set(p, d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], d["bcx"], d["bcy"])
    for _ in range(3):
        b.step()
    for p, (f, d) in enumerate(zip(fs, ds)):
        np.testing.assert_array_equal(M.to_numpy(d["x"]), oracle_steps(oracle, f, 1, iord, 3),
                                      err_msg="domain %d" % p)
    b.close()


@pytest.mark.parametrize("iord", [2, 3])
@pytest.mark.parametrize("ibc", IBCS, ids=IDS)
def test_adjoint_on_seams(M, oracle, ibc, iord):
    """The record and reverse kernels of seam warps (pair sums through the
    wrap maps) against the oracle's reverse-mode AD, two steps."""
    f, target = problem(N, ibc, seed=91 + iord)
    set_density(f, "unit")
    J, xN, gx, g1, g2, g3, _ = gpu_adjoint_run(M, f, target, 2, iord=iord, gauge=1)
    Jo, xNo, gxo, g1o, g2o, g3o = oracle_adjoint(oracle, f, target, 2, iord=iord, gauge=1)
    np.testing.assert_array_equal(W.interior(xN), W.interior(xNo))
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert rel(gx, gxo) <= 1e-11
    for a, b in ((g1, g1o), (g2, g2o), (g3, g3o)):
        assert rel(a, b) <= 1e-11
