"""Bit patterns of the FP64 fast paths against the oracle.

The FP64 kernels take shortcuts that must not change a bit:
- warps whose densities are all exactly 1 drop the products and quotients by
  them;
- the donor flux pp(a)*y1 - pn(a)*y2 is one multiplication, with the sign of a
  zero result rebuilt from the operands' sign bits;
- limiter ratios of at least 1 are stored as 1;
- the predictor's 0.5*gc and r = 1 are folded.
These cases put unit and non-unit warps side by side (one perturbed cell),
zero patches, negative zeros and zero velocities in the inputs, and compare
the raw 64-bit patterns, so a zero of the wrong sign fails."""
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


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def zero_laden(n, ibc, seed, perturb):
    """Signed random field with a zero block, scattered -0.0 cells and zero
    Courant numbers; h = rhr = 1 except one cell when `perturb`."""
    f = W.random_fields(*n, ibc=ibc, seed=seed, courant=0.3, sign_change=True)
    rng = np.random.default_rng(seed + 100)
    f.x[20:50, 3:7, 2:5] = 0.0
    neg = rng.random(f.x.shape) < 0.05
    f.x[neg] = -0.0
    for a in (f.u1, f.u2, f.u3):
        a[rng.random(a.shape) < 0.1] = 0.0
        a[rng.random(a.shape) < 0.05] = -0.0
    f.u1[30:40, :, 3] = 0.0
    f.h[...] = 1.0
    f.rhr[...] = 1.0
    if perturb:
        f.h[45, 5, 4] = 1.125
        f.rhr[45, 5, 4] = 0.875
    return f


@pytest.mark.parametrize("perturb", [False, True], ids=["unit", "one_cell_off"])
@pytest.mark.parametrize("iord", [2, 3, 5])
@pytest.mark.parametrize("t_adv", [1, 2], ids=["gauge", "std"])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)], ids=["periodic", "walls"])
def test_step_bits_with_zeros_and_unit_density(M, oracle, ibc, t_adv, iord, perturb):
    n = (80, 10, 8)  # x extent > 64: whole warps away from every wall
    f = zero_laden(n, ibc, seed=11 + iord + 3 * t_adv, perturb=perturb)
    g = f.copy()
    d = {k: M.fortran_device(getattr(f, k)) for k in ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}
    ws = M.Workspace(*n, 1, *ibc, iord=iord, nonos=1, gauge=1 if t_adv == 1 else 0, precision=64)
    for _ in range(3):
        ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], d["bcx"], d["bcy"])
    out = M.to_numpy(d["x"])
    ws.close()
    oracle.advec_dwarf(oracle.grid(*n, 1, *ibc), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3, g.rhr, g.h,
                       t_adv=t_adv, iord=iord, nsteps=3)
    assert np.signbit(g.x).any() and (g.x == 0).any()
    np.testing.assert_array_equal(bits(out), bits(g.x))


@pytest.mark.parametrize("perturb", [False, True], ids=["unit", "one_cell_off"])
@pytest.mark.parametrize("dt_ratio", [1.0, 0.75])
def test_predictor_bits_unit_density(M, oracle, dt_ratio, perturb):
    import torch
    rng = np.random.default_rng(7)
    n, m, l, ih = 70, 6, 5, 1
    sh = W.shapes(n, m, l, ih)
    lev = sh["psi"] + (3,)
    ox, oy, oz = (np.asfortranarray(rng.uniform(-1, 1, lev)) for _ in range(3))
    for a in (ox, oy, oz):
        a[rng.random(lev) < 0.1] = -0.0
    h = np.asfortranarray(np.ones(sh["psi"]))
    if perturb:
        h[40, 3, 2] = 0.9375
    u1, u2, u3 = (W.zeros(sh[k]) for k in ("u1", "u2", "u3"))
    args = dict(dxi=0.5, dyi=0.25, dzi=2.0, dt=0.3, dt_ratio=dt_ratio)
    dv = {k: M.fortran_device(a) for k, a in dict(ox=ox, oy=oy, oz=oz, h=h, u1=u1, u2=u2, u3=u3).items()}
    ws = M.Workspace(n, m, l, ih, 1, 1, 1, precision=64)
    ws.velprd(dv["ox"], dv["oy"], dv["oz"], dv["h"], args["dxi"], args["dyi"], args["dzi"], args["dt"],
              args["dt_ratio"], dv["u1"], dv["u2"], dv["u3"])
    torch.cuda.synchronize()
    oracle.velprd(oracle.grid(n, m, l, ih, 1, 1, 1), ox, oy, oz, h, args["dxi"], args["dyi"], args["dzi"],
                  args["dt"], args["dt_ratio"], u1, u2, u3)
    for k, a in dict(ox=ox, oy=oy, oz=oz).items():
        got = M.to_numpy(dv[k])
        for lv in range(3):
            np.testing.assert_array_equal(bits(W.interior(got[..., lv])), bits(W.interior(a[..., lv])),
                                          err_msg="%s level %d" % (k, lv))
    I, J, K = slice(ih, ih + n), slice(ih, ih + m), slice(ih, ih + l)
    for k, a, sl in (("u1", u1, (slice(ih, ih + n + 1), J, K)), ("u2", u2, (I, slice(ih, ih + m + 1), K)),
                     ("u3", u3, (I, J, slice(ih, ih + l + 1)))):
        np.testing.assert_array_equal(bits(M.to_numpy(dv[k])[sl]), bits(a[sl]), err_msg=k)
    ws.close()
