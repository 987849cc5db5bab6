"""FP64 products by powers of two on the integer pipe (scale_down) against the
oracle's multiplications, bit for bit, where the fast path does not apply.

The kernels lower the exponent field of a normal operand instead of
multiplying by 0.5, 0.125 or 0.03125 (the C-grid averages of velprdA_to_C,
module_velprd.f90:197-361; the n+1/2 momenta of velprd_traj0 when
0.5*dt*dxi is a power of two, :60-83; vdyf and the cross terms of the
pseudo-velocities, antidiff3d-gauge-gpubc.f90:157-203).  Zeros keep their
sign; subnormal results and subnormal, infinite or NaN operands take the
multiplication.  These cases put every one of those paths under the
predictor and the step and compare with the oracle:
- momenta mixing +-0, subnormals, numbers at the bottom of the normal range
  (whose halves are subnormal), numbers near the top (whose sums overflow)
  and infinities;
- a step on a field of magnitude 1e-307, whose pseudo-velocities and
  corrective fluxes are subnormal or zero in part.
"""
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


def edge_values(rng, shape):
    """Normal numbers mixed with the operands that leave the fast path."""
    tiny = np.finfo(np.float64).tiny          # 2^-1022
    sub = np.finfo(np.float64).smallest_subnormal
    cats = [
        lambda n: rng.uniform(-1, 1, n),
        lambda n: np.zeros(n),
        lambda n: -np.zeros(n),
        lambda n: sub * rng.integers(-2 ** 40, 2 ** 40, n),
        lambda n: tiny * rng.uniform(-4, 4, n),
        lambda n: rng.choice([-1.0, 1.0], n) * tiny * rng.integers(1, 5, n),
        lambda n: 1.5e308 * rng.uniform(-1, 1, n),
        lambda n: rng.choice([-np.inf, np.inf], n),
    ]
    n = int(np.prod(shape))
    pick = rng.integers(0, len(cats), n)
    out = np.empty(n)
    for c, f in enumerate(cats):
        sel = pick == c
        out[sel] = f(int(sel.sum()))
    return np.asfortranarray(out.reshape(shape))


def same_bits_or_nan(got, want, what):
    """Equal values with equal zero signs; NaNs equal each other (their
    payloads differ between the host's and the device's arithmetic)."""
    np.testing.assert_array_equal(got, want, err_msg=what)
    fin = ~np.isnan(want)
    np.testing.assert_array_equal(np.signbit(got[fin]), np.signbit(want[fin]), err_msg=what + " (signs)")


@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)])
@pytest.mark.parametrize("steps", [(1.0, 1.0, 1.0, 1.0), (0.25, 0.5, 2.0, 0.5), (0.3, 1.0, 1.0, 1.0)],
                         ids=["hg_half", "hg_pow2_mixed", "hg_not_pow2"])
def test_predictor_edge_operands(M, oracle, ibc, steps):
    import torch
    dxi, dyi, dzi, dt = steps
    rng = np.random.default_rng(17 + sum(ibc))
    n, m, l, ih = 12, 10, 8, 1
    sh = W.shapes(n, m, l, ih)
    lev = sh["psi"] + (3,)
    o = [edge_values(rng, lev) for _ in range(3)]
    h = np.asfortranarray(rng.uniform(0.8, 1.2, sh["psi"]))
    h[2:5, 3:6, :] = 1.0  # unit-density warps and cells as well
    u = [W.zeros(sh[k]) for k in ("u1", "u2", "u3")]
    do = [M.fortran_device(a) for a in o]
    du = [M.fortran_device(a) for a in u]
    ws = M.Workspace(n, m, l, ih, *ibc, precision=64)
    ws.velprd(do[0], do[1], do[2], M.fortran_device(h), dxi, dyi, dzi, dt, 1.0, du[0], du[1], du[2])
    torch.cuda.synchronize()
    ws.close()
    with np.errstate(invalid="ignore", over="ignore"):
        oracle.velprd(oracle.grid(n, m, l, ih, *ibc), o[0], o[1], o[2], h, dxi, dyi, dzi, dt, 1.0, u[0], u[1], u[2])
    for c in range(3):
        got = M.to_numpy(do[c])
        for lv in range(3):
            same_bits_or_nan(W.interior(got[..., lv]), W.interior(o[c][..., lv]), "momentum %d level %d" % (c, lv))
    I, J, K = slice(ih, ih + n), slice(ih, ih + m), slice(ih, ih + l)
    same_bits_or_nan(M.to_numpy(du[0])[ih:ih + n + 1, J, K], u[0][ih:ih + n + 1, J, K], "u1")
    same_bits_or_nan(M.to_numpy(du[1])[I, ih:ih + m + 1, K], u[1][I, ih:ih + m + 1, K], "u2")
    same_bits_or_nan(M.to_numpy(du[2])[I, J, ih:ih + l + 1], u[2][I, J, ih:ih + l + 1], "u3")


@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)])
@pytest.mark.parametrize("t_adv,iord", [(1, 3), (2, 2)], ids=["gauge_i3", "std_i2"])
def test_step_on_a_tiny_field(M, oracle, ibc, t_adv, iord):
    """psi of magnitude 1e-307 with blocks of +-0: the pseudo-velocities'
    products by 0.5 and 2^-5 meet subnormal and zero operands."""
    import torch
    n, m, l = 40, 24, 12
    f = W.random_fields(n, m, l, ibc=ibc, seed=29, courant=0.3)
    x = W.interior(f.x)
    x *= 1e-307
    x[5:15, 3:9, 2:6] = 0.0
    x[20:30, 10:20, 4:10] = -0.0
    f.bcx[...] *= 1e-307
    f.bcy[...] *= 1e-307
    d = {k: M.fortran_device(getattr(f, k)) for k in ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}
    g = f.copy()
    for _ in range(2):
        M.advec_dwarf(4, t_adv, False, False, n, m, l, f.ih, 0, *ibc, d["x"], d["bcx"], d["bcy"], d["u1"],
                      d["u2"], d["u3"], d["rhr"], d["h"], iord=iord, nonos=1)
    torch.cuda.synchronize()
    out = M.to_numpy(d["x"])
    M.release_cached()
    oracle.advec_dwarf(oracle.grid(n, m, l, f.ih, *ibc), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3, g.rhr, g.h,
                       legacyoptmode=4, t_adv=t_adv, iord=iord, nonos=1, nsteps=2)
    got, want = W.interior(out), W.interior(g.x)
    assert np.any((want != 0) & (np.abs(want) < np.finfo(np.float64).tiny)), "no subnormal value was reached"
    np.testing.assert_array_equal(got.view(np.uint64), want.view(np.uint64))
