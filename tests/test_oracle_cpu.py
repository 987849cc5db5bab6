"""CPU checks of the oracle: the reference's known answer, conservation and
limiter-bound invariants, FP32 vs FP64, and the committed golden vectors."""
import os

import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _grid(O, f):
    return O.grid(f.np, f.mp, f.lp, f.ih, f.ibcx, f.ibcy, f.ibcz)


def test_kat_rotating_sphere_error_norm(oracle):
    """advection_dwarf_test_modular.f90:157-158: gauge MPDATA (DWARF3), 59^3,
    one revolution -> "Error L2 norm" 0.0028 (the reference's only known answer)."""
    f, meta = W.kat_rotating_sphere(59)
    oracle.advec_dwarf(_grid(oracle, f), f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h,
                       legacyoptmode=4, t_adv=1, iord=2, nonos=1, nsteps=meta["nt"])
    err = W.error_l2(f.x, meta["xtest"], 59 ** 3, meta["timetot"])
    assert round(err, 4) == 0.0028, err
    assert abs(err - 0.0028) < 5e-5
    # nonoscillatory: the field stays within the initial range [0, 4]
    xi = W.interior(f.x)
    assert xi.min() >= -1e-12 and xi.max() <= 4.0 + 1e-12


@pytest.mark.parametrize("t_adv", [1, 2])
@pytest.mark.parametrize("iord", [2, 3])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0), (1, 0, 1)])
def test_oracle_conserves_h_over_rhr_mass(oracle, t_adv, iord, ibc):
    """Flux form: sum(h*x_new/rhr) == sum(h*x_old) when no flux crosses the
    boundary (periodic axes; open walls with zero velocities on the wall
    faces; z walls with w = 0)."""
    f = W.random_fields(11, 9, 7, ibc=ibc, seed=7 + iord)
    ih = f.ih
    if not ibc[0]:
        f.u1[ih, :, :] = 0.0
        f.u1[ih + f.np, :, :] = 0.0
    if not ibc[1]:
        f.u2[:, ih, :] = 0.0
        f.u2[:, ih + f.mp, :] = 0.0
    if not ibc[2]:
        f.u3[...] = 0.0
    before = float((W.interior(f.h) * W.interior(f.x)).sum())
    oracle.advec_dwarf(_grid(oracle, f), f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h,
                       t_adv=t_adv, iord=iord)
    after = float((W.interior(f.h) * W.interior(f.x) / W.interior(f.rhr)).sum())
    assert abs(after - before) <= 1e-13 * abs(before)


def _star_bounds(x_in, xant, ibc, ih=1):
    """max/min over the 7-point stars of x_in (zero-gradient halo) and xant
    (reflection halo), z walls excluding the outside neighbour."""
    a = W.interior(x_in, ih)
    b = W.interior(xant, ih)
    out = []
    for arr, mode in ((a, "edge"), (b, "reflect")):
        pads = []
        for ax, per in enumerate(ibc):
            m = "wrap" if per else (mode if ax < 2 else "edge")
            pads.append(m)
        p = arr
        for ax, m in enumerate(pads):
            width = [(0, 0)] * 3
            width[ax] = (1, 1)
            p = np.pad(p, width, mode=m)
        c = p[1:-1, 1:-1, 1:-1]
        nb = [p[:-2, 1:-1, 1:-1], p[2:, 1:-1, 1:-1], p[1:-1, :-2, 1:-1], p[1:-1, 2:, 1:-1],
              p[1:-1, 1:-1, :-2], p[1:-1, 1:-1, 2:]]
        out.append((np.maximum.reduce([c] + nb), np.minimum.reduce([c] + nb)))
    return np.maximum(out[0][0], out[1][0]), np.minimum(out[0][1], out[1][1])


@pytest.mark.parametrize("t_adv", [1, 2])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)])
def test_oracle_limiter_bounds(oracle, t_adv, ibc):
    """nonoscillatory option: with rhr = 1 every new value lies within the
    local extrema of the input and the upwind field."""
    f = W.random_fields(12, 10, 8, ibc=ibc, seed=3)
    f.rhr[...] = 1.0
    g = _grid(oracle, f)
    x_in = f.x.copy(order="F")
    xant = oracle.upwind(g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h)
    # open walls: the upwind pass sees bcx/bcy in psi's halo
    x_up = x_in.copy(order="F")
    oracle.advec_dwarf(g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h, t_adv=t_adv, iord=2)
    mx, mn = _star_bounds(x_up, xant, ibc)
    xn = W.interior(f.x)
    tol = 1e-12 * np.abs(xn).max()
    assert (xn <= mx + tol).all() and (xn >= mn - tol).all()


def test_oracle_fp32_tracks_fp64(oracle):
    f = W.random_fields(10, 9, 8, ibc=(1, 1, 1), seed=11)
    f32 = f.astype(np.float32)
    g = _grid(oracle, f)
    oracle.advec_dwarf(g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h, t_adv=2, nsteps=5)
    oracle.advec_dwarf(g, f32.x, f32.bcx, f32.bcy, f32.u1, f32.u2, f32.u3, f32.rhr, f32.h, t_adv=2,
                       nsteps=5)
    a, b = W.interior(f.x), W.interior(f32.x).astype(np.float64)
    assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max()


def test_oracle_reproduces_golden_vectors(oracle):
    """Regression pin: the committed golden outputs (tests/golden/make_golden.py)."""
    from tests.golden import make_golden as G
    for case in G.CASES:
        ref = np.load(os.path.join(GOLDEN, case["name"] + ".npz"))
        f = G.build_case(case)
        G.run_oracle(oracle, f, case)
        np.testing.assert_array_equal(f.x, ref["x"], err_msg=case["name"])


def test_oracle_rejects_bad_calls(oracle):
    f = W.random_fields(4, 4, 4, seed=0)
    g = oracle.grid(1, 4, 4, 1, 0, 0, 0)  # open x needs np >= 2
    with pytest.raises(ValueError):
        oracle.advec_dwarf(g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h)
    g = _grid(oracle, f)
    with pytest.raises(ValueError):
        oracle.advec_dwarf(g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h, legacyoptmode=3)
