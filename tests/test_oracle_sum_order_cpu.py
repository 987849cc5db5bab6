"""How far the oracle's fixed order of the 4-face velocity sums moves a field.

The reference writes the six sums of the cross terms without parentheses
(antidiff3d-gauge-gpubc.f90:163-203, antidiff3d-standard-gpubc.f90:99-157),
so a Fortran compiler may evaluate them in any order.  The oracle and the
CUDA kernels fix one, the sum of two cell-centred pairs; the oracle's literal
mode evaluates them left to right as written.  After 100 steps the two orders
agree to a few ulps on smooth fields (the benchmark's deformational flow and
the reference's own rotating-sphere test), at iord 2 and 3, in both forms.
"""
import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W


def _run(O, f, t_adv, iord, literal, steps):
    g = f.copy()
    O.set_literal_sums(literal)
    try:
        O.advec_dwarf(O.grid(g.np, g.mp, g.lp, g.ih, g.ibcx, g.ibcy, g.ibcz), g.x, g.bcx, g.bcy, g.u1, g.u2,
                      g.u3, g.rhr, g.h, legacyoptmode=4, t_adv=t_adv, iord=iord, nonos=1, nsteps=steps)
    finally:
        O.set_literal_sums(0)
    return W.interior(g.x)


def _gap(a, b):
    return float(np.abs(a - b).max() / np.abs(a).max())


@pytest.mark.parametrize("t_adv", [1, 2])
@pytest.mark.parametrize("iord", [2, 3])
def test_literal_order_gap_deformational(oracle, t_adv, iord):
    """Deformational flow (the benchmark's field and velocity), 32x32x16
    periodic, 100 steps: L-infinity relative gap below 1e-13 (measured
    1.2e-15 to 1.7e-14)."""
    f = W.deformational(32, 32, 16)
    a = _run(oracle, f, t_adv, iord, 0, 100)
    b = _run(oracle, f, t_adv, iord, 1, 100)
    assert not np.array_equal(a, b), "the two orders should differ in some ulp"
    assert _gap(a, b) <= 1e-13, _gap(a, b)


def test_literal_order_gap_rotating_sphere(oracle):
    """The reference's own test case (59^3 open walls, gauge, iord=2), 100
    of its 556 steps: gap below 1e-13 (measured 7.8e-16)."""
    f, _ = W.kat_rotating_sphere(59)
    a = _run(oracle, f, 1, 2, 0, 100)
    b = _run(oracle, f, 1, 2, 1, 100)
    assert _gap(a, b) <= 1e-13, _gap(a, b)


def test_default_order_is_restored(oracle):
    """The switch is scoped: the default order reproduces a plain run."""
    f = W.deformational(16, 16, 8)
    a = _run(oracle, f, 1, 3, 0, 3)
    _run(oracle, f, 1, 3, 1, 3)
    b = _run(oracle, f, 1, 3, 0, 3)
    np.testing.assert_array_equal(a, b)
