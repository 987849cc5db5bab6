"""Multi-step parity of the benchmark's whole chain against the oracle.

Each step of the headline workload is: the A-grid Courant numbers at t_n
(pattern x cos(pi t/T) for u and v, steady w), the velocity predictor
(velprd_traj0 + velprdA_to_C, module_velprd.f90:58-83,197-361) with the
driver's level roll (velprd_driver.f90:254-270), then one gauge MPDATA step,
iord=3, nonoscillatory (antidiff3d-gauge-gpubc.f90:89-428, with the recursion
for the third pass).  The tests run that chain through the C ABI and the CPU
oracle on the same inputs and compare every value bit for bit: psi, the
C-grid Courant numbers and the three momentum levels.

The A-grid momenta at level 0 are formed on the host once per step and
uploaded to both, so that the comparison covers the library alone.
"""
import os

import numpy as np
import pytest

import bench
from advectionhpctester_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


class Chain:
    """The benchmark's step on the host (oracle) and on the device (library)."""

    def __init__(self, M, O, nx, ny, nz, dnp, T=200.0):
        self.M, self.O, self.T, self.dnp = M, O, T, dnp
        f, pats = bench.make_state(nx, ny, nz, dnp, T=T)
        self.f, self.pats = f, pats
        sh = f.x.shape + (3,)
        self.o = [np.zeros(sh, dtype=dnp, order="F") for _ in range(3)]
        for c in range(3):
            fac = dnp(bench.time_factor(-1, T)) if c < 2 else dnp(1.0)
            self.o[c][..., 2] = pats[c] * fac
        self.g = O.grid(nx, ny, nz, 1, 1, 1, 1)
        self.d = {k: M.fortran_device(getattr(f, k), dtype=dnp) for k in ("x", "u1", "u2", "u3", "h", "rhr")}
        self.do = [M.fortran_device(a, dtype=dnp) for a in self.o]
        prec = 64 if dnp == np.float64 else 32
        self.ws = M.Workspace(nx, ny, nz, 1, 1, 1, 1, iord=3, nonos=1, gauge=1, precision=prec)

    def level0(self, n):
        fac = self.dnp(bench.time_factor(n, self.T))
        return [self.pats[c] * fac if c < 2 else self.pats[c].copy() for c in range(3)]

    def step(self, n):
        import torch
        lv = self.level0(n)
        f = self.f
        for c in range(3):
            self.o[c][..., 0] = lv[c]
            self.do[c][..., 0].copy_(torch.from_numpy(np.asfortranarray(lv[c])))
        self.O.velprd(self.g, self.o[0], self.o[1], self.o[2], f.h, 1.0, 1.0, 1.0, 1.0, 1.0, f.u1, f.u2, f.u3)
        self.O.advec_dwarf(self.g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h, legacyoptmode=4, t_adv=1,
                           iord=3, nonos=1)
        d = self.d
        self.ws.velprd(self.do[0], self.do[1], self.do[2], d["h"], 1.0, 1.0, 1.0, 1.0, 1.0, d["u1"], d["u2"],
                       d["u3"])
        self.ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])

    def check(self, what):
        M, f = self.M, self.f
        got = W.interior(M.to_numpy(self.d["x"]))
        want = W.interior(f.x)
        err = float(np.abs(got - want).max() / np.abs(want).max())
        assert err <= 1e-12, "%s: psi L-inf relative error %g" % (what, err)
        np.testing.assert_array_equal(got, want, err_msg="%s: psi" % what)

    def check_all(self, what):
        self.check(what)
        M, f, n, m, l = self.M, self.f, self.f.np, self.f.mp, self.f.lp
        I, J, K = slice(1, 1 + n), slice(1, 1 + m), slice(1, 1 + l)
        np.testing.assert_array_equal(M.to_numpy(self.d["u1"])[1:n + 2, J, K], f.u1[1:n + 2, J, K], err_msg=what)
        np.testing.assert_array_equal(M.to_numpy(self.d["u2"])[I, 1:m + 2, K], f.u2[I, 1:m + 2, K], err_msg=what)
        np.testing.assert_array_equal(M.to_numpy(self.d["u3"])[I, J, 1:l + 2], f.u3[I, J, 1:l + 2], err_msg=what)
        for c in range(3):
            got = M.to_numpy(self.do[c])
            for lv in range(3):
                np.testing.assert_array_equal(W.interior(got[..., lv]), W.interior(self.o[c][..., lv]),
                                              err_msg="%s: momentum %d level %d" % (what, c, lv))

    def close(self):
        self.ws.close()


@pytest.mark.parametrize("dnp", [np.float64, np.float32], ids=["fp64", "fp32"])
def test_headline_chain_100_steps(M, oracle, dnp):
    """The headline chain on a 64x64x32 periodic grid for 100 steps (half of
    the flow's period T = 200 steps), bit for bit every 25 steps."""
    ch = Chain(M, oracle, 64, 64, 32, dnp)
    for n in range(100):
        ch.step(n)
        if (n + 1) % 25 == 0:
            ch.check("step %d" % (n + 1))
    ch.check_all("after 100 steps")
    ch.close()


def test_headline_chain_full_size(M, oracle):
    """The headline configuration itself, 512x512x128 FP64, for 5 steps
    against the OpenMP oracle on every host core."""
    import torch
    oracle.set_threads(os.cpu_count() or 1)
    try:
        ch = Chain(M, oracle, 512, 512, 128, np.float64)
        for n in range(5):
            ch.step(n)
        torch.cuda.synchronize()
        ch.check_all("512x512x128 after 5 steps")
        ch.close()
    finally:
        oracle.set_threads(min(8, os.cpu_count() or 1))


def test_kat_field_matches_oracle(M, oracle):
    """The reference's known-answer test (59^3 open walls, rotating sphere,
    gauge iord=2, 556 steps through advec_dwarf): the GPU field equals the
    oracle's bit for bit after every step has run, and its error norm is
    the reference's 0.0028."""
    f, meta = W.kat_rotating_sphere(59)
    g = f.copy()
    d = {k: M.fortran_device(getattr(f, k)) for k in ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}
    for _ in range(meta["nt"]):
        M.advec_dwarf(4, 1, False, False, f.np, f.mp, f.lp, f.ih, 0, f.ibcx, f.ibcy, f.ibcz, d["x"], d["bcx"],
                      d["bcy"], d["u1"], d["u2"], d["u3"], d["rhr"], d["h"], iord=2, nonos=1)
    out = M.to_numpy(d["x"])
    M.release_cached()
    oracle.advec_dwarf(oracle.grid(g.np, g.mp, g.lp, g.ih, g.ibcx, g.ibcy, g.ibcz), g.x, g.bcx, g.bcy, g.u1,
                       g.u2, g.u3, g.rhr, g.h, legacyoptmode=4, t_adv=1, iord=2, nonos=1, nsteps=meta["nt"])
    np.testing.assert_array_equal(W.interior(out), W.interior(g.x))
    np.testing.assert_array_equal(out, g.x)  # the halo the step leaves too
    err = W.error_l2(out, meta["xtest"], 59 ** 3, meta["timetot"])
    assert round(err, 4) == 0.0028, err
