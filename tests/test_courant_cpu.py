"""Courant control of the predictor on the CPU: the oracle's compute_courants
(common/diagutils.f90:588-672) against a numpy restatement, and its
velprd_driver (advection/src_algorithms/velprd_driver.f90:16-270) in each
branch: plain, substepping, adaptive time step, error exits.  Plus the C
ABI's argument checks, which return before any CUDA call."""
import ctypes

import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W


def np_courants(st, level, dt=1.0, ih=1):
    sl = (slice(ih, -ih),) * 3
    if level == 1:
        a, b, c = (np.abs((dt * 1.0) * st[n][..., 0][sl]) for n in ("ox", "oy", "oz"))
    else:
        dinv = 1.0 / st["h"][sl]
        a, b, c = (np.abs(st[n][..., 1][sl] * dinv) for n in ("ox", "oy", "oz"))
    return np.array([(a + b + c).max(), (a + b).max(), (a + c).max(), (b + c).max(), a.max(), b.max(), c.max()])


def state(**kw):
    s = dict(nsubsteps=1, nsubsteps_o=1, dtn=1.0, dtnold=1.0, lsubstepping=0, ltimeadapt=0, lvertsplit=0,
             lcrdiag_nphlf=0, crmaxlim=1.0, dtmax=10.0)
    s.update(kw)
    return s


def run_driver(oracle, st, g, s, dt=1.0):
    return oracle.velprd_driver(g, s, st["ox"], st["oy"], st["oz"], st["uadv"], st["vadv"], st["wadv"], st["h"],
                                1.0, 1.0, 1.0, dt, u=st["u"], v=st["v"], w=st["w"])


@pytest.mark.parametrize("level", [1, 2])
def test_oracle_courants_match_numpy(oracle, level):
    st = W.predictor_case(10, 8, 6, courant=1.7, seed=3)
    g = oracle.grid(10, 8, 6, 1, 0, 0, 0)
    if level == 2:  # fill level 1 first, as the driver does
        oracle.velprd(g, st["ox"], st["oy"], st["oz"], st["h"], 1.0, 1.0, 1.0, 1.0, 1.0,
                      st["uadv"], st["vadv"], st["wadv"])
    cr = oracle.compute_courants(g, level, st["ox"], st["oy"], st["oz"], st["h"], 1.0, 1.0, 1.0, 1.0)
    np.testing.assert_array_equal(cr, np_courants(st, level))


def test_plain_driver_is_the_predictor(oracle):
    """No substepping, no adaptivity, Courant at n: velprd_traj0 + velprdA_to_C
    + the roll with dt_ratio 1 (velprd_driver.f90:236-270)."""
    a = W.predictor_case(10, 8, 6, courant=0.7, seed=4)
    b = {k: v.copy(order="F") for k, v in a.items()}
    g = oracle.grid(10, 8, 6, 1, 0, 0, 0)
    rc, diag = run_driver(oracle, a, g, state())
    assert rc == 0 and diag[8] == 1.0
    oracle.velprd(g, b["ox"], b["oy"], b["oz"], b["h"], 1.0, 1.0, 1.0, 1.0, 1.0, b["uadv"], b["vadv"], b["wadv"],
                  u=b["u"], v=b["v"], w=b["w"])
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("lcrdiag_nphlf", [0, 1])
@pytest.mark.parametrize("lvertsplit", [0, 1])
def test_substepping_brings_courant_below_limit(oracle, lcrdiag_nphlf, lvertsplit):
    st = W.predictor_case(12, 10, 8, courant=2.6, seed=5)
    g = oracle.grid(12, 10, 8, 1, 1, 1, 1)
    s = state(lsubstepping=1, lvertsplit=lvertsplit, lcrdiag_nphlf=lcrdiag_nphlf, crmaxlim=0.9)
    rc, diag = run_driver(oracle, st, g, s)
    assert rc == 0
    n = s["nsubsteps"]
    assert n >= 2 and s["nsubsteps_o"] == n
    assert s["dtn"] == 1.0 / n and s["dtnold"] == s["dtn"]
    assert diag[7] <= 0.9  # cr_for_dt of the accepted substep
    # the next call, inside substepping, keeps nsubsteps (velprd_driver.f90:125-126)
    rc, diag = run_driver(oracle, st, g, s)
    assert rc == 0 and s["nsubsteps"] >= n


def test_adaptive_step_lowers_dt(oracle):
    st = W.predictor_case(12, 10, 8, courant=2.0, seed=6)
    g = oracle.grid(12, 10, 8, 1, 0, 0, 0)
    s = state(ltimeadapt=1, crmaxlim=0.8, dtmax=5.0)
    rc, diag = run_driver(oracle, st, g, s)
    assert rc == 0
    assert s["dtn"] < 1.0 and s["dtnold"] == 1.0
    assert diag[7] <= 0.8
    assert diag[8] == s["dtn"] / s["dtnold"]


def test_driver_error_exits(oracle):
    st = W.predictor_case(8, 8, 6, courant=40.0, seed=7)
    g = oracle.grid(8, 8, 6, 1, 0, 0, 0)
    rc, _ = run_driver(oracle, st, g, state(lsubstepping=1, ltimeadapt=1))
    assert rc == -2  # STOP "substepping and adaptivity not supported together" (:74)
    rc, _ = run_driver(oracle, st, g, state(lsubstepping=1, nsubsteps=2, nsubsteps_o=2))
    assert rc == -9  # STOP 'Courant > 1 for nsubsteps >1' (:123): 40/2 > 10


def test_capi_driver_checks_without_gpu(native_lib):
    """Argument checks return before any CUDA call."""
    lib = native_lib
    ns, nso = ctypes.c_int(1), ctypes.c_int(1)
    dtn, dtnold = ctypes.c_double(1.0), ctypes.c_double(1.0)
    fake = ctypes.c_void_p(256)
    args = lambda lsub, ladapt, ipoles, arrs: (
        ctypes.byref(ns), ctypes.byref(nso), lsub, ctypes.byref(dtn), ctypes.byref(dtnold), ladapt, 0, 0, 1.0, 1.0,
        *arrs, ipoles, 0, 0, 0, 8, 8, 6, 1, 1.0, 1.0, 1.0, 1.0, None, None)
    ten = [fake] * 10
    assert lib.mpdata_velprd_driver_f64(*args(1, 1, 0, ten)) == -2
    assert lib.mpdata_velprd_driver_f64(*args(0, 0, 1, ten)) == -7
    assert lib.mpdata_velprd_driver_f64(*args(0, 0, 0, [None] * 10)) == -3
    cr = (ctypes.c_double * 7)()
    assert lib.mpdata_compute_courants_f64(cr, fake, fake, fake, fake, 3, 1.0, 1.0, 1.0, 1.0, 8, 8, 6, 1,
                                           None) == -2
    assert lib.mpdata_strerror(-9).decode().startswith("Courant control failed")
