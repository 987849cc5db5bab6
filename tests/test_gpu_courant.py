"""Courant control on the GPU against the oracle, bit for bit: the seven
maxima of compute_courants (common/diagutils.f90:588-672) and every branch
of velprd_driver (advection/src_algorithms/velprd_driver.f90:16-270) over
three consecutive calls, FP64 and FP32, open and periodic boundaries.  Every
array (all momentum levels with their halos, the physical velocities, the
C-grid Courant numbers) and every scalar the driver updates must match."""
import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W

pytestmark = pytest.mark.gpu

N = (14, 10, 8)


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


def to_dev(M, st):
    return {k: M.fortran_device(v) for k, v in st.items()}


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("level", [1, 2])
def test_courants_match_oracle(M, oracle, dtype, level):
    st = W.predictor_case(*N, courant=1.9, seed=11, dtype=dtype)
    g = oracle.grid(*N, 1, 0, 0, 0)
    if level == 2:
        oracle.velprd(g, st["ox"], st["oy"], st["oz"], st["h"], 1.0, 1.0, 1.0, 1.0, 1.0,
                      st["uadv"], st["vadv"], st["wadv"])
    want = oracle.compute_courants(g, level, st["ox"], st["oy"], st["oz"], st["h"], 0.5, 0.25, 2.0, 1.5)
    d = to_dev(M, st)
    got = M.compute_courants(level, d["ox"], d["oy"], d["oz"], d["h"], 0.5, 0.25, 2.0, 1.5, *N, 1)
    np.testing.assert_array_equal(np.array(got, dtype=dtype), want)


MODES = {
    "plain_n": dict(),
    "plain_nphlf": dict(lcrdiag_nphlf=1),
    "substep": dict(lsubstepping=1, crmaxlim=0.9),
    "substep_nphlf_split": dict(lsubstepping=1, crmaxlim=0.9, lcrdiag_nphlf=1, lvertsplit=1),
    "substep_split": dict(lsubstepping=1, crmaxlim=0.9, lvertsplit=1),
    "adapt": dict(ltimeadapt=1, crmaxlim=0.8, dtmax=3.0),
    "adapt_nphlf_split": dict(ltimeadapt=1, crmaxlim=0.8, dtmax=3.0, lcrdiag_nphlf=1, lvertsplit=1),
}


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("ibc", [(0, 0, 0), (1, 1, 1)])
@pytest.mark.parametrize("mode", sorted(MODES))
def test_driver_matches_oracle(M, oracle, mode, ibc, dtype):
    import torch
    st = W.predictor_case(*N, courant=2.4, seed=13, dtype=dtype)
    d = to_dev(M, st)
    g = oracle.grid(*N, 1, *ibc)
    base = dict(nsubsteps=1, nsubsteps_o=1, dtn=1.0, dtnold=1.0, lsubstepping=0, ltimeadapt=0, lvertsplit=0,
                lcrdiag_nphlf=0, crmaxlim=1.0, dtmax=10.0)
    base.update(MODES[mode])
    so, sg = dict(base), dict(base)
    for call in range(3):
        rc, diag_o = oracle.velprd_driver(g, so, st["ox"], st["oy"], st["oz"], st["uadv"], st["vadv"],
                                          st["wadv"], st["h"], 1.0, 1.0, 1.0, 1.0, u=st["u"], v=st["v"],
                                          w=st["w"])
        assert rc == 0, (mode, call)
        diag_g = M.velprd_driver(sg, d["ox"], d["oy"], d["oz"], d["u"], d["v"], d["w"], d["uadv"], d["vadv"],
                                 d["wadv"], d["h"], 0, *ibc, *N, 1, 1.0, 1.0, 1.0, 1.0)
        torch.cuda.synchronize()
        assert sg == so, (mode, call, sg, so)
        np.testing.assert_array_equal(np.array(diag_g), diag_o)
        for k in st:
            np.testing.assert_array_equal(M.to_numpy(d[k]), st[k], err_msg="%s call %d: %s" % (mode, call, k))


def test_driver_reports_fatal_courant(M):
    st = W.predictor_case(*N, courant=40.0, seed=17)
    d = to_dev(M, st)
    s = dict(nsubsteps=2, nsubsteps_o=2, dtn=0.5, dtnold=0.5, lsubstepping=1, ltimeadapt=0, lvertsplit=0,
             lcrdiag_nphlf=0, crmaxlim=1.0, dtmax=10.0)
    with pytest.raises(M.MpdataError) as e:
        M.velprd_driver(s, d["ox"], d["oy"], d["oz"], d["u"], d["v"], d["w"], d["uadv"], d["vadv"], d["wadv"],
                        d["h"], 0, 0, 0, 0, *N, 1, 1.0, 1.0, 1.0, 1.0)
    assert e.value.code == -9
