"""GPU adjoint of the MPDATA step (gauge and standard forms, iord 2 to 4) against
the oracle's FP64 un-checkpointed adjoint (reverse-mode AD of the oracle's
own step): single-step reverse, sqrt(N)-checkpointed run, the dot-product
test against the oracle's tangent-linear model, and central finite
differences of J computed on the GPU."""
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


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def problem(n, ibc, seed, sign_change=False):
    f = W.random_fields(*n, ibc=ibc, seed=seed, courant=0.25, sign_change=sign_change)
    rng = np.random.default_rng(seed + 1)
    target = np.asfortranarray(f.x * 0.9 + rng.uniform(-0.05, 0.05, f.x.shape))
    return f, target


def gpu_adjoint_run(M, f, target, nsteps, nonos=1, interval=0, precision=64, iord=2, gauge=1):
    import torch
    dt = np.float64 if precision == 64 else np.float32
    d = {k: M.fortran_device(getattr(f, k), dtype=dt) for k in ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}
    tg = M.fortran_device(target, dtype=dt)
    gx = torch.zeros_like(d["x"])
    gu = [torch.zeros_like(d[k]) for k in ("u1", "u2", "u3")]
    ws = M.Workspace(f.np, f.mp, f.lp, f.ih, f.ibcx, f.ibcy, f.ibcz, iord=iord, nonos=nonos, gauge=gauge,
                     precision=precision)
    J, peak = ws.adjoint_run(nsteps, d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], tg, gx, *gu,
                             d["bcx"], d["bcy"], interval=interval)
    out = (J, M.to_numpy(d["x"]), M.to_numpy(gx), *[M.to_numpy(t) for t in gu], peak)
    ws.close()
    return out


def oracle_adjoint(oracle, f, target, nsteps, nonos=1, iord=2, gauge=1):
    g = oracle.grid(f.np, f.mp, f.lp, f.ih, f.ibcx, f.ibcy, f.ibcz)
    return oracle.adjoint(g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h, target, t_adv=1 if gauge else 2,
                          iord=iord, nonos=nonos, nsteps=nsteps)


@pytest.mark.parametrize("iord", [2, 3, 4])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0), (1, 0, 0)])
@pytest.mark.parametrize("nonos", [1, 0])
def test_single_step_adjoint_matches_oracle(M, oracle, ibc, nonos, iord):
    """Every corrective pass reversed: the later passes' "a" velocities are
    the previous pass's limited ones and their bounds continue the previous
    pass's running extrema."""
    f, target = problem((12, 10, 8), ibc, seed=31)
    J, xN, gx, g1, g2, g3, _ = gpu_adjoint_run(M, f, target, 1, nonos=nonos, iord=iord)
    Jo, xNo, gxo, g1o, g2o, g3o = oracle_adjoint(oracle, f, target, 1, nonos=nonos, iord=iord)
    np.testing.assert_array_equal(W.interior(xN), W.interior(xNo))
    assert abs(J - Jo) <= 1e-13 * abs(Jo)
    assert rel(gx, gxo) <= 1e-12
    for a, b in ((g1, g1o), (g2, g2o), (g3, g3o)):
        assert rel(a, b) <= 1e-12


@pytest.mark.parametrize("iord", [2, 3])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)])
def test_checkpointed_run_matches_unCheckpointed_oracle(M, oracle, ibc, iord):
    """7 steps, checkpoints every 3 (segments of 3, 3, 1) against the
    oracle's un-checkpointed FP64 adjoint."""
    f, target = problem((12, 10, 8), ibc, seed=41)
    J, _, gx, g1, g2, g3, peak = gpu_adjoint_run(M, f, target, 7, interval=3, iord=iord)
    Jo, _, gxo, g1o, g2o, g3o = oracle_adjoint(oracle, f, target, 7, iord=iord)
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert rel(gx, gxo) <= 1e-11
    for a, b in ((g1, g1o), (g2, g2o), (g3, g3o)):
        assert rel(a, b) <= 1e-11
    assert peak > 0
    # default interval ceil(sqrt(7)) = 3 gives the same gradients
    J2, _, gx2, *_ = gpu_adjoint_run(M, f, target, 7, iord=iord)
    assert rel(gx2, gx) <= 1e-13


@pytest.mark.parametrize("iord", [2, 3])
def test_dot_product_against_tangent_linear(M, oracle, iord):
    """<dx0, dJ/dx0> + <du, dJ/du> from the GPU adjoint equals the oracle
    tangent-linear derivative of J along (dx0, du) to 1e-12."""
    f, target = problem((12, 10, 8), (1, 1, 1), seed=51)
    nsteps = 4
    J, _, gx, g1, g2, g3, _ = gpu_adjoint_run(M, f, target, nsteps, iord=iord)
    rng = np.random.default_rng(52)
    for trial in range(3):
        dx = np.asfortranarray(rng.uniform(-1, 1, f.x.shape))
        du = [np.asfortranarray(rng.uniform(-1, 1, a.shape)) for a in (f.u1, f.u2, f.u3)]
        tl = oracle.tangent_dJ(oracle.grid(12, 10, 8, 1, 1, 1, 1), f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr,
                               f.h, target, dx, *du, nsteps=nsteps, iord=iord)
        dot = (gx * dx).sum() + (g1 * du[0]).sum() + (g2 * du[1]).sum() + (g3 * du[2]).sum()
        assert abs(dot - tl) <= 1e-12 * abs(tl), (trial, dot, tl)


def test_central_finite_differences(M):
    """J evaluated by the GPU forward step: (J(p+eps d) - J(p-eps d))/(2 eps)
    against <d, grad J> for random directions in psi_0 and in u, eps=1e-6."""
    import torch
    f, target = problem((16, 12, 8), (1, 1, 1), seed=61)
    nsteps = 3
    _, _, gx, g1, g2, g3, _ = gpu_adjoint_run(M, f, target, nsteps)

    def J_of(ff):
        d = {k: M.fortran_device(getattr(ff, k)) for k in ("x", "u1", "u2", "u3", "h", "rhr")}
        ws = M.Workspace(ff.np, ff.mp, ff.lp, 1, 1, 1, 1, iord=2, nonos=1, gauge=1, precision=64)
        for _ in range(nsteps):
            ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
        torch.cuda.synchronize()
        ws.close()
        r = W.interior(M.to_numpy(d["x"])) - W.interior(target)
        return 0.5 * float((r * r).sum())

    rng = np.random.default_rng(62)
    eps = 1e-6
    worst = 0.0
    for trial in range(8):
        dx = np.zeros_like(f.x)
        W.interior(dx)[...] = rng.uniform(-1, 1, (16, 12, 8))
        du = [np.zeros_like(a) for a in (f.u1, f.u2, f.u3)]
        if trial % 2:  # velocity directions (interior faces 1..n, periodic)
            du[0][1:17, 1:13, 1:9] = rng.uniform(-0.05, 0.05, (16, 12, 8))
            du[1][1:17, 1:13, 1:9] = rng.uniform(-0.05, 0.05, (16, 12, 8))
            du[2][1:17, 1:13, 1:9] = rng.uniform(-0.05, 0.05, (16, 12, 8))
        fp, fm = f.copy(), f.copy()
        for a, b, c in ((fp.x, fm.x, dx), (fp.u1, fm.u1, du[0]), (fp.u2, fm.u2, du[1]), (fp.u3, fm.u3, du[2])):
            a += eps * c
            b -= eps * c
        fd = (J_of(fp) - J_of(fm)) / (2 * eps)
        dot = (gx * dx).sum() + (g1 * du[0]).sum() + (g2 * du[1]).sum() + (g3 * du[2]).sum()
        worst = max(worst, abs(fd - dot) / abs(dot))
    assert worst <= 1e-6, worst


def test_fp32_adjoint_tracks_fp64(M):
    f, target = problem((12, 10, 8), (1, 1, 1), seed=71)
    _, _, gx64, g164, *_ = gpu_adjoint_run(M, f, target, 3)
    _, _, gx32, g132, *_ = gpu_adjoint_run(M, f, target, 3, precision=32)
    assert rel(gx32.astype(np.float64), gx64) <= 1e-4
    assert rel(g132.astype(np.float64), g164) <= 1e-4


@pytest.mark.parametrize("iord", [2, 3])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0), (0, 1, 0)])
@pytest.mark.parametrize("nonos", [1, 0])
def test_standard_form_adjoint_matches_oracle(M, oracle, ibc, nonos, iord):
    """Standard form (t_adv=2) on a field that changes sign: vdyfa/vcorra
    with their absolute values, the unlimited donor fluxes of the bounds, the
    sign-aware limited velocity and the donor fluxes of x/rhr."""
    f, target = problem((12, 10, 8), ibc, seed=81, sign_change=True)
    J, xN, gx, g1, g2, g3, _ = gpu_adjoint_run(M, f, target, 1, nonos=nonos, iord=iord, gauge=0)
    Jo, xNo, gxo, g1o, g2o, g3o = oracle_adjoint(oracle, f, target, 1, nonos=nonos, iord=iord, gauge=0)
    np.testing.assert_array_equal(W.interior(xN), W.interior(xNo))
    assert abs(J - Jo) <= 1e-13 * abs(Jo)
    assert rel(gx, gxo) <= 1e-12
    for a, b in ((g1, g1o), (g2, g2o), (g3, g3o)):
        assert rel(a, b) <= 1e-12


def test_standard_form_checkpointed_run(M, oracle):
    f, target = problem((12, 10, 8), (1, 1, 1), seed=91, sign_change=True)
    J, _, gx, g1, g2, g3, _ = gpu_adjoint_run(M, f, target, 5, interval=2, iord=2, gauge=0)
    Jo, _, gxo, g1o, g2o, g3o = oracle_adjoint(oracle, f, target, 5, iord=2, gauge=0)
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert rel(gx, gxo) <= 1e-11
    for a, b in ((g1, g1o), (g2, g2o), (g3, g3o)):
        assert rel(a, b) <= 1e-11


def test_adjoint_rejects_unsupported(M):
    import torch
    ws = M.Workspace(8, 8, 8, 1, 1, 1, 1, iord=1, nonos=1, gauge=1, precision=64)
    z = [M.fortran_empty(ws.shapes[k], torch.float64) for k in ("psi", "u1", "u2", "u3", "psi", "psi", "psi")]
    with pytest.raises(M.MpdataError):  # iord=1 is the upwind step alone: nothing to reverse here
        ws.step_adjoint(z[0], z[1], z[2], z[3], z[4], z[5], z[6], z[1].clone(), z[2].clone(), z[3].clone())
    ws.close()


@pytest.mark.parametrize("perturb", [False, True], ids=["unit", "one_cell_off"])
@pytest.mark.parametrize("iord", [2, 3])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)])
@pytest.mark.parametrize("gauge", [1, 0])
def test_interior_warps_adjoint_matches_oracle(M, oracle, gauge, ibc, iord, perturb):
    """An x extent of 80 gives whole warps away from every wall, whose record
    and reverse kernels read without index maps, take the pair sums (FP64
    gauge) and, where h = rhr = 1 across the warp, drop the density factors.
    One perturbed cell puts unit and non-unit warps side by side."""
    f, target = problem((80, 10, 8), ibc, seed=41 + iord, sign_change=not gauge)
    f.h[...] = 1.0
    f.rhr[...] = 1.0
    if perturb:
        f.h[45, 5, 4] = 1.125
        f.rhr[45, 5, 4] = 0.875
    J, xN, gx, g1, g2, g3, _ = gpu_adjoint_run(M, f, target, 2, iord=iord, gauge=gauge)
    Jo, xNo, gxo, g1o, g2o, g3o = oracle_adjoint(oracle, f, target, 2, iord=iord, gauge=gauge)
    np.testing.assert_array_equal(W.interior(xN), W.interior(xNo))
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert rel(gx, gxo) <= 1e-11
    for a, b in ((g1, g1o), (g2, g2o), (g3, g3o)):
        assert rel(a, b) <= 1e-11
