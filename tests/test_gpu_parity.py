"""GPU parity of the CUDA path (through the C ABI) against the CPU oracle.

Strict-IEEE kernels: FP64 and FP32 results are compared bit for bit with the
oracle evaluated in the same precision; FP32 against FP64 within 1e-5
relative L-infinity."""
import os

import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


def dev(M, f):
    import torch
    dt = torch.float64 if f.dtype == np.float64 else torch.float32
    return {k: M.fortran_device(getattr(f, k), dtype=f.dtype) for k in
            ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}, dt


def run_gpu(M, f, opt=4, t_adv=1, iord=2, nonos=1, steps=1):
    """Steps through the Workspace API; returns psi as a Fortran numpy array."""
    d, _ = dev(M, f)
    prec = 64 if f.dtype == np.float64 else 32
    ws = M.Workspace(f.np, f.mp, f.lp, f.ih, f.ibcx, f.ibcy, f.ibcz, iord=iord if opt == 4 else 1,
                     nonos=nonos if opt == 4 else 0, gauge=1 if t_adv == 1 else 0, precision=prec)
    for _ in range(steps):
        ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], d["bcx"], d["bcy"])
    out = M.to_numpy(d["x"])
    ws.close()
    return out


def run_dwarf(M, f, opt=4, t_adv=1, iord=2, nonos=1, steps=1):
    """Steps through the advec_dwarf drop-in."""
    d, _ = dev(M, f)
    for _ in range(steps):
        M.advec_dwarf(opt, t_adv, False, False, f.np, f.mp, f.lp, f.ih, 0, f.ibcx, f.ibcy, f.ibcz,
                      d["x"], d["bcx"], d["bcy"], d["u1"], d["u2"], d["u3"], d["rhr"], d["h"],
                      iord=iord, nonos=nonos)
    return M.to_numpy(d["x"])


def _cases():
    from tests.golden import make_golden as G
    return G.CASES


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_golden_bit_exact(M, case):
    from tests.golden import make_golden as G
    ref = np.load(os.path.join(GOLDEN, case["name"] + ".npz"))
    f = G.build_case(case)
    out = run_gpu(M, f, opt=case["opt"], t_adv=case["t_adv"], iord=case["iord"], nonos=case["nonos"],
                  steps=case["steps"])
    # whole array: interior and the halo cells the step writes
    np.testing.assert_array_equal(out, ref["x"])


@pytest.mark.parametrize("case", _cases()[:4], ids=lambda c: c["name"])
def test_golden_through_advec_dwarf(M, case):
    from tests.golden import make_golden as G
    ref = np.load(os.path.join(GOLDEN, case["name"] + ".npz"))
    f = G.build_case(case)
    out = run_dwarf(M, f, opt=case["opt"], t_adv=case["t_adv"], iord=case["iord"], nonos=case["nonos"],
                    steps=case["steps"])
    np.testing.assert_array_equal(out, ref["x"])
    M.release_cached()


@pytest.mark.parametrize("n", [(1, 5, 4), (5, 1, 4), (6, 5, 1), (33, 17, 9), (2, 2, 2)])
@pytest.mark.parametrize("t_adv", [1, 2])
def test_edge_sizes_periodic(M, oracle, n, t_adv):
    """Thin and odd periodic domains (1-cell thick axes, sizes off the tile)."""
    f = W.random_fields(*n, ibc=(1, 1, 1), seed=sum(n) + t_adv)
    g = f.copy()
    out = run_gpu(M, f, t_adv=t_adv, iord=3, steps=3)
    oracle.advec_dwarf(oracle.grid(g.np, g.mp, g.lp, 1, 1, 1, 1), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3,
                       g.rhr, g.h, t_adv=t_adv, iord=3, nsteps=3)
    np.testing.assert_array_equal(out, g.x)


@pytest.mark.parametrize("n", [(2, 2, 2), (2, 7, 3), (35, 3, 2)])
def test_edge_sizes_reference_bc(M, oracle, n):
    f = W.random_fields(*n, ibc=(0, 0, 0), seed=sum(n))
    g = f.copy()
    out = run_gpu(M, f, t_adv=2, iord=2, steps=2)
    oracle.advec_dwarf(oracle.grid(g.np, g.mp, g.lp, 1, 0, 0, 0), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3,
                       g.rhr, g.h, t_adv=2, iord=2, nsteps=2)
    np.testing.assert_array_equal(out, g.x)


@pytest.mark.parametrize("unit", [False, True], ids=["variable_density", "unit_density"])
@pytest.mark.parametrize("n", [(40, 36, 17), (36, 40, 35)])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0), (1, 0, 1)])
def test_fp64_gauge_plane_chunks(M, oracle, n, ibc, unit):
    """FP64 gauge steps whose pseudo-velocity kernel marches chunks of 16
    planes: a last chunk of one plane (lp 17) or three (lp 35), the wall or
    wrapped planes 1 and lp, warps at the x and y edges, and warps whose faces
    are all of unit density or not; bit for bit against the oracle."""
    f = W.random_fields(*n, ibc=ibc, seed=sum(n) + 7 * ibc[0] + 3 * ibc[1])
    if unit:
        f.h[...] = 1.0
        f.rhr[...] = 1.0
    g = f.copy()
    out = run_gpu(M, f, t_adv=1, iord=3, steps=2)
    oracle.advec_dwarf(oracle.grid(g.np, g.mp, g.lp, 1, *ibc), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3,
                       g.rhr, g.h, t_adv=1, iord=3, nsteps=2)
    np.testing.assert_array_equal(out, g.x)


@pytest.mark.parametrize("t_adv", [1, 2])
def test_zero_background_fp64(M, oracle, t_adv):
    """Two balls on an exactly zero background in the deformational flow: most
    star extrema are +0 (the FP64 limiter keeps their key-order values once
    the star shows no NaN and no -0), 4 steps at iord 3, bit for bit against
    the oracle."""
    f = W.deformational(48, 40, 24, balls=True)
    g = f.copy()
    out = run_gpu(M, f, t_adv=t_adv, iord=3, steps=4)
    oracle.advec_dwarf(oracle.grid(48, 40, 24, 1, 1, 1, 1), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3,
                       g.rhr, g.h, t_adv=t_adv, iord=3, nsteps=4)
    np.testing.assert_array_equal(out, g.x)
    assert (W.interior(out) == 0).mean() > 0.5


@pytest.mark.parametrize("gauge", [1, 0])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_limiter_bounds_never_violated(M, gauge, ibc, dtype):
    """With h = rhr = 1, every step's output lies inside the running extrema
    the nonoscillatory limiter kept (x_in and every pass's stars), counted on
    the device after each of 5 steps; one cell pushed out of its bounds is
    counted."""
    import torch
    f = W.random_fields(40, 24, 12, ibc=ibc, seed=23, courant=0.4, sign_change=not gauge)
    f.h[...] = 1.0
    f.rhr[...] = 1.0
    f = f.astype(dtype) if dtype != np.float64 else f
    d, _ = dev(M, f)
    ws = M.Workspace(f.np, f.mp, f.lp, f.ih, *ibc, iord=3, nonos=1, gauge=gauge,
                     precision=64 if dtype == np.float64 else 32)
    tol = (1e-12 if dtype == np.float64 else 1e-5) * float(np.abs(f.x).max())
    for _ in range(5):
        ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], d["bcx"], d["bcy"])
        assert ws.bound_violations(d["x"], tol) == 0
    bad = d["x"].clone()
    bad[5, 6, 7] += 10.0
    assert ws.bound_violations(bad, tol) == 1
    ws.close()


def test_solid_body_100_steps_fp64(M, oracle):
    """64x64x32 periodic solid-body rotation, standard MPDATA, 100 steps:
    L-inf relative error <= 1e-12 (bit-exact expected), mass conserved."""
    f = W.solid_body_z()
    g = f.copy()
    out = run_gpu(M, f, t_adv=2, iord=2, steps=100)
    oracle.advec_dwarf(oracle.grid(64, 64, 32, 1, 1, 1, 1), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3,
                       g.rhr, g.h, t_adv=2, iord=2, nsteps=100)
    a, b = W.interior(out), W.interior(g.x)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    np.testing.assert_array_equal(a, b)
    m0 = float(W.interior(W.solid_body_z().x).sum())
    assert abs(float(a.sum()) - m0) <= 1e-12 * m0


def test_solid_body_fp32_vs_fp64(M):
    f64 = W.solid_body_z()
    f32 = W.solid_body_z(dtype=np.float32)
    a = W.interior(run_gpu(M, f64, t_adv=2, steps=100))
    b = W.interior(run_gpu(M, f32, t_adv=2, steps=100)).astype(np.float64)
    err = np.abs(a - b).max() / np.abs(a).max()
    assert err <= 1e-5, err


def test_kat_rotating_sphere_gpu(M):
    """The reference's known answer on the GPU: Error L2 norm 0.0028."""
    f, meta = W.kat_rotating_sphere(59)
    out = run_dwarf(M, f, opt=4, t_adv=1, iord=2, nonos=1, steps=meta["nt"])
    err = W.error_l2(out, meta["xtest"], 59 ** 3, meta["timetot"])
    assert round(err, 4) == 0.0028, err
    M.release_cached()


def test_predictor_matches_oracle(M, oracle):
    import torch
    for ibc in ((1, 1, 1), (0, 0, 0)):
        rng = np.random.default_rng(5)
        n, m, l, ih = 10, 9, 7, 1
        sh = W.shapes(n, m, l, ih)
        lev = sh["psi"] + (3,)
        ox, oy, oz, u, v, w = (np.asfortranarray(rng.uniform(-1, 1, lev)) for _ in range(6))
        h = np.asfortranarray(rng.uniform(0.8, 1.2, sh["psi"]))
        u1, u2, u3 = (W.zeros(sh[k]) for k in ("u1", "u2", "u3"))
        args = dict(dxi=0.5, dyi=0.25, dzi=2.0, dt=0.3, dt_ratio=0.75)
        dv = {k: M.fortran_device(a) for k, a in dict(ox=ox, oy=oy, oz=oz, u=u, v=v, w=w, h=h, u1=u1,
                                                      u2=u2, u3=u3).items()}
        ws = M.Workspace(n, m, l, ih, *ibc, precision=64)
        ws.velprd(dv["ox"], dv["oy"], dv["oz"], dv["h"], args["dxi"], args["dyi"], args["dzi"],
                  args["dt"], args["dt_ratio"], dv["u1"], dv["u2"], dv["u3"], dv["u"], dv["v"], dv["w"])
        torch.cuda.synchronize()
        g = oracle.grid(n, m, l, ih, *ibc)
        oracle.velprd(g, ox, oy, oz, h, args["dxi"], args["dyi"], args["dzi"], args["dt"],
                      args["dt_ratio"], u1, u2, u3, u, v, w)
        for k, a in dict(ox=ox, oy=oy, oz=oz, u=u, v=v, w=w).items():
            got = M.to_numpy(dv[k])
            np.testing.assert_array_equal(W.interior(got[..., 0]), W.interior(a[..., 0]), err_msg=k)
            for lv in (1, 2):
                np.testing.assert_array_equal(W.interior(got[..., lv]), W.interior(a[..., lv]),
                                              err_msg="%s level %d" % (k, lv))
        I, J, K = slice(ih, ih + n), slice(ih, ih + m), slice(ih, ih + l)
        np.testing.assert_array_equal(M.to_numpy(dv["u1"])[ih:ih + n + 1, J, K], u1[ih:ih + n + 1, J, K])
        np.testing.assert_array_equal(M.to_numpy(dv["u2"])[I, ih:ih + m + 1, K], u2[I, ih:ih + m + 1, K])
        np.testing.assert_array_equal(M.to_numpy(dv["u3"])[I, J, ih:ih + l + 1], u3[I, J, ih:ih + l + 1])
        ws.close()


def test_full_size_properties_fp64(M):
    """512x512x128 periodic deformational flow, gauge iord=3: mass conserved
    to round-off and every value finite (the flow is divergent, so no global
    bound applies)."""
    import torch
    f = W.deformational(512, 512, 128)
    d, _ = dev(M, f)
    m0 = float(d["x"][1:-1, 1:-1, 1:-1].sum())
    ws = M.Workspace(512, 512, 128, 1, 1, 1, 1, iord=3, nonos=1, gauge=1, precision=64)
    for _ in range(3):
        ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], d["bcx"], d["bcy"])
    torch.cuda.synchronize()
    xi = d["x"][1:-1, 1:-1, 1:-1]
    m1 = float(xi.sum())
    assert abs(m1 - m0) <= 1e-12 * abs(m0)
    assert bool(torch.isfinite(xi).all())
    ws.close()


def test_bad_arguments_raise(M):
    import torch
    ws = M.Workspace(8, 8, 8, 1, 1, 1, 1, precision=64)
    f = W.random_fields(8, 8, 8, ibc=(1, 1, 1))
    d, _ = dev(M, f)
    with pytest.raises(ValueError):
        ws.step(d["x"].float(), d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    with pytest.raises(ValueError):
        ws.step(d["x"][:-1], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    with pytest.raises(ValueError):
        ws.step(d["x"].cpu(), d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    ws.close()
    ws = M.Workspace(8, 8, 8, 1, 0, 0, 0, precision=64)
    with pytest.raises(M.MpdataError):  # open walls need bcx/bcy
        ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    ws.close()
    torch.cuda.synchronize()


@pytest.mark.parametrize("ibc", [(0, 0, 0), (1, 1, 1), (1, 0, 0)])
@pytest.mark.parametrize("liner", [0, 1])
def test_rho_gauge_density_step(M, oracle, ibc, liner):
    """mpdata3d_rho_gauge_gpubc: every output (x_in, x_incomp, rhoadv, rhr,
    pexr1, pexr2, mass fluxes u1..u3, the three momentum levels) bit for bit."""
    import torch
    n, m, l, ih = 11, 9, 7, 1
    rng = np.random.default_rng(17 + liner + 2 * sum(ibc))
    sh = W.shapes(n, m, l, ih)
    lev = sh["psi"] + (3,)
    arrs = dict(ox=rng.uniform(-0.3, 0.3, lev), oy=rng.uniform(-0.3, 0.3, lev), oz=rng.uniform(-0.3, 0.3, lev),
                u1=np.zeros(sh["u1"]), u2=np.zeros(sh["u2"]), u3=np.zeros(sh["u3"]),
                x_in=rng.uniform(0.5, 1.5, sh["psi"]), x_incomp=rng.uniform(0.5, 1.5, sh["psi"]),
                h=rng.uniform(0.8, 1.2, sh["psi"]), rhoadv=np.zeros(sh["psi"]), rhr=np.zeros(sh["psi"]),
                pexe=rng.uniform(0.9, 1.1, sh["psi"]), pexr1=np.zeros(sh["psi"]), pexr2=np.zeros(sh["psi"]),
                bcx=rng.uniform(0.5, 1.5, sh["bcx"]), bcy=rng.uniform(0.5, 1.5, sh["bcy"]))
    arrs = {k: np.asfortranarray(v) for k, v in arrs.items()}
    dv = {k: M.fortran_device(v) for k, v in arrs.items()}
    ws = M.Workspace(n, m, l, ih, *ibc, iord=2, nonos=1, gauge=1, precision=64)
    sc = dict(dxi=1.0, dyi=1.0, dzi=1.0, dt=1.0, dt_ratio=1.0)
    ws.mpdata3d_rho_gauge_gpubc(dv["ox"], dv["oy"], dv["oz"], dv["u1"], dv["u2"], dv["u3"], dv["x_in"],
                                dv["x_incomp"], dv["h"], dv["rhoadv"], dv["rhr"], dv["pexe"], dv["pexr1"],
                                dv["pexr2"], bcx=dv["bcx"], bcy=dv["bcy"], liner=liner, **sc)
    torch.cuda.synchronize()
    oracle.rho_gauge(oracle.grid(n, m, l, ih, *ibc), arrs["ox"], arrs["oy"], arrs["oz"], arrs["u1"], arrs["u2"],
                     arrs["u3"], arrs["x_in"], arrs["x_incomp"], arrs["h"], arrs["rhoadv"], arrs["rhr"],
                     arrs["pexe"], arrs["pexr1"], arrs["pexr2"], arrs["bcx"], arrs["bcy"], liner=liner, **sc)
    I, J, K = slice(ih, ih + n), slice(ih, ih + m), slice(ih, ih + l)
    for k in ("x_in", "x_incomp", "rhoadv", "rhr", "pexr1", "pexr2"):
        np.testing.assert_array_equal(W.interior(M.to_numpy(dv[k])), W.interior(arrs[k]), err_msg=k)
    np.testing.assert_array_equal(M.to_numpy(dv["x_in"]), arrs["x_in"], err_msg="x_in with halo")
    np.testing.assert_array_equal(M.to_numpy(dv["u1"])[ih:ih + n + 1, J, K], arrs["u1"][ih:ih + n + 1, J, K])
    np.testing.assert_array_equal(M.to_numpy(dv["u2"])[I, ih:ih + m + 1, K], arrs["u2"][I, ih:ih + m + 1, K])
    np.testing.assert_array_equal(M.to_numpy(dv["u3"])[I, J, ih:ih + l + 1], arrs["u3"][I, J, ih:ih + l + 1])
    ws.close()
