"""Adjoint of the density step after its predictor (mpdata_rho_gauge_adjoint_*)
through the C ABI.

The density step (mpdata3d-rho-gauge-gpubc.f90:106-606) advances psi with
the C-grid Courant numbers of the predictor and outputs psi, x_incomp,
pexr1, pexr2, rhr and the mass fluxes u1..u3.  The reverse is checked
- against the oracle's reverse-mode AD of the same step (orc_rho_adjoint_f64,
  itself pinned by central differences on the host) at iord 2, the
  reference's one corrective pass, in FP64 (1e-12) and FP32 (1e-4), with and
  without cotangents on the mass fluxes;
- end to end at iord 3 (a pass count the reference's density step does not
  have): the gradient with respect to psi, x_incomp, pexe and the A-grid
  momenta, composed with the predictor adjoint, against central differences
  of the GPU's own predictor + density step (limiter off, Courant numbers
  away from 0).
"""
import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W

pytestmark = pytest.mark.gpu

OUT_PSI = ("x", "xc", "p1", "p2", "rhr")
OUT_U = ("u1", "u2", "u3")


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def problem(n, seed):
    rng = np.random.default_rng(seed)
    sh = W.shapes(*n, 1)
    f = {k: np.asfortranarray(rng.uniform(1.0, 2.0, sh["psi"])) for k in ("x", "xc")}
    f["h"] = np.asfortranarray(rng.uniform(0.8, 1.2, sh["psi"]))
    f["pexe"] = np.asfortranarray(rng.uniform(0.5, 1.5, sh["psi"]))
    for k in OUT_U:
        f[k] = np.asfortranarray(0.2 + rng.uniform(-0.05, 0.05, sh[k]))
    f["bcx"] = np.asfortranarray(rng.uniform(1.0, 2.0, (n[1], n[2], 2)))
    f["bcy"] = np.asfortranarray(rng.uniform(1.0, 2.0, (n[0], n[2], 2)))
    return sh, f


def cotangents(n, sh, seed):
    rng = np.random.default_rng(seed)
    I, J, K = slice(1, 1 + n[0]), slice(1, 1 + n[1]), slice(1, 1 + n[2])
    lam = {}
    for k in OUT_PSI:
        a = np.zeros(sh["psi"])
        a[I, J, K] = rng.uniform(-1, 1, n)
        lam[k] = np.asfortranarray(a)
    for k, fs in (("u1", (slice(1, 2 + n[0]), J, K)), ("u2", (I, slice(1, 2 + n[1]), K)),
                  ("u3", (I, J, slice(1, 2 + n[2])))):
        a = np.zeros(sh[k])
        a[fs] = rng.uniform(-1, 1, a[fs].shape)
        lam[k] = np.asfortranarray(a)
    return lam


def gpu_rho_adjoint(M, n, ibc, f, lam, iord=2, nonos=1, precision=64, mass=True):
    import torch
    dt = np.float64 if precision == 64 else np.float32
    dev = lambda a: M.fortran_device(a, dtype=dt)
    ws = M.Workspace(*n, 1, *ibc, iord=iord, nonos=nonos, gauge=1, precision=precision)
    lx = dev(lam["x"])
    gu = [dev(np.zeros_like(f[k])) for k in OUT_U]
    gxc, gpe = dev(np.zeros_like(f["x"])), dev(np.zeros_like(f["x"]))
    lm = [dev(lam[k]) for k in OUT_U] if mass else [None] * 3
    ws.rho_gauge_adjoint(*[dev(f[k]) for k in OUT_U], dev(f["x"]), dev(f["xc"]), dev(f["h"]), dev(f["pexe"]),
                         lx, *gu, gxc, gpe, l_u1=lm[0], l_u2=lm[1], l_u3=lm[2], l_xincomp=dev(lam["xc"]),
                         l_pexr1=dev(lam["p1"]), l_pexr2=dev(lam["p2"]), l_rhr=dev(lam["rhr"]),
                         bcx=dev(f["bcx"]), bcy=dev(f["bcy"]))
    torch.cuda.synchronize()
    ws.close()
    return [M.to_numpy(t).astype(np.float64) for t in (lx, *gu, gxc, gpe)]


def oracle_rho_adjoint(O, n, ibc, f, lam, mass=True):
    g = O.grid(*n, 1, *ibc)
    lm = [lam[k] for k in OUT_U] if mass else [None] * 3
    return O.rho_adjoint(g, f["u1"], f["u2"], f["u3"], f["x"], f["xc"], f["h"], f["pexe"], f["bcx"], f["bcy"],
                         l_x=lam["x"], l_u1=lm[0], l_u2=lm[1], l_u3=lm[2], l_xinc=lam["xc"], l_p1=lam["p1"],
                         l_p2=lam["p2"], l_rhr=lam["rhr"])


@pytest.mark.parametrize("mass", [True, False], ids=["with_mass_fluxes", "no_mass_fluxes"])
@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0), (1, 0, 0)])
def test_rho_adjoint_matches_oracle_ad(M, oracle, ibc, mass):
    n = (12, 10, 8)
    sh, f = problem(n, 61 + sum(ibc))
    lam = cotangents(n, sh, 71 + sum(ibc))
    got = gpu_rho_adjoint(M, n, ibc, f, lam, mass=mass)
    want = oracle_rho_adjoint(oracle, n, ibc, f, lam, mass=mass)
    for name, a, b in zip(("psi", "u1", "u2", "u3", "x_incomp", "pexe"), got, want):
        assert rel(a, b) <= 1e-12, (name, rel(a, b))


def test_rho_adjoint_fp32_against_fp64_oracle(M, oracle):
    n, ibc = (12, 10, 8), (1, 1, 1)
    sh, f = problem(n, 81)
    lam = cotangents(n, sh, 82)
    got = gpu_rho_adjoint(M, n, ibc, f, lam, precision=32)
    want = oracle_rho_adjoint(oracle, n, ibc, f, lam)
    for name, a, b in zip(("psi", "u1", "u2", "u3", "x_incomp", "pexe"), got, want):
        assert rel(a, b) <= 1e-4, (name, rel(a, b))


def test_rho_adjoint_rejects_bad_calls(M):
    import torch
    n = (8, 6, 4)
    sh, f = problem(n, 5)
    dev = lambda a: M.fortran_device(a)
    ws = M.Workspace(*n, 1, 1, 1, 1, iord=2, nonos=1, gauge=0, precision=64)   # standard form
    z = lambda k: dev(np.zeros(sh[k]))
    args = [dev(f[k]) for k in OUT_U] + [dev(f["x"]), dev(f["xc"]), dev(f["h"]), dev(f["pexe"]), z("psi")]
    args += [z("u1"), z("u2"), z("u3"), z("psi"), z("psi")]
    with pytest.raises(M.MpdataError):
        ws.rho_gauge_adjoint(*args)
    ws.close()
    ws = M.Workspace(*n, 1, 1, 1, 1, iord=2, nonos=1, gauge=1, precision=64)
    with pytest.raises(M.MpdataError):   # mass-flux cotangents come three together
        ws.rho_gauge_adjoint(*args, l_u1=z("u1"))
    ws.close()
    torch.cuda.synchronize()


def test_density_step_gradient_through_the_predictor(M):
    """iord 3, limiter off: J = <l, outputs> of predictor + density step;
    the gradient with respect to psi, x_incomp, pexe and the A-grid momenta
    (levels 0 and 2), from the density step's adjoint and the predictor's,
    against central differences of the GPU forward (eps = 1e-4) along 6
    seeded unit directions."""
    import torch
    n, ibc = (16, 12, 8), (1, 1, 1)
    rng = np.random.default_rng(91)
    sh, f = problem(n, 92)
    lam = cotangents(n, sh, 93)
    I, J, K = slice(1, 1 + n[0]), slice(1, 1 + n[1]), slice(1, 1 + n[2])
    lev = [np.zeros(sh["psi"] + (3,), order="F") for _ in range(3)]
    for a in lev:  # drift plus noise: every Courant number stays away from 0
        a[I, J, K, 0] = 0.2 + rng.uniform(-0.05, 0.05, n)
        a[I, J, K, 2] = 0.2 + rng.uniform(-0.05, 0.05, n)
    dev = lambda a: M.fortran_device(np.asfortranarray(a))
    ws = M.Workspace(*n, 1, *ibc, iord=3, nonos=0, gauge=1, precision=64)
    pargs = (1.0, 1.0, 1.0, 1.0, 0.75)

    def forward(x, xc, pe, levs):
        st = [dev(a) for a in levs]
        u = [dev(np.zeros(sh[k])) for k in OUT_U]
        d = {k: dev(v) for k, v in (("x", x), ("xc", xc))}
        z = lambda: dev(np.zeros(sh["psi"]))
        ra, rr, p1, p2 = z(), z(), z(), z()
        ws.rho_gauge(st[0], st[1], st[2], u[0], u[1], u[2], d["x"], d["xc"], dev(f["h"]), ra, rr, dev(pe), p1, p2,
                     *pargs)
        out = dict(x=d["x"], xc=d["xc"], p1=p1, p2=p2, rhr=rr, u1=u[0], u2=u[1], u3=u[2])
        return sum(float((lam[k] * M.to_numpy(out[k])).sum()) for k in lam)

    # the Courant numbers the step advects with: the predictor alone on copies
    st = [dev(a) for a in lev]
    u = [dev(np.zeros(sh[k])) for k in OUT_U]
    ws.velprd(st[0], st[1], st[2], dev(f["h"]), *pargs, u[0], u[1], u[2])
    uc = [M.to_numpy(t) for t in u]
    g = gpu_rho_adjoint(M, n, ibc, {**f, "u1": uc[0], "u2": uc[1], "u3": uc[2]}, lam, iord=3, nonos=0)
    gx, gu, gxc, gpe = g[0], g[1:4], g[4], g[5]
    gst = [dev(np.zeros(sh["psi"] + (3,))) for _ in range(3)]
    ws.velprd_adjoint(gst[0], gst[1], gst[2], dev(f["h"]), *pargs, *[dev(a) for a in gu])
    torch.cuda.synchronize()
    glev = [M.to_numpy(t) for t in gst]
    eps = 1e-4
    for d in range(6):
        dirs = {k: np.zeros(sh["psi"]) for k in ("x", "xc", "pexe")}
        for k in dirs:
            dirs[k][I, J, K] = rng.standard_normal(n)
        dl = [np.zeros(sh["psi"] + (3,)) for _ in range(3)]
        for a in dl:
            a[I, J, K, 0] = rng.standard_normal(n)
            a[I, J, K, 2] = rng.standard_normal(n)
        nrm = np.sqrt(sum(float((a ** 2).sum()) for a in list(dirs.values()) + dl))
        dirs = {k: a / nrm for k, a in dirs.items()}
        dl = [a / nrm for a in dl]
        dot = (float((gx * dirs["x"]).sum()) + float((gxc * dirs["xc"]).sum()) + float((gpe * dirs["pexe"]).sum())
               + sum(float((glev[c][..., 0] * dl[c][..., 0]).sum()) + float((glev[c][..., 2] * dl[c][..., 2]).sum())
                     for c in range(3)))
        jp = forward(f["x"] + eps * dirs["x"], f["xc"] + eps * dirs["xc"], f["pexe"] + eps * dirs["pexe"],
                     [a + eps * b for a, b in zip(lev, dl)])
        jm = forward(f["x"] - eps * dirs["x"], f["xc"] - eps * dirs["xc"], f["pexe"] - eps * dirs["pexe"],
                     [a - eps * b for a, b in zip(lev, dl)])
        fd = (jp - jm) / (2 * eps)
        assert abs(fd - dot) <= 1e-6 * abs(dot), (d, fd, dot)
    ws.close()
