"""The oracle's reverse-mode AD of the density step after its predictor
(orc_rho_adjoint_f64, the checker of mpdata_rho_gauge_adjoint_*) against
central differences of the oracle's own forward (orc_rho_step_f64).

J = <l, outputs> for seeded cotangents of every output (psi, x_incomp, pexr1,
pexr2, rhr on the interior, the mass fluxes on the faces 1..n+1).  The inputs
are smooth away from the forward's branches: densities, fields and pexe
positive, Courant numbers 0.2 +- 0.05 (away from the kinks at 0).  Along
seeded unit directions in the inputs (psi, u1..u3, x_incomp, pexe), the
central difference with eps = 1e-6 agrees with the gradient to 1e-6."""
import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W


def problem(ibc, seed, n=(6, 5, 4)):
    rng = np.random.default_rng(seed)
    sh = W.shapes(*n, 1)
    f = {k: np.asfortranarray(rng.uniform(1.0, 2.0, sh["psi"])) for k in ("x", "xc")}
    f["h"] = np.asfortranarray(rng.uniform(0.8, 1.2, sh["psi"]))
    f["pexe"] = np.asfortranarray(rng.uniform(0.5, 1.5, sh["psi"]))
    for c, k in enumerate(("u1", "u2", "u3")):
        f[k] = np.asfortranarray(0.2 + rng.uniform(-0.05, 0.05, sh[k]))
    f["bcx"] = np.asfortranarray(rng.uniform(1.0, 2.0, (n[1], n[2], 2)))
    f["bcy"] = np.asfortranarray(rng.uniform(1.0, 2.0, (n[0], n[2], 2)))
    return n, sh, f


def forward(O, g, f):
    x, xc = f["x"].copy(order="F"), f["xc"].copy(order="F")
    u = [f[k].copy(order="F") for k in ("u1", "u2", "u3")]
    z = lambda: np.zeros_like(x, order="F")
    ra, rr, p1, p2 = z(), z(), z(), z()
    O.rho_step(g, u[0], u[1], u[2], x, xc, f["h"], ra, rr, f["pexe"], p1, p2, f["bcx"], f["bcy"])
    return dict(x=x, xc=xc, p1=p1, p2=p2, rhr=rr, u1=u[0], u2=u[1], u3=u[2])


def masks(n, sh):
    I, J, K = slice(1, 1 + n[0]), slice(1, 1 + n[1]), slice(1, 1 + n[2])
    m = {}
    for k in ("x", "xc", "p1", "p2", "rhr"):
        a = np.zeros(sh["psi"], bool)
        a[I, J, K] = True
        m[k] = a
    for k, fs in (("u1", (slice(1, 2 + n[0]), J, K)), ("u2", (I, slice(1, 2 + n[1]), K)),
                  ("u3", (I, J, slice(1, 2 + n[2])))):
        a = np.zeros(sh[k], bool)
        a[fs] = True
        m[k] = a
    return m


@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0), (1, 0, 0)])
def test_oracle_rho_adjoint_matches_central_differences(oracle, ibc):
    n, sh, f = problem(ibc, 41 + sum(ibc))
    g = oracle.grid(*n, 1, *ibc)
    rng = np.random.default_rng(7 + sum(ibc))
    m = masks(n, sh)
    lam = {k: np.asfortranarray(np.where(m[k], rng.uniform(-1, 1, m[k].shape), 0.0)) for k in m}
    grads = oracle.rho_adjoint(g, f["u1"], f["u2"], f["u3"], f["x"], f["xc"], f["h"], f["pexe"], f["bcx"], f["bcy"],
                               l_x=lam["x"], l_u1=lam["u1"], l_u2=lam["u2"], l_u3=lam["u3"], l_xinc=lam["xc"],
                               l_p1=lam["p1"], l_p2=lam["p2"], l_rhr=lam["rhr"])
    names = ("x", "u1", "u2", "u3", "xc", "pexe")
    G = dict(zip(names, grads))

    def J(ff):
        out = forward(oracle, g, ff)
        return sum(float((lam[k] * out[k]).sum()) for k in lam)

    inner = masks(n, sh)["x"]
    for d in range(8):
        dirs = {}
        for k in names:
            a = rng.standard_normal(f[k].shape)
            if k in ("x", "xc", "pexe"):
                a = np.where(inner, a, 0.0)
            dirs[k] = a
        nrm = np.sqrt(sum(float((a ** 2).sum()) for a in dirs.values()))
        dirs = {k: a / nrm for k, a in dirs.items()}
        dot = sum(float((G[k] * dirs[k]).sum()) for k in names)
        eps = 1e-6
        fp = {**f, **{k: np.asfortranarray(f[k] + eps * dirs[k]) for k in names}}
        fm = {**f, **{k: np.asfortranarray(f[k] - eps * dirs[k]) for k in names}}
        fd = (J(fp) - J(fm)) / (2 * eps)
        assert abs(fd - dot) <= 1e-6 * max(abs(dot), 1.0), (d, fd, dot)
