"""Adjoint of the velocity predictor (mpdata_velprd_adjoint_*) through the C ABI.

The predictor (velprd_traj0 + velprdA_to_C, module_velprd.f90:58-83,197-361,
and the level roll of velprd_driver.f90:254-270) is linear in the momenta of
levels 0 and 2 for fixed h and time steps.  Its outputs are the C-grid Courant
numbers, level 1 and the rolled level 2.  The adjoint is checked two ways:
- against the exact transpose built from the oracle's forward predictor, one
  column per unit input (small grids, periodic, open and mixed boundaries);
- by the dot-product test through the GPU forward at a larger size.
"""
import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ARGS = dict(dxi=0.5, dyi=0.25, dzi=2.0, dt=0.3)


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


def faces(n, m, l, ih=1):
    """Index slices of the faces 1..n+1 of u1, u2, u3 and of the interior."""
    I, J, K = slice(ih, ih + n), slice(ih, ih + m), slice(ih, ih + l)
    return (slice(ih, ih + n + 1), J, K), (I, slice(ih, ih + m + 1), K), (I, J, slice(ih, ih + l + 1)), (I, J, K)


def oracle_forward(O, g, n, m, l, l0, l2, h, r):
    sh = W.shapes(n, m, l, 1)
    st = []
    for c in range(3):
        a = np.zeros(sh["psi"] + (3,), order="F")
        a[..., 0] = l0[c]
        a[..., 2] = l2[c]
        st.append(a)
    u = [W.zeros(sh[k]) for k in ("u1", "u2", "u3")]
    O.velprd(g, st[0], st[1], st[2], h, ARGS["dxi"], ARGS["dyi"], ARGS["dzi"], ARGS["dt"], r, u[0], u[1], u[2])
    return u, [a[..., 1] for a in st], [a[..., 2] for a in st]


def pairing(cot, out, n, m, l):
    f1, f2, f3, inner = faces(n, m, l)
    cu, c1, c2 = cot
    u, L1, L2 = out
    s = sum(float((cu[c][f] * u[c][f]).sum()) for c, f in zip(range(3), (f1, f2, f3)))
    s += sum(float((c1[c][inner] * L1[c][inner]).sum()) + float((c2[c][inner] * L2[c][inner]).sum())
             for c in range(3))
    return s


def random_cot(rng, n, m, l):
    sh = W.shapes(n, m, l, 1)
    f1, f2, f3, inner = faces(n, m, l)
    cu = []
    for k, f in zip(("u1", "u2", "u3"), (f1, f2, f3)):
        a = W.zeros(sh[k])
        a[f] = rng.uniform(-1, 1, a[f].shape)
        cu.append(a)
    c1, c2 = [], []
    for lst in (c1, c2):
        for c in range(3):
            a = W.zeros(sh["psi"])
            a[inner] = rng.uniform(-1, 1, a[inner].shape)
            lst.append(a)
    return cu, c1, c2


def gpu_adjoint(M, n, m, l, ibc, h, cot, r, dtype=np.float64):
    import torch
    cu, c1, c2 = cot
    sh = W.shapes(n, m, l, 1)
    g0 = np.zeros(sh["psi"] + (3,), order="F")
    stacks = []
    for c in range(3):
        a = g0.copy(order="F")
        a[..., 1] = c1[c]
        a[..., 2] = c2[c]
        stacks.append(M.fortran_device(a, dtype=dtype))
    ws = M.Workspace(n, m, l, 1, *ibc, precision=64 if dtype == np.float64 else 32)
    ws.velprd_adjoint(stacks[0], stacks[1], stacks[2], M.fortran_device(h, dtype=dtype), ARGS["dxi"], ARGS["dyi"],
                      ARGS["dzi"], ARGS["dt"], r, *[M.fortran_device(a, dtype=dtype) for a in cu])
    torch.cuda.synchronize()
    ws.close()
    out = [M.to_numpy(t).astype(np.float64) for t in stacks]
    return [o[..., 0] for o in out], [o[..., 2] for o in out]


@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0), (1, 0, 1), (0, 1, 0)])
@pytest.mark.parametrize("r", [1.0, 0.75])
def test_predictor_adjoint_is_the_oracle_transpose(M, oracle, ibc, r):
    n, m, l = 4, 3, 3
    rng = np.random.default_rng(11 + sum(ibc) + int(4 * r))
    sh = W.shapes(n, m, l, 1)
    h = np.asfortranarray(rng.uniform(0.8, 1.2, sh["psi"]))
    cot = random_cot(rng, n, m, l)
    g0, g2 = gpu_adjoint(M, n, m, l, ibc, h, cot, r)
    g = oracle.grid(n, m, l, 1, *ibc)
    _, _, _, inner = faces(n, m, l)
    zero = [W.zeros(sh["psi"]) for _ in range(3)]
    scale = 0.0
    for c in range(3):
        scale = max(scale, np.abs(g0[c][inner]).max(), np.abs(g2[c][inner]).max())
    for c in range(3):
        for lvl, got in ((0, g0), (2, g2)):
            for i in range(n):
                for j in range(m):
                    for k in range(l):
                        e = [z.copy(order="F") for z in zero]
                        e[c][1 + i, 1 + j, 1 + k] = 1.0
                        l0, l2 = (e, zero) if lvl == 0 else (zero, e)
                        want = pairing(cot, oracle_forward(oracle, g, n, m, l, l0, l2, h, r), n, m, l)
                        assert abs(got[c][1 + i, 1 + j, 1 + k] - want) <= 1e-12 * scale, (c, lvl, i, j, k)


@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)])
@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-12), (np.float32, 1e-5)], ids=["fp64", "fp32"])
def test_predictor_adjoint_dot_product(M, ibc, dtype, tol):
    """<cot, F(d)> = <F^T cot, d> with the GPU forward, 40x24x12."""
    import torch
    n, m, l = 40, 24, 12
    rng = np.random.default_rng(3 + sum(ibc))
    sh = W.shapes(n, m, l, 1)
    r = 0.75
    h = np.asfortranarray(rng.uniform(0.8, 1.2, sh["psi"]))
    _, _, _, inner = faces(n, m, l)
    d0 = [W.zeros(sh["psi"]) for _ in range(3)]
    d2 = [W.zeros(sh["psi"]) for _ in range(3)]
    for a in d0 + d2:
        a[inner] = rng.uniform(-1, 1, a[inner].shape)
    # forward on the GPU: the outputs for the input (d0, d2)
    st = []
    for c in range(3):
        a = np.zeros(sh["psi"] + (3,), order="F")
        a[..., 0] = d0[c]
        a[..., 2] = d2[c]
        st.append(M.fortran_device(a, dtype=dtype))
    u = [M.fortran_device(W.zeros(sh[k]), dtype=dtype) for k in ("u1", "u2", "u3")]
    ws = M.Workspace(n, m, l, 1, *ibc, precision=64 if dtype == np.float64 else 32)
    ws.velprd(st[0], st[1], st[2], M.fortran_device(h, dtype=dtype), ARGS["dxi"], ARGS["dyi"], ARGS["dzi"],
              ARGS["dt"], r, u[0], u[1], u[2])
    torch.cuda.synchronize()
    ws.close()
    stn = [M.to_numpy(t).astype(np.float64) for t in st]
    out = ([M.to_numpy(t).astype(np.float64) for t in u], [a[..., 1] for a in stn], [a[..., 2] for a in stn])
    cot = random_cot(rng, n, m, l)
    lhs = pairing(cot, out, n, m, l)
    g0, g2 = gpu_adjoint(M, n, m, l, ibc, h, cot, r, dtype)
    rhs = sum(float((g0[c][inner] * d0[c][inner]).sum()) + float((g2[c][inner] * d2[c][inner]).sum())
              for c in range(3))
    assert abs(lhs - rhs) <= tol * max(abs(lhs), 1.0), (lhs, rhs)


def test_gradient_wrt_momenta_through_a_step(M):
    """dJ/d(A-grid momenta) of J = 0.5 |psi_1 - target|^2 after the predictor
    and one gauge step, composed from the step adjoint's dJ/du and the
    predictor adjoint, against central differences of the GPU forward
    (eps = 1e-4) along 6 seeded unit directions in levels 0 and 2.  J is smooth:
    the limiter is off and every Courant number stays away from 0, where the
    donor flux and |u| have kinks."""
    import torch
    n, m, l = 24, 20, 10
    ibc = (1, 1, 1)
    rng = np.random.default_rng(31)
    sh = W.shapes(n, m, l, 1)
    _, _, _, inner = faces(n, m, l)
    f = W.random_fields(n, m, l, ibc=ibc, seed=8)
    lev = [np.zeros(sh["psi"] + (3,), order="F") for _ in range(3)]
    for a in lev:  # a drift plus noise: every Courant number stays away from the kinks at 0
        a[inner + (0,)] = 0.2 + rng.uniform(-0.05, 0.05, (n, m, l))
        a[inner + (2,)] = 0.2 + rng.uniform(-0.05, 0.05, (n, m, l))
    tgt = f.x + 0.1 * np.asfortranarray(rng.uniform(-1, 1, f.x.shape))
    dev = lambda a: M.fortran_device(np.asfortranarray(a))
    h, rhr, target = dev(f.h), dev(f.rhr), dev(tgt)
    ws = M.Workspace(n, m, l, 1, *ibc, iord=2, nonos=0, gauge=1, precision=64)

    def forward(levs):
        st = [dev(a) for a in levs]
        u = [dev(W.zeros(sh[k])) for k in ("u1", "u2", "u3")]
        ws.velprd(st[0], st[1], st[2], h, 1.0, 1.0, 1.0, 1.0, 0.75, u[0], u[1], u[2])
        psi = dev(f.x)
        ws.step(psi, u[0], u[1], u[2], h, rhr)
        return psi, u

    psi1, u = forward(lev)
    lam = (psi1 - target).clone()
    lam[0, :, :] = 0
    lam[-1, :, :] = 0
    lam[:, 0, :] = 0
    lam[:, -1, :] = 0
    lam[:, :, 0] = 0
    lam[:, :, -1] = 0
    gu = [torch.zeros_like(t) for t in u]
    ws.step_adjoint(dev(f.x), u[0], u[1], u[2], h, rhr, lam, *gu)
    gst = [dev(np.zeros(sh["psi"] + (3,), order="F")) for _ in range(3)]
    ws.velprd_adjoint(gst[0], gst[1], gst[2], h, 1.0, 1.0, 1.0, 1.0, 0.75, *gu)
    torch.cuda.synchronize()
    g = [M.to_numpy(t) for t in gst]

    def J(levs):
        p, _ = forward(levs)
        return 0.5 * float(((M.to_numpy(p) - tgt)[inner] ** 2).sum())

    eps = 1e-4
    for d in range(6):
        dirs = [np.zeros(sh["psi"] + (3,), order="F") for _ in range(3)]
        for a in dirs:
            a[inner + (0,)] = rng.standard_normal((n, m, l))
            a[inner + (2,)] = rng.standard_normal((n, m, l))
        nrm = np.sqrt(sum(float((a ** 2).sum()) for a in dirs))
        dirs = [a / nrm for a in dirs]
        dot = sum(float((g[c][inner + (0,)] * dirs[c][inner + (0,)]).sum()) +
                  float((g[c][inner + (2,)] * dirs[c][inner + (2,)]).sum()) for c in range(3))
        jp = J([a + eps * e for a, e in zip(lev, dirs)])
        jm = J([a - eps * e for a, e in zip(lev, dirs)])
        fd = (jp - jm) / (2 * eps)
        assert abs(fd - dot) <= 1e-6 * abs(dot), (d, fd, dot)
    ws.close()
