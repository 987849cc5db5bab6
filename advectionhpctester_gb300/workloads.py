"""Synthetic inputs for the MPDATA step, in the reference's Fortran layout.

Every array is a numpy array in Fortran order with the reference's halo
extents (ih halo cells on each side; the C-grid arrays carry one extra face
along their own axis):

  psi-shaped (np+2ih, mp+2ih, lp+2ih)       u1 (np+1+2ih, mp+2ih, lp+2ih)
  u2 (np+2ih, mp+1+2ih, lp+2ih)             u3 (np+2ih, mp+2ih, lp+1+2ih)
  bcx (mp, lp, 2)                           bcy (np, lp, 2)

Workloads:
  kat_rotating_sphere  the reference's own test case, set_initial15
                       (advection/src_testdata/advection_test_setup.f90:174-255)
                       with init_data (:619-637) and the C-grid averaging of
                       velprdA_to_C_ver2 (advection/src_algorithms/module_velprd.f90:366-520);
                       59^3, dt = 0.018*2*pi, nt = 556, open x/y and wall z.
  solid_body_z         64x64x32 periodic solid-body rotation about z, Courant 0.4,
                       Gaussian cone psi (the CPU-runnable workload).
  deformational        512x512x128-style periodic time-varying deformational flow
                       with max Courant 0.5 and noise + two cones (seeded).
No public data set is involved: every input is generated from closed-form
expressions and seeded generators.
"""
import math

import numpy as np


def shapes(np_, mp, lp, ih=1):
    s = (np_ + 2 * ih, mp + 2 * ih, lp + 2 * ih)
    return dict(psi=s, u1=(s[0] + 1, s[1], s[2]), u2=(s[0], s[1] + 1, s[2]),
                u3=(s[0], s[1], s[2] + 1), bcx=(mp, lp, 2), bcy=(np_, lp, 2))


def zeros(shape, dtype=np.float64):
    return np.zeros(shape, dtype=dtype, order="F")


def interior(a, ih=1):
    """View of the interior cells of a psi-shaped array."""
    return a[ih:a.shape[0] - ih, ih:a.shape[1] - ih, ih:a.shape[2] - ih]


class Fields:
    """One MPDATA problem: psi, C-grid Courant numbers, densities, Dirichlet
    halo values and the boundary flags."""

    def __init__(self, np_, mp, lp, ih=1, ibcx=0, ibcy=0, ibcz=0, dtype=np.float64):
        self.np, self.mp, self.lp, self.ih = np_, mp, lp, ih
        self.ibcx, self.ibcy, self.ibcz = ibcx, ibcy, ibcz
        sh = shapes(np_, mp, lp, ih)
        self.x = zeros(sh["psi"], dtype)
        self.u1 = zeros(sh["u1"], dtype)
        self.u2 = zeros(sh["u2"], dtype)
        self.u3 = zeros(sh["u3"], dtype)
        self.h = zeros(sh["psi"], dtype)
        self.rhr = zeros(sh["psi"], dtype)
        self.bcx = zeros(sh["bcx"], dtype)
        self.bcy = zeros(sh["bcy"], dtype)
        self.h[...] = 1.0
        self.rhr[...] = 1.0

    @property
    def dtype(self):
        return self.x.dtype

    def astype(self, dtype):
        f = Fields(self.np, self.mp, self.lp, self.ih, self.ibcx, self.ibcy, self.ibcz, dtype)
        for k in ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy"):
            getattr(f, k)[...] = getattr(self, k)
        for k, v in self.__dict__.items():
            if k not in f.__dict__:
                setattr(f, k, v)
        return f

    def copy(self):
        return self.astype(self.dtype)

    def cells(self):
        return self.np * self.mp * self.lp


# ---------------------------------------------------------------------------
# The reference's known-answer test: rotating sphere on 59^3
# ---------------------------------------------------------------------------

def a_to_c_open(ua, va, wa, f):
    """velprdA_to_C_ver2 with ibcx=ibcy=ibcz=0 (module_velprd.f90:386-517):
    one-sided halo extrapolation 2a(1)-a(2) on every wall, then C-grid
    averaging u1(i) = 0.5*(a(i)+a(i-1)) for faces 1..n+1."""
    ih = f.ih
    n, m, l = f.np, f.mp, f.lp
    I = slice(ih, ih + n)
    J = slice(ih, ih + m)
    K = slice(ih, ih + l)
    ua = ua.copy(order="F")
    va = va.copy(order="F")
    wa = wa.copy(order="F")
    ua[ih - 1, J, K] = 2.0 * ua[ih, J, K] - ua[ih + 1, J, K]
    ua[ih + n, J, K] = 2.0 * ua[ih + n - 1, J, K] - ua[ih + n - 2, J, K]
    va[I, ih - 1, K] = 2.0 * va[I, ih, K] - va[I, ih + 1, K]
    va[I, ih + m, K] = 2.0 * va[I, ih + m - 1, K] - va[I, ih + m - 2, K]
    wa[I, J, ih - 1] = 2.0 * wa[I, J, ih] - wa[I, J, ih + 1]
    wa[I, J, ih + l] = 2.0 * wa[I, J, ih + l - 1] - wa[I, J, ih + l - 2]
    # faces 1..n+1 sit at array positions ih..ih+n of the C-grid arrays
    f.u1[ih:ih + n + 1, J, K] = 0.5 * (ua[ih:ih + n + 1, J, K] + ua[ih - 1:ih + n, J, K])
    f.u2[I, ih:ih + m + 1, K] = 0.5 * (va[I, ih:ih + m + 1, K] + va[I, ih - 1:ih + m, K])
    f.u3[I, J, ih:ih + l + 1] = 0.5 * (wa[I, J, ih:ih + l + 1] + wa[I, J, ih - 1:ih + l])


def kat_rotating_sphere(n=59, ih=1, dtype=np.float64):
    """set_initial15 + init_data on an n^3 open/wall grid (the reference default
    test, advection_dwarf_test_modular.f90:96-141).  Returns (fields, meta)."""
    dx00 = 100.0
    dx = dx00 / (n - 1)           # eulag_lib_parameters.f90:499-501
    dt = 0.018 * 2.0 * math.acos(-1.0)   # advection_dwarf_test_modular.f90:97
    nt = 556
    f = Fields(n, n, n, ih, 0, 0, 0, np.float64)
    sqrt3i = 1.0 / math.sqrt(3.0)
    x0 = y0 = z0 = 0.5 * dx00
    xc = x0 - 0.25 * dx00 * sqrt3i
    yc = y0 + 0.25 * dx00 * sqrt3i
    zc = z0 + 0.25 * dx00 * sqrt3i
    r2 = 15.0 * 15.0
    omega = 0.1 / math.sqrt(3.0)
    idx = np.arange(1, n + 1, dtype=np.float64)
    ia = idx[:, None, None]
    ja = idx[None, :, None]
    ka = idx[None, None, :]
    xp, yp, zp = ia * dx, ja * dx, ka * dx
    tmp = (xp - xc) * (xp - xc) + (yp - yc) * (yp - yc) + (zp - zc) * (zp - zc)
    interior(f.x, ih)[...] = np.where(tmp <= r2, 4.0, 0.0)
    sh = f.x.shape
    ua = zeros(sh)
    va = zeros(sh)
    wa = zeros(sh)
    interior(ua, ih)[...] = (-(omega * (ja * dx - y0)) + omega * (ka * dx - z0)) * dt / dx + 0 * ia
    interior(va, ih)[...] = (omega * (ia * dx - x0) - omega * (ka * dx - z0)) * dt / dx + 0 * ja
    interior(wa, ih)[...] = (-(omega * (ia * dx - x0)) + omega * (ja * dx - y0)) * dt / dx + 0 * ka
    a_to_c_open(ua, va, wa, f)
    meta = dict(name="kat_rotating_sphere_%d" % n, dt=dt, nt=nt, timetot=nt * dt,
                xtest=interior(f.x, ih).copy(), t_adv=1, iord=2, nonos=1)
    if dtype != np.float64:
        f = f.astype(dtype)
    return f, meta


def error_l2(x, xtest, n_cells, timetot, ih=1):
    """test_solution_error (advection_test_setup.f90:595-617):
    sqrt(sum((x0-x)^2)/N)/T."""
    d = (xtest.astype(np.float64) - interior(x, ih).astype(np.float64)) ** 2
    return math.sqrt(float(d.sum()) * (1.0 / n_cells)) / timetot


def energy_l2(x, xtest, n_cells, timetot, ih=1):
    """test_solution_energy (advection_test_setup.f90:472-492):
    sqrt(|sum x^2 - sum x0^2|/N)/T."""
    a = float((interior(x, ih).astype(np.float64) ** 2).sum())
    e = float((xtest.astype(np.float64) ** 2).sum())
    return math.sqrt(abs(a - e) * (1.0 / n_cells)) / timetot


# ---------------------------------------------------------------------------
# Periodic synthetic workloads
# ---------------------------------------------------------------------------

def solid_body_z(np_=64, mp=64, lp=32, ih=1, courant=0.4, dtype=np.float64, std=True):
    """64x64x32 periodic grid, dx=dy=dz=dt=1, h=rhr=1; steady solid-body rotation
    about the z axis through the domain centre sampled on the cell faces
    (u1=-w(y-yc), u2=w(x-xc), u3=0: discretely divergence-free), w chosen so
    max|u| = courant; psi = 1 + 4 exp(-r^2/(2*4^2)) centred at (16,32,16)."""
    f = Fields(np_, mp, lp, ih, 1, 1, 1, np.float64)
    xc, yc = np_ / 2.0 + 0.5, mp / 2.0 + 0.5      # cell i centre at x = i
    # face i (between cells i-1 and i) sits at x = i - 1/2
    xf = np.arange(1, np_ + 2) - 0.5
    yf = np.arange(1, mp + 2) - 0.5
    xcell = np.arange(1, np_ + 1, dtype=np.float64)
    ycell = np.arange(1, mp + 1, dtype=np.float64)
    rmax = max(abs(yf - yc).max(), abs(xf - xc).max())
    w = courant / rmax
    J = slice(ih, ih + mp)
    I = slice(ih, ih + np_)
    K = slice(ih, ih + lp)
    f.u1[ih:ih + np_ + 1, J, K] = (-w * (ycell - yc))[None, :, None] + 0 * xf[:, None, None]
    f.u2[I, ih:ih + mp + 1, K] = (w * (xcell - xc))[:, None, None] + 0 * yf[None, :, None]
    f.u3[...] = 0.0
    zcell = np.arange(1, lp + 1, dtype=np.float64)
    r2 = ((xcell - 16.0)[:, None, None] ** 2 + (ycell - 32.0)[None, :, None] ** 2
          + (zcell - 16.0)[None, None, :] ** 2)
    interior(f.x, ih)[...] = 1.0 + 4.0 * np.exp(-r2 / (2.0 * 4.0 ** 2))
    f.meta = dict(name="solid_body_z_%dx%dx%d" % (np_, mp, lp), t_adv=2, iord=2, nonos=1)
    return f.astype(dtype) if dtype != np.float64 else f


def deformational_agrid(np_, mp, lp, t, T, courant=0.5):
    """A-grid (cell-centred) Courant numbers of the time-varying deformational
    flow u = sin^2(pi x) sin(2 pi y) cos(pi t/T), v = -sin^2(pi y) sin(2 pi x) cos(pi t/T),
    w = 0.1 sin(2 pi z); x,y,z in [0,1) at cell centres; scaled so that the
    t=0 maximum of |u|+|v|+|w| is `courant`."""
    x = (np.arange(np_) + 0.5) / np_
    y = (np.arange(mp) + 0.5) / mp
    z = (np.arange(lp) + 0.5) / lp
    ct = math.cos(math.pi * t / T)
    u = (np.sin(math.pi * x) ** 2)[:, None, None] * np.sin(2 * math.pi * y)[None, :, None] * ct
    v = -(np.sin(math.pi * y) ** 2)[None, :, None] * np.sin(2 * math.pi * x)[:, None, None] * ct
    w = 0.1 * np.sin(2 * math.pi * z)[None, None, :]
    u = np.broadcast_to(u, (np_, mp, lp))
    v = np.broadcast_to(v, (np_, mp, lp))
    w = np.broadcast_to(w, (np_, mp, lp))
    scale = courant / 1.1   # max|u| = max|v| = 1 at t=0, max|w| = 0.1
    return u * scale, v * scale, w * scale


def deformational(np_=512, mp=512, lp=128, ih=1, courant=0.5, seed=20261203, dtype=np.float64,
                  nsteps=200, balls=False):
    """Periodic deformational-flow workload: psi ~ U[1,2] (seeded) plus two
    Gaussian cones (amplitude 1, sigma 0.05 L); C-grid Courant numbers are the
    periodic face averages of the A-grid flow at t=0.  balls: psi is instead
    two balls of value 4 (radius 0.15 L) on an exactly zero background, as in
    the reference's rotating-sphere test."""
    f = Fields(np_, mp, lp, ih, 1, 1, 1, np.float64)
    rng = np.random.default_rng(seed)
    x = (np.arange(np_) + 0.5) / np_
    y = (np.arange(mp) + 0.5) / mp
    z = (np.arange(lp) + 0.5) / lp
    psi = np.zeros((np_, mp, lp)) if balls else 1.0 + rng.random((np_, mp, lp))
    for (cx, cy, cz) in ((0.35, 0.35, 0.5), (0.65, 0.65, 0.5)):
        r2 = ((x - cx)[:, None, None] ** 2 + (y - cy)[None, :, None] ** 2
              + (z - cz)[None, None, :] ** 2)
        if balls:
            psi[r2 <= 0.15 ** 2] = 4.0
        else:
            psi += np.exp(-r2 / (2 * 0.05 ** 2))
    interior(f.x, ih)[...] = psi
    ua, va, wa = deformational_agrid(np_, mp, lp, 0.0, float(nsteps))
    set_c_grid_periodic(f, ua, va, wa)
    f.meta = dict(name="deformational_%dx%dx%d" % (np_, mp, lp), t_adv=1, iord=3, nonos=1,
                  T=float(nsteps))
    return f.astype(dtype) if dtype != np.float64 else f


def set_c_grid_periodic(f, ua, va, wa):
    """C-grid faces from A-grid interior values with a periodic wrap:
    u1(i) = 0.5*(a(i)+a(i-1)), face n+1 == face 1."""
    ih = f.ih
    n, m, l = f.np, f.mp, f.lp
    I = slice(ih, ih + n)
    J = slice(ih, ih + m)
    K = slice(ih, ih + l)
    u = 0.5 * (ua + np.roll(ua, 1, axis=0))
    v = 0.5 * (va + np.roll(va, 1, axis=1))
    w = 0.5 * (wa + np.roll(wa, 1, axis=2))
    f.u1[ih:ih + n, J, K] = u
    f.u1[ih + n, J, K] = u[0]
    f.u2[I, ih:ih + m, K] = v
    f.u2[I, ih + m, K] = v[:, 0]
    f.u3[I, J, ih:ih + l] = w
    f.u3[I, J, ih + l] = w[:, :, 0]


def random_fields(np_, mp, lp, ih=1, ibc=(0, 0, 0), seed=0, courant=0.3, dtype=np.float64,
                  sign_change=False):
    """Seeded random problem for parity tests: psi in [0.5,1.5] (or a signed
    field), random C-grid Courant numbers in [-courant, courant], h and rhr in
    [0.8,1.2], random Dirichlet halo values."""
    rng = np.random.default_rng(seed)
    f = Fields(np_, mp, lp, ih, *ibc, np.float64)
    f.x[...] = rng.uniform(-1.0, 1.0, f.x.shape) if sign_change else rng.uniform(0.5, 1.5, f.x.shape)
    for a in (f.u1, f.u2, f.u3):
        a[...] = rng.uniform(-courant, courant, a.shape)
    f.h[...] = rng.uniform(0.8, 1.2, f.h.shape)
    f.rhr[...] = rng.uniform(0.8, 1.2, f.rhr.shape)
    f.bcx[...] = rng.uniform(0.5, 1.5, f.bcx.shape)
    f.bcy[...] = rng.uniform(0.5, 1.5, f.bcy.shape)
    return f.astype(dtype) if dtype != np.float64 else f


def predictor_case(np_, mp, lp, ih=1, courant=2.0, seed=0, dtype=np.float64):
    """Seeded inputs of the predictor and its Courant control: momentum
    stacks ox/oy/oz and physical velocities u/v/w (psi-shaped x 3 levels,
    Fortran order), h in [0.8,1.2], dx = dy = dz = 1 and dt = 1, with level 0
    scaled so that the level-1 Courant maximum |ox|+|oy|+|oz| is about
    `courant`; level 2 (n-1 momenta) is level 0 times h plus 10% noise."""
    rng = np.random.default_rng(seed)
    s = (np_ + 2 * ih, mp + 2 * ih, lp + 2 * ih, 3)
    h = np.asfortranarray(rng.uniform(0.8, 1.2, s[:3]))
    st = {}
    for name in ("ox", "oy", "oz"):
        a = np.zeros(s, order="F")
        a[..., 0] = rng.uniform(-1.0, 1.0, s[:3]) * (courant / 3.0)
        a[..., 2] = a[..., 0] * h * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, s[:3]))
        st[name] = a
    for name in ("u", "v", "w"):
        st[name] = np.asfortranarray(rng.uniform(-1.0, 1.0, s))
    st["h"] = h
    shp = shapes(np_, mp, lp, ih)
    st["uadv"] = np.zeros(shp["u1"], order="F")
    st["vadv"] = np.zeros(shp["u2"], order="F")
    st["wadv"] = np.asfortranarray(rng.uniform(-1.0, 1.0, shp["u3"]))  # lvertsplit halves it
    if dtype != np.float64:
        st = {k: np.asfortranarray(v.astype(dtype)) for k, v in st.items()}
    return st
