"""ctypes front end of the C++ oracle (test infrastructure only).

Arrays are numpy arrays in Fortran order with the reference's halo extents
(see mpdata_oracle.h).  Every function mirrors one reference entry point:

  advec_dwarf  advection/src_drivers/advec.f90:116-244
  upwind       advection/src_algorithms/upwind3d-gpubc.f90:20-201
  velprd       advection/src_algorithms/module_velprd.f90:15-89,166-364 and
               advection/src_algorithms/velprd_driver.f90:254-270
  a_to_c       advection/src_algorithms/module_velprd.f90:366-520
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


class OrcGrid(ctypes.Structure):
    _fields_ = [("np", ctypes.c_int), ("mp", ctypes.c_int), ("lp", ctypes.c_int),
                ("ih", ctypes.c_int), ("ibcx", ctypes.c_int), ("ibcy", ctypes.c_int),
                ("ibcz", ctypes.c_int)]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        I = ctypes.c_int
        for name in ("orc_advec_dwarf_f64", "orc_advec_dwarf_f32"):
            f = getattr(_lib, name)
            f.argtypes = [ctypes.POINTER(OrcGrid), I, I, I, I] + [P] * 8
            f.restype = I
        for name in ("orc_advec_steps_f64", "orc_advec_steps_f32"):
            f = getattr(_lib, name)
            f.argtypes = [ctypes.POINTER(OrcGrid), I, I, I, I, I] + [P] * 8
            f.restype = I
        _lib.orc_upwind_f64.argtypes = [ctypes.POINTER(OrcGrid)] + [P] * 9
        _lib.orc_upwind_f64.restype = I
        D = ctypes.c_double
        F = ctypes.c_float
        _lib.orc_velprd_f64.argtypes = [ctypes.POINTER(OrcGrid)] + [P] * 7 + [D] * 5 + [P] * 3
        _lib.orc_velprd_f64.restype = I
        _lib.orc_velprd_f32.argtypes = [ctypes.POINTER(OrcGrid)] + [P] * 7 + [F] * 5 + [P] * 3
        _lib.orc_velprd_f32.restype = I
        _lib.orc_rho_gauge_f64.argtypes = [ctypes.POINTER(OrcGrid)] + [P] * 19 + [D] * 5 + [I]
        _lib.orc_rho_gauge_f64.restype = I
        _lib.orc_adjoint_f64.argtypes = [ctypes.POINTER(OrcGrid), I, I, I, I] + [P] * 15
        _lib.orc_adjoint_f64.restype = I
        _lib.orc_tangent_adjoint_f64.argtypes = [ctypes.POINTER(OrcGrid), I, I, I, I] + [P] * 20
        _lib.orc_tangent_adjoint_f64.restype = I
        _lib.orc_rho_adjoint_f64.argtypes = [ctypes.POINTER(OrcGrid)] + [P] * 23
        _lib.orc_rho_step_f64.argtypes = [ctypes.POINTER(OrcGrid)] + [P] * 13 + [I]
        _lib.orc_rho_step_f64.restype = I
        _lib.orc_rho_adjoint_f64.restype = I
        _lib.orc_a_to_c_f64.argtypes = [ctypes.POINTER(OrcGrid)] + [P] * 6
        _lib.orc_a_to_c_f64.restype = I
        for name, R in (("f64", D), ("f32", F)):
            f = getattr(_lib, "orc_compute_courants_" + name)
            f.argtypes = [ctypes.POINTER(OrcGrid), I] + [P] * 4 + [R] * 4 + [P]
            f.restype = I
            f = getattr(_lib, "orc_velprd_driver_" + name)
            f.argtypes = ([ctypes.POINTER(OrcGrid), ctypes.POINTER(I), ctypes.POINTER(I), I, ctypes.POINTER(R),
                           ctypes.POINTER(R), I, I, I, R, R] + [P] * 10 + [R] * 4 + [P])
            f.restype = I
        _lib.orc_set_literal_sums.argtypes = [I]
        _lib.orc_set_threads.argtypes = [I]
        _lib.orc_get_threads.restype = I
    return _lib


def set_threads(n):
    lib().orc_set_threads(int(n))


def set_literal_sums(on):
    """1: evaluate the 4-face velocity sums left to right in the reference's
    written order; 0: the pair order the CUDA kernels reproduce."""
    lib().orc_set_literal_sums(1 if on else 0)


def _ptr(a, dtype):
    if a is None:
        return None
    assert a.dtype == dtype and a.flags.f_contiguous, "oracle arrays must be Fortran-ordered %s" % dtype
    return a.ctypes.data


def grid(np_, mp, lp, ih=1, ibcx=0, ibcy=0, ibcz=0):
    return OrcGrid(np_, mp, lp, ih, ibcx, ibcy, ibcz)


def advec_dwarf(g, x, x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv, legacyoptmode=4, t_adv=1,
                iord=2, nonos=1, nsteps=1):
    """In-place MPDATA step(s) on x; returns nothing, raises on a bad call."""
    dt = x.dtype
    fn = {np.float64: "orc_advec_steps_f64", np.float32: "orc_advec_steps_f32"}[dt.type]
    rc = getattr(lib(), fn)(ctypes.byref(g), int(nsteps), int(legacyoptmode), int(t_adv), int(iord),
                            int(nonos), _ptr(x, dt), _ptr(x_lr, dt), _ptr(x_bt, dt), _ptr(uadv, dt),
                            _ptr(vadv, dt), _ptr(wadv, dt), _ptr(rhr, dt), _ptr(rhoadv, dt))
    if rc != 0:
        raise ValueError("oracle advec_dwarf failed with code %d" % rc)


def upwind(g, x, bcx, bcy, u1, u2, u3, rhr, h):
    xant = np.zeros_like(x, order="F")
    d = np.float64
    rc = lib().orc_upwind_f64(ctypes.byref(g), _ptr(x, d), _ptr(bcx, d), _ptr(bcy, d), _ptr(u1, d),
                              _ptr(u2, d), _ptr(u3, d), _ptr(rhr, d), _ptr(h, d), _ptr(xant, d))
    if rc != 0:
        raise ValueError("oracle upwind failed with code %d" % rc)
    return xant


def velprd(g, ox, oy, oz, h, dxi, dyi, dzi, dt, dt_ratio, u1, u2, u3, u=None, v=None, w=None):
    """Predictor in place: ox/oy/oz are (..., 3) level stacks, Fortran ordered."""
    d = ox.dtype
    fn = {np.float64: "orc_velprd_f64", np.float32: "orc_velprd_f32"}[d.type]
    rc = getattr(lib(), fn)(ctypes.byref(g), _ptr(ox, d), _ptr(oy, d), _ptr(oz, d), _ptr(u, d),
                            _ptr(v, d), _ptr(w, d), _ptr(h, d), dxi, dyi, dzi, dt, dt_ratio,
                            _ptr(u1, d), _ptr(u2, d), _ptr(u3, d))
    if rc != 0:
        raise ValueError("oracle velprd failed with code %d" % rc)


def compute_courants(g, ntimelevel, ox, oy, oz, h, dxi, dyi, dzi, dt):
    """compute_courants of level stacks ox/oy/oz (..., 3): the seven maxima
    (cr3d, crxy, crxz, cryz, crx, cry, crz) as an array of the field dtype."""
    d = ox.dtype
    sfx = {np.float64: "f64", np.float32: "f32"}[d.type]
    cr = np.zeros(7, dtype=d)
    rc = getattr(lib(), "orc_compute_courants_" + sfx)(ctypes.byref(g), int(ntimelevel), _ptr(ox, d), _ptr(oy, d),
                                                       _ptr(oz, d), _ptr(h, d), dxi, dyi, dzi, dt, _ptr(cr, d))
    if rc != 0:
        raise ValueError("oracle compute_courants failed with code %d" % rc)
    return cr


def velprd_driver(g, state, ox, oy, oz, uadv, vadv, wadv, h, dxi, dyi, dzi, dt, u=None, v=None, w=None):
    """velprd_driver in place.  state: dict with nsubsteps, nsubsteps_o, dtn,
    dtnold (updated), lsubstepping, ltimeadapt, lvertsplit, lcrdiag_nphlf,
    crmaxlim, dtmax.  Returns (code, diag[9])."""
    d = ox.dtype
    sfx = {np.float64: "f64", np.float32: "f32"}[d.type]
    R = ctypes.c_double if d == np.float64 else ctypes.c_float
    ns, nso = ctypes.c_int(state["nsubsteps"]), ctypes.c_int(state["nsubsteps_o"])
    dtn, dtnold = R(state["dtn"]), R(state["dtnold"])
    diag = np.zeros(9)
    rc = getattr(lib(), "orc_velprd_driver_" + sfx)(
        ctypes.byref(g), ctypes.byref(ns), ctypes.byref(nso), int(state["lsubstepping"]), ctypes.byref(dtn),
        ctypes.byref(dtnold), int(state["ltimeadapt"]), int(state["lvertsplit"]), int(state["lcrdiag_nphlf"]),
        state["crmaxlim"], state["dtmax"], _ptr(ox, d), _ptr(oy, d), _ptr(oz, d), _ptr(u, d), _ptr(v, d),
        _ptr(w, d), _ptr(uadv, d), _ptr(vadv, d), _ptr(wadv, d), _ptr(h, d), dxi, dyi, dzi, dt,
        _ptr(diag, np.float64))
    state.update(nsubsteps=ns.value, nsubsteps_o=nso.value, dtn=dtn.value, dtnold=dtnold.value)
    return rc, diag


def rho_gauge(g, ox, oy, oz, u1, u2, u3, x_in, x_incomp, h, rhoadv, rhr, pexe, pexr1, pexr2, bcx,
              bcy, dxi, dyi, dzi, dt, dt_ratio, liner=0, u=None, v=None, w=None):
    d = np.float64
    rc = lib().orc_rho_gauge_f64(ctypes.byref(g), _ptr(ox, d), _ptr(oy, d), _ptr(oz, d), _ptr(u, d),
                                 _ptr(v, d), _ptr(w, d), _ptr(u1, d), _ptr(u2, d), _ptr(u3, d),
                                 _ptr(x_in, d), _ptr(x_incomp, d), _ptr(h, d), _ptr(rhoadv, d),
                                 _ptr(rhr, d), _ptr(pexe, d), _ptr(pexr1, d), _ptr(pexr2, d),
                                 _ptr(bcx, d), _ptr(bcy, d), dxi, dyi, dzi, dt, dt_ratio, int(liner))
    if rc != 0:
        raise ValueError("oracle rho_gauge failed with code %d" % rc)


def rho_step(g, u1, u2, u3, x_in, x_incomp, h, rhoadv, rhr, pexe, pexr1, pexr2, bcx, bcy, liner=0):
    """The density step after its predictor, in place (u1..u3 become the mass fluxes)."""
    d = np.float64
    rc = lib().orc_rho_step_f64(ctypes.byref(g), _ptr(u1, d), _ptr(u2, d), _ptr(u3, d), _ptr(x_in, d),
                                _ptr(x_incomp, d), _ptr(h, d), _ptr(rhoadv, d), _ptr(rhr, d), _ptr(pexe, d),
                                _ptr(pexr1, d), _ptr(pexr2, d), _ptr(bcx, d), _ptr(bcy, d), int(liner))
    if rc != 0:
        raise ValueError("oracle rho_step failed with code %d" % rc)


def rho_adjoint(g, u1, u2, u3, x_in, x_incomp, h, pexe, bcx, bcy, l_x=None, l_u1=None, l_u2=None, l_u3=None,
                l_xinc=None, l_p1=None, l_p2=None, l_rhr=None):
    """Reverse-mode AD of the density step after its predictor: returns
    (dJ/dpsi_in, dJ/du1, dJ/du2, dJ/du3, dJ/dx_incomp_in, dJ/dpexe) for the
    output cotangents l_* (None: zero)."""
    d = np.float64
    gx, gc, gp = (np.zeros_like(x_in, order="F") for _ in range(3))
    g1, g2, g3 = (np.zeros_like(a, order="F") for a in (u1, u2, u3))
    rc = lib().orc_rho_adjoint_f64(ctypes.byref(g), _ptr(u1, d), _ptr(u2, d), _ptr(u3, d), _ptr(x_in, d),
                                   _ptr(x_incomp, d), _ptr(h, d), _ptr(pexe, d), _ptr(bcx, d), _ptr(bcy, d),
                                   _ptr(l_x, d), _ptr(l_u1, d), _ptr(l_u2, d), _ptr(l_u3, d), _ptr(l_xinc, d),
                                   _ptr(l_p1, d), _ptr(l_p2, d), _ptr(l_rhr, d), _ptr(gx, d), _ptr(g1, d),
                                   _ptr(g2, d), _ptr(g3, d), _ptr(gc, d), _ptr(gp, d))
    if rc != 0:
        raise ValueError("oracle rho_adjoint failed with code %d" % rc)
    return gx, g1, g2, g3, gc, gp


def adjoint(g, x0, bcx, bcy, u1, u2, u3, rhr, h, target, t_adv=1, iord=2, nonos=1, nsteps=1):
    """Returns (J, x_N, dJ/dx0, dJ/du1, dJ/du2, dJ/du3) by AD of the oracle."""
    d = np.float64
    J = ctypes.c_double(0.0)
    xN = np.zeros_like(x0, order="F")
    gx = np.zeros_like(x0, order="F")
    g1, g2, g3 = (np.zeros_like(a, order="F") for a in (u1, u2, u3))
    rc = lib().orc_adjoint_f64(ctypes.byref(g), int(t_adv), int(iord), int(nonos), int(nsteps),
                               _ptr(x0, d), _ptr(bcx, d), _ptr(bcy, d), _ptr(u1, d), _ptr(u2, d),
                               _ptr(u3, d), _ptr(rhr, d), _ptr(h, d), _ptr(target, d), ctypes.byref(J),
                               _ptr(xN, d), _ptr(gx, d), _ptr(g1, d), _ptr(g2, d), _ptr(g3, d))
    if rc != 0:
        raise ValueError("oracle adjoint failed with code %d" % rc)
    return J.value, xN, gx, g1, g2, g3


def tangent_dJ(g, x0, bcx, bcy, u1, u2, u3, rhr, h, target, dx0, du1, du2, du3, t_adv=1, iord=2,
               nonos=1, nsteps=1):
    """Directional derivative of J along (dx0, du) by the tangent-linear model."""
    d = np.float64
    J = ctypes.c_double(0.0)
    dJ = ctypes.c_double(0.0)
    gx = np.zeros_like(x0, order="F")
    g1, g2, g3 = (np.zeros_like(a, order="F") for a in (u1, u2, u3))
    rc = lib().orc_tangent_adjoint_f64(ctypes.byref(g), int(t_adv), int(iord), int(nonos), int(nsteps),
                                       _ptr(x0, d), _ptr(bcx, d), _ptr(bcy, d), _ptr(u1, d), _ptr(u2, d),
                                       _ptr(u3, d), _ptr(rhr, d), _ptr(h, d), _ptr(target, d),
                                       ctypes.byref(J), None, _ptr(gx, d), _ptr(g1, d), _ptr(g2, d),
                                       _ptr(g3, d), _ptr(dx0, d), _ptr(du1, d), _ptr(du2, d), _ptr(du3, d),
                                       ctypes.byref(dJ))
    if rc != 0:
        raise ValueError("oracle tangent failed with code %d" % rc)
    return dJ.value


def a_to_c(g, uadv, vadv, wadv, u1, u2, u3):
    d = np.float64
    rc = lib().orc_a_to_c_f64(ctypes.byref(g), _ptr(uadv, d), _ptr(vadv, d), _ptr(wadv, d),
                              _ptr(u1, d), _ptr(u2, d), _ptr(u3, d))
    if rc != 0:
        raise ValueError("oracle a_to_c failed with code %d" % rc)
