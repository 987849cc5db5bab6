"""Host-side mirror of the reference's MPDATA interface over the C ABI.

Names, argument order and meaning follow the reference:

  advec_dwarf   advection/src_drivers/advec.f90:116-244 (the dwarf driver)
  Workspace     the module-global scratch of scratch_datafields_modular.f90:119-134,
                owned explicitly; .step() is upwind3d_gpubc + antidiff3d_*_gpubc,
                .velprd() is velprd_traj0 + velprdA_to_C + the driver's level roll
                (module_velprd.f90:15-364, velprd_driver.f90:254-270)

Arrays are CUDA tensors whose memory is Fortran-ordered with the reference's
halo extents (see `fortran_device` to make one from a numpy array).  Errors
raise MpdataError instead of the reference's STOP.  There is no CPU path: if
the CUDA library is not built or no GPU is present, calls fail.
"""
import numpy as np

from . import _native
from ._native import MpdataError, check

try:  # torch provides device memory and streams (plumbing only)
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _require_torch():
    if torch is None:
        raise RuntimeError("torch is required for device memory")


def fortran_device(a, device="cuda", dtype=None):
    """Copy a Fortran-ordered numpy array to a CUDA tensor with Fortran strides
    (logical shape equal to the numpy shape)."""
    _require_torch()
    a = np.asarray(a)
    if dtype is not None:
        a = a.astype(dtype)
    flat = np.ascontiguousarray(a.reshape(-1, order="F"))
    t = torch.from_numpy(flat).to(device)
    return t.reshape(tuple(reversed(a.shape))).permute(*reversed(range(a.ndim)))


def fortran_empty(shape, dtype, device="cuda"):
    _require_torch()
    t = torch.zeros(tuple(reversed(shape)), dtype=dtype, device=device)
    return t.permute(*reversed(range(len(shape))))


def to_numpy(t):
    """Fortran-ordered numpy copy of a Fortran-strided tensor."""
    h = t.detach().permute(*reversed(range(t.ndim))).contiguous().cpu().numpy()
    return np.asfortranarray(h.transpose(*reversed(range(h.ndim))))


def _is_fortran(t):
    st = 1
    for n, s in zip(t.shape, t.stride()):
        if n > 1 and s != st:
            return False
        st *= n
    return True


def _ptr(t, dtype, shape=None, name="array"):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor" % name)
    if t.dtype != dtype:
        raise ValueError("%s must be %s, got %s" % (name, dtype, t.dtype))
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError("%s must have shape %s (reference halo extents), got %s"
                         % (name, tuple(shape), tuple(t.shape)))
    if not _is_fortran(t):
        raise ValueError("%s must be Fortran-ordered" % name)
    return t.data_ptr()


def _stream(stream):
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def shapes(np_, mp, lp, ih):
    s = (np_ + 2 * ih, mp + 2 * ih, lp + 2 * ih)
    return dict(psi=s, u1=(s[0] + 1, s[1], s[2]), u2=(s[0], s[1] + 1, s[2]),
                u3=(s[0], s[1], s[2] + 1), bcx=(mp, lp, 2), bcy=(np_, lp, 2))


class Workspace:
    """Device scratch for one grid and option set (see mpdata_ws_create)."""

    def __init__(self, np_, mp, lp, ih=1, ibcx=0, ibcy=0, ibcz=0, iord=2, nonos=1, gauge=1,
                 precision=64):
        _require_torch()
        self.lib = _native.load()
        self.grid = _native.MpdataGrid(np_, mp, lp, ih, ibcx, ibcy, ibcz)
        self.opts = _native.MpdataOpts(iord, nonos, gauge, precision, 0)
        self.dtype = torch.float64 if precision == 64 else torch.float32
        self.shapes = shapes(np_, mp, lp, ih)
        h = _native.P()
        check(self.lib.mpdata_ws_create(self.grid, self.opts, h), "mpdata_ws_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            check(self.lib.mpdata_ws_destroy(self.handle), "mpdata_ws_destroy")
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, psi, u1, u2, u3, h, rhr, bcx=None, bcy=None, stream=None):
        """One MPDATA step, psi updated in place (upwind3d_gpubc +
        antidiff3d_gauge_gpubc / antidiff3d_standard_gpubc)."""
        s, d = self.shapes, self.dtype
        fn = self.lib.mpdata_step_f64 if self.opts.precision == 64 else self.lib.mpdata_step_f32
        check(fn(self.handle, _ptr(psi, d, s["psi"], "psi"), _ptr(u1, d, s["u1"], "u1"),
                 _ptr(u2, d, s["u2"], "u2"), _ptr(u3, d, s["u3"], "u3"), _ptr(h, d, s["psi"], "h"),
                 _ptr(rhr, d, s["psi"], "rhr"), _ptr(bcx, d, s["bcx"], "bcx"),
                 _ptr(bcy, d, s["bcy"], "bcy"), _stream(stream)), "mpdata_step")

    def velprd(self, ox, oy, oz, h, dxi, dyi, dzi, dt, dt_ratio, u1, u2, u3, u=None, v=None, w=None,
               stream=None):
        """Velocity predictor; ox/oy/oz (and u/v/w) are (..., 3) level stacks."""
        s, d = self.shapes, self.dtype
        lev = s["psi"] + (3,)
        fn = self.lib.mpdata_velprd_f64 if self.opts.precision == 64 else self.lib.mpdata_velprd_f32
        check(fn(self.handle, _ptr(ox, d, lev, "ox"), _ptr(oy, d, lev, "oy"), _ptr(oz, d, lev, "oz"),
                 _ptr(u, d, lev, "u"), _ptr(v, d, lev, "v"), _ptr(w, d, lev, "w"),
                 _ptr(h, d, s["psi"], "h"), dxi, dyi, dzi, dt, dt_ratio, _ptr(u1, d, s["u1"], "u1"),
                 _ptr(u2, d, s["u2"], "u2"), _ptr(u3, d, s["u3"], "u3"), _stream(stream)),
              "mpdata_velprd")

    def velprd_adjoint(self, gox, goy, goz, h, dxi, dyi, dzi, dt, dt_ratio, gu1, gu2, gu3, stream=None):
        """Adjoint of velprd (mpdata_velprd_adjoint_*): gu1..gu3 hold dJ/du;
        gox/goy/goz are (..., 3) gradient stacks (level 1: dJ/d(level 1), level
        2: dJ/d(the rolled level 2) on entry); level 0 accumulates dJ/d(level 0)
        and level 2 becomes dJ/d(the level 2 read)."""
        s, d = self.shapes, self.dtype
        lev = s["psi"] + (3,)
        fn = self.lib.mpdata_velprd_adjoint_f64 if self.opts.precision == 64 else self.lib.mpdata_velprd_adjoint_f32
        check(fn(self.handle, _ptr(h, d, s["psi"], "h"), dxi, dyi, dzi, dt, dt_ratio, _ptr(gu1, d, s["u1"], "gu1"),
                 _ptr(gu2, d, s["u2"], "gu2"), _ptr(gu3, d, s["u3"], "gu3"), _ptr(gox, d, lev, "gox"),
                 _ptr(goy, d, lev, "goy"), _ptr(goz, d, lev, "goz"), _stream(stream)),
              "mpdata_velprd_adjoint")

    def rho_gauge(self, ox, oy, oz, u1, u2, u3, x_in, x_incomp, h, rhoadv, rhr, pexe, pexr1, pexr2,
                  dxi, dyi, dzi, dt, dt_ratio, bcx=None, bcy=None, liner=0, u=None, v=None, w=None,
                  stream=None):
        """Density step mpdata3d_rho_gauge_gpubc (mpdata3d-rho-gauge-gpubc.f90:23-622):
        predictor, upwind keeping its fluxes, gauge antidiffusion; writes
        x_in, x_incomp, rhoadv, rhr, pexr1, pexr2 and the mass fluxes u1..u3."""
        s, d = self.shapes, self.dtype
        lev = s["psi"] + (3,)
        fn = self.lib.mpdata_rho_gauge_f64 if self.opts.precision == 64 else self.lib.mpdata_rho_gauge_f32
        ps = lambda t, n: _ptr(t, d, s["psi"], n)
        check(fn(self.handle, _ptr(ox, d, lev, "ox"), _ptr(oy, d, lev, "oy"), _ptr(oz, d, lev, "oz"),
                 _ptr(u, d, lev, "u"), _ptr(v, d, lev, "v"), _ptr(w, d, lev, "w"), _ptr(u1, d, s["u1"], "u1"),
                 _ptr(u2, d, s["u2"], "u2"), _ptr(u3, d, s["u3"], "u3"), ps(x_in, "x_in"),
                 ps(x_incomp, "x_incomp"), ps(h, "h"), ps(rhoadv, "rhoadv"), ps(rhr, "rhr"), ps(pexe, "pexe"),
                 ps(pexr1, "pexr1"), ps(pexr2, "pexr2"), _ptr(bcx, d, s["bcx"], "bcx"),
                 _ptr(bcy, d, s["bcy"], "bcy"), dxi, dyi, dzi, dt, dt_ratio, int(liner), _stream(stream)),
              "mpdata_rho_gauge")

    # the reference's name for the density step
    mpdata3d_rho_gauge_gpubc = rho_gauge

    def rho_gauge_adjoint(self, u1, u2, u3, x_in, x_incomp, h, pexe, lam, g_u1, g_u2, g_u3, g_xincomp, g_pexe,
                          l_u1=None, l_u2=None, l_u3=None, l_xincomp=None, l_pexr1=None, l_pexr2=None,
                          l_rhr=None, bcx=None, bcy=None, stream=None):
        """Reverse of the density step after its predictor (mpdata_rho_gauge_adjoint_*):
        u1..u3 are the C-grid Courant numbers the step advected with, x_in and
        x_incomp its inputs.  lam (dJ/dpsi after the step) becomes dJ/dpsi
        before it; the l_* cotangents of the mass fluxes, x_incomp, pexr1,
        pexr2 and rhr (None: zero) enter too.  dJ/du is added into
        g_u1..g_u3; g_xincomp and g_pexe receive dJ/d(x_incomp input) and
        dJ/dpexe on the interior."""
        s, d = self.shapes, self.dtype
        fn = (self.lib.mpdata_rho_gauge_adjoint_f64 if self.opts.precision == 64
              else self.lib.mpdata_rho_gauge_adjoint_f32)
        ps = lambda t, n: _ptr(t, d, s["psi"], n)
        check(fn(self.handle, _ptr(u1, d, s["u1"], "u1"), _ptr(u2, d, s["u2"], "u2"), _ptr(u3, d, s["u3"], "u3"),
                 ps(x_in, "x_in"), ps(x_incomp, "x_incomp"), ps(h, "h"), ps(pexe, "pexe"),
                 _ptr(bcx, d, s["bcx"], "bcx"), _ptr(bcy, d, s["bcy"], "bcy"), ps(lam, "lam"),
                 _ptr(l_u1, d, s["u1"], "l_u1"), _ptr(l_u2, d, s["u2"], "l_u2"), _ptr(l_u3, d, s["u3"], "l_u3"),
                 ps(l_xincomp, "l_xincomp"), ps(l_pexr1, "l_pexr1"), ps(l_pexr2, "l_pexr2"), ps(l_rhr, "l_rhr"),
                 _ptr(g_u1, d, s["u1"], "g_u1"), _ptr(g_u2, d, s["u2"], "g_u2"), _ptr(g_u3, d, s["u3"], "g_u3"),
                 ps(g_xincomp, "g_xincomp"), ps(g_pexe, "g_pexe"), _stream(stream)), "mpdata_rho_gauge_adjoint")

    def step_adjoint(self, psi_in, u1, u2, u3, h, rhr, lam, g_u1, g_u2, g_u3, bcx=None, bcy=None,
                     stream=None):
        """Reverse of one step: lam (dJ/dpsi_new) becomes dJ/dpsi_in; dJ/du is
        added into g_u1..g_u3.  psi_in is the field at the step's start."""
        s, d = self.shapes, self.dtype
        fn = self.lib.mpdata_step_adjoint_f64 if self.opts.precision == 64 else self.lib.mpdata_step_adjoint_f32
        check(fn(self.handle, _ptr(psi_in, d, s["psi"], "psi_in"), _ptr(u1, d, s["u1"], "u1"),
                 _ptr(u2, d, s["u2"], "u2"), _ptr(u3, d, s["u3"], "u3"), _ptr(h, d, s["psi"], "h"),
                 _ptr(rhr, d, s["psi"], "rhr"), _ptr(bcx, d, s["bcx"], "bcx"), _ptr(bcy, d, s["bcy"], "bcy"),
                 _ptr(lam, d, s["psi"], "lam"), _ptr(g_u1, d, s["u1"], "g_u1"), _ptr(g_u2, d, s["u2"], "g_u2"),
                 _ptr(g_u3, d, s["u3"], "g_u3"), _stream(stream)), "mpdata_step_adjoint")

    def adjoint_run(self, nsteps, psi, u1, u2, u3, h, rhr, target, g_psi0, g_u1, g_u2, g_u3, bcx=None,
                    bcy=None, interval=0, stream=None):
        """J = 0.5*|psi_N - target|^2 after nsteps steps and its gradients with
        sqrt(N) checkpointing.  psi: psi_0 in, psi_N out.  Returns (J, peak_bytes)."""
        import ctypes
        s, d = self.shapes, self.dtype
        fn = self.lib.mpdata_adjoint_run_f64 if self.opts.precision == 64 else self.lib.mpdata_adjoint_run_f32
        J = ctypes.c_double(0.0)
        peak = ctypes.c_longlong(0)
        check(fn(self.handle, int(nsteps), int(interval), _ptr(psi, d, s["psi"], "psi"), _ptr(u1, d, s["u1"], "u1"),
                 _ptr(u2, d, s["u2"], "u2"), _ptr(u3, d, s["u3"], "u3"), _ptr(h, d, s["psi"], "h"),
                 _ptr(rhr, d, s["psi"], "rhr"), _ptr(bcx, d, s["bcx"], "bcx"), _ptr(bcy, d, s["bcy"], "bcy"),
                 _ptr(target, d, s["psi"], "target"), J, _ptr(g_psi0, d, s["psi"], "g_psi0"),
                 _ptr(g_u1, d, s["u1"], "g_u1"), _ptr(g_u2, d, s["u2"], "g_u2"), _ptr(g_u3, d, s["u3"], "g_u3"),
                 peak, _stream(stream)), "mpdata_adjoint_run")
        return J.value, peak.value

    def profile(self, enable=True):
        """Start (or stop) per-stage CUDA-event timing of this workspace."""
        check(self.lib.mpdata_ws_profile(self.handle, 1 if enable else 0), "mpdata_ws_profile")

    def stage_times(self):
        """{stage name: (total ms, launches)} accumulated since profile()."""
        import ctypes
        n = 16
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_longlong * n)()
        rc = self.lib.mpdata_ws_stage_times(self.handle, n, ms, cnt)
        if rc < 0:
            check(rc, "mpdata_ws_stage_times")
        return {self.lib.mpdata_stage_name(i).decode(): (ms[i], cnt[i]) for i in range(rc)}

    def bound_violations(self, psi, tol=0.0, stream=None):
        """Cells of psi outside the limiter's running extrema of the last step
        (nonos, iord >= 3)."""
        import ctypes
        out = ctypes.c_longlong(0)
        check(self.lib.mpdata_ws_bound_violations(self.handle, _ptr(psi, self.dtype, self.shapes["psi"], "psi"),
                                                  float(tol), ctypes.byref(out), _stream(stream)),
              "mpdata_ws_bound_violations")
        return out.value

    def error_word(self):
        out = _native.I(0)
        check(self.lib.mpdata_ws_error(self.handle, out), "mpdata_ws_error")
        return out.value


class Batch:
    """Many MPDATA problems advanced together, one launch per stage
    (mpdata_batch_*).  `problems` is a list of dicts with keys np, mp, lp and
    optionally ibcx, ibcy, ibcz (default periodic), gauge (default 1) and
    velocity_group (default: the problem's own index)."""

    def __init__(self, problems, ih=1, iord=2, nonos=1, precision=64):
        _require_torch()
        self.lib = _native.load()
        arr = (_native.MpdataProblem * len(problems))()
        self.shapes = []
        for n, p in enumerate(problems):
            arr[n] = _native.MpdataProblem(p["np"], p["mp"], p["lp"], p.get("ibcx", 1), p.get("ibcy", 1),
                                           p.get("ibcz", 1), p.get("gauge", 1), p.get("velocity_group", n))
            self.shapes.append(shapes(p["np"], p["mp"], p["lp"], ih))
        self.problems = [dict(p) for p in problems]
        self.precision = precision
        self.dtype = torch.float64 if precision == 64 else torch.float32
        h = _native.P()
        check(self.lib.mpdata_batch_create(len(problems), arr, ih, iord, nonos, precision, h),
              "mpdata_batch_create")
        self.handle = h
        self._keep = {}

    def set(self, p, psi, u1, u2, u3, h, rhr, bcx=None, bcy=None):
        s, d = self.shapes[p], self.dtype
        check(self.lib.mpdata_batch_set(self.handle, p, _ptr(psi, d, s["psi"], "psi"), _ptr(u1, d, s["u1"], "u1"),
                                        _ptr(u2, d, s["u2"], "u2"), _ptr(u3, d, s["u3"], "u3"),
                                        _ptr(h, d, s["psi"], "h"), _ptr(rhr, d, s["psi"], "rhr"),
                                        _ptr(bcx, d, s["bcx"], "bcx"), _ptr(bcy, d, s["bcy"], "bcy")),
              "mpdata_batch_set")
        self._keep[p] = (psi, u1, u2, u3, h, rhr, bcx, bcy)  # keep the tensors alive

    def step(self, stream=None):
        check(self.lib.mpdata_batch_step(self.handle, _stream(stream)), "mpdata_batch_step")

    def graph(self, enable=True):
        check(self.lib.mpdata_batch_graph(self.handle, 1 if enable else 0), "mpdata_batch_graph")

    def tune(self, stream=None):
        bx, by = _native.I(0), _native.I(0)
        check(self.lib.mpdata_batch_tune(self.handle, _stream(stream), bx, by), "mpdata_batch_tune")
        return bx.value, by.value

    def shape(self, bx, by, stream=None):
        """Tile shape bx x by (a multiple of 32, at most 256 threads) without timing."""
        check(self.lib.mpdata_batch_set_shape(self.handle, int(bx), int(by), _stream(stream)),
              "mpdata_batch_set_shape")

    def profile(self, enable=True):
        check(self.lib.mpdata_batch_profile(self.handle, 1 if enable else 0), "mpdata_batch_profile")

    def stage_times(self):
        import ctypes
        n = 16
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_longlong * n)()
        rc = self.lib.mpdata_batch_stage_times(self.handle, n, ms, cnt)
        if rc < 0:
            check(rc, "mpdata_batch_stage_times")
        return {self.lib.mpdata_stage_name(i).decode(): (ms[i], cnt[i]) for i in range(rc)}

    def close(self):
        if getattr(self, "handle", None):
            check(self.lib.mpdata_batch_destroy(self.handle), "mpdata_batch_destroy")
            self.handle = None
            self._keep = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# Field order and antidiffusion choice of CE_advection
# (advection_CEtimestep_twostep_GPUBC.f90:150-159, 309-339): "mpdata3d" fields
# take the standard form unless mpdata_alg_choice is 1, "mpdatm3d" fields the
# gauge form unless it is 2.
CE_FIELDS = (("th", "mpdata3d"), ("u", "mpdatm3d"), ("v", "mpdatm3d"), ("w", "mpdatm3d"),
             ("tht", "mpdatm3d"), ("pstr", "mpdatm3d"), ("qv", "mpdata3d"), ("qc", "mpdata3d"),
             ("qr", "mpdata3d"), ("qi", "mpdata3d"), ("qs", "mpdata3d"), ("qg", "mpdata3d"))


def ce_form(kind, mpdata_alg_choice):
    """1 = gauge, 0 = standard, for a CE_advection field kind."""
    if mpdata_alg_choice == 1:
        return 1
    if mpdata_alg_choice == 2:
        return 0
    return 1 if kind == "mpdatm3d" else 0


_ce_cache = {}


def ce_advection(mpdata_alg_choice, liner, ipoles, ibcx, ibcy, ibcz, np_, mp, lp, ih, rhr, rhoadv,
                 uadv, vadv, wadv, stream=None, **fields):
    """The reference's multi-field step CE_advection
    (advection_CEtimestep_twostep_GPUBC.f90:27-376) on CUDA tensors: every
    field given as name=(x, x_lr, x_bt) (th, u, v, w, tht, pstr required;
    qv, qc, qr, qi, qs, qg optional) is advected by the shared velocity in ONE
    batched step.  liner=1 stops after the upwind pass, as the reference does."""
    if ipoles != 0:
        raise MpdataError(-7, "ce_advection")
    names = [n for n, _ in CE_FIELDS if n in fields]
    for req in ("th", "u", "v", "w", "tht", "pstr"):
        if req not in fields:
            raise ValueError("ce_advection needs field %r" % req)
    unknown = set(fields) - {n for n, _ in CE_FIELDS}
    if unknown:
        raise ValueError("unknown fields %s" % sorted(unknown))
    kinds = dict(CE_FIELDS)
    forms = tuple(ce_form(kinds[n], mpdata_alg_choice) for n in names)
    prec = 64 if uadv.dtype == torch.float64 else 32
    iord = 1 if liner else 2
    key = (np_, mp, lp, ih, ibcx, ibcy, ibcz, forms, prec, iord)
    b = _ce_cache.get(key)
    if b is None:
        probs = [dict(np=np_, mp=mp, lp=lp, ibcx=ibcx, ibcy=ibcy, ibcz=ibcz, gauge=f, velocity_group=0)
                 for f in forms]
        b = _ce_cache[key] = Batch(probs, ih=ih, iord=iord, nonos=1, precision=prec)
    for p, n in enumerate(names):
        x, x_lr, x_bt = fields[n]
        b.set(p, x, uadv, vadv, wadv, rhoadv, rhr, x_lr, x_bt)
    b.step(stream)


def advec_dwarf(legacyoptmode, t_adv, lupdatemulti, lvertsplit, np_, mp, lp, ih, ipoles, ibcx, ibcy,
                ibcz, x, x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv, iord=2, nonos=1, stream=None):
    """The reference's dwarf driver (advec.f90:116-244) on CUDA tensors."""
    _require_torch()
    lib = _native.load()
    d = x.dtype
    if d not in (torch.float64, torch.float32):
        raise ValueError("x must be float64 or float32")
    s = shapes(np_, mp, lp, ih) if min(np_, mp, lp, ih) > 0 else None
    g = (lambda k: s[k]) if s else (lambda k: None)
    fn = lib.mpdata_advec_dwarf_f64 if d == torch.float64 else lib.mpdata_advec_dwarf_f32
    check(fn(legacyoptmode, t_adv, int(bool(lupdatemulti)), int(bool(lvertsplit)), np_, mp, lp, ih,
             ipoles, ibcx, ibcy, ibcz, _ptr(x, d, g("psi"), "x"), _ptr(x_lr, d, g("bcx"), "x_lr"),
             _ptr(x_bt, d, g("bcy"), "x_bt"), _ptr(uadv, d, g("u1"), "uadv"),
             _ptr(vadv, d, g("u2"), "vadv"), _ptr(wadv, d, g("u3"), "wadv"),
             _ptr(rhr, d, g("psi"), "rhr"), _ptr(rhoadv, d, g("psi"), "rhoadv"), iord, nonos,
             _stream(stream)), "advec_dwarf")


def compute_courants(ntimelevel, ox, oy, oz, h, dxi, dyi, dzi, dt, np_, mp, lp, ih, stream=None):
    """compute_courants (common/diagutils.f90:588-672) on CUDA level stacks
    ox/oy/oz (..., 3): returns (cr3d, crxy, crxz, cryz, crx, cry, crz)."""
    _require_torch()
    import ctypes
    lib = _native.load()
    d = ox.dtype
    s = shapes(np_, mp, lp, ih)
    lev = s["psi"] + (3,)
    ct = ctypes.c_double if d == torch.float64 else ctypes.c_float
    cr = (ct * 7)()
    fn = lib.mpdata_compute_courants_f64 if d == torch.float64 else lib.mpdata_compute_courants_f32
    check(fn(ctypes.cast(cr, ctypes.c_void_p), _ptr(ox, d, lev, "ox"), _ptr(oy, d, lev, "oy"),
             _ptr(oz, d, lev, "oz"), _ptr(h, d, s["psi"], "h"), int(ntimelevel), dxi, dyi, dzi, dt,
             np_, mp, lp, ih, _stream(stream)), "mpdata_compute_courants")
    return tuple(float(c) for c in cr)


def velprd_driver(state, ox, oy, oz, u, v, w, uadv, vadv, wadv, h, ipoles, ibcx, ibcy, ibcz, np_, mp, lp, ih,
                  dxi, dyi, dzi, dt, stream=None):
    """velprd_driver (advection/src_algorithms/velprd_driver.f90:16-270) on
    CUDA tensors.  state is a dict with the reference's scalars: nsubsteps,
    nsubsteps_o, dtn, dtnold (INOUT, updated in place), lsubstepping,
    ltimeadapt, lvertsplit, lcrdiag_nphlf, crmaxlim, dtmax.  Returns the last
    (cr3d, crxy, crxz, cryz, crx, cry, crz, cr_for_dt, dt_ratio)."""
    _require_torch()
    import ctypes
    lib = _native.load()
    d = ox.dtype
    s = shapes(np_, mp, lp, ih)
    lev = s["psi"] + (3,)
    R = ctypes.c_double if d == torch.float64 else ctypes.c_float
    ns, nso = ctypes.c_int(state["nsubsteps"]), ctypes.c_int(state["nsubsteps_o"])
    dtn, dtnold = R(state["dtn"]), R(state["dtnold"])
    diag = (ctypes.c_double * 9)()
    fn = lib.mpdata_velprd_driver_f64 if d == torch.float64 else lib.mpdata_velprd_driver_f32
    check(fn(ctypes.byref(ns), ctypes.byref(nso), int(state["lsubstepping"]), ctypes.byref(dtn),
             ctypes.byref(dtnold), int(state["ltimeadapt"]), int(state["lvertsplit"]), int(state["lcrdiag_nphlf"]),
             state["crmaxlim"], state["dtmax"], _ptr(ox, d, lev, "ox"), _ptr(oy, d, lev, "oy"),
             _ptr(oz, d, lev, "oz"), _ptr(u, d, lev, "u"), _ptr(v, d, lev, "v"), _ptr(w, d, lev, "w"),
             _ptr(uadv, d, s["u1"], "uadv"), _ptr(vadv, d, s["u2"], "vadv"), _ptr(wadv, d, s["u3"], "wadv"),
             _ptr(h, d, s["psi"], "h"), ipoles, ibcx, ibcy, ibcz, np_, mp, lp, ih, dxi, dyi, dzi, dt,
             ctypes.cast(diag, ctypes.c_void_p), _stream(stream)), "mpdata_velprd_driver")
    state.update(nsubsteps=ns.value, nsubsteps_o=nso.value, dtn=dtn.value, dtnold=dtnold.value)
    return tuple(diag)


def pnet_out_chunk(var_name, file_name, imode, ifrmd, var, np_, mp, lp, ih, ia1=0, ia2=0, ia3=0, imem=0,
                   stream=None):
    """pnet_out_chunk (common/mpi_parallel.f90:7481) from a Fortran-ordered
    CUDA tensor or numpy array of extents n+ia*imem+2*ih per axis (psi-shaped
    when imem is 0): the full 3-D modes (0 float, 1 double, 34 float without
    time), the staggered blocks 2-4, the halo strips 6-9, the planes 10-13 and
    35, the lines 20-22 and the point variable 30; writes netCDF classic
    (64-bit offset)."""
    lib = _native.load()
    dev = torch is not None and isinstance(var, torch.Tensor)
    if dev:
        d = var.dtype
        shape = (np_ + ia1 * imem + 2 * ih, mp + ia2 * imem + 2 * ih, lp + ia3 * imem + 2 * ih)
        ptr = _ptr(var, d, shape, "var")
        f64 = d == torch.float64
    else:
        if not var.flags.f_contiguous:
            raise ValueError("var must be Fortran-ordered")
        ptr = var.ctypes.data
        f64 = var.dtype == np.float64
    fn = lib.mpdata_pnet_out_chunk_f64 if f64 else lib.mpdata_pnet_out_chunk_f32
    check(fn(var_name.encode(), str(file_name).encode(), int(imode), int(ia1), int(ia2), int(ia3), int(ifrmd),
             int(imem), ptr, np_, mp, lp, ih, 1 if dev else 0, _stream(stream) if dev else None),
          "mpdata_pnet_out_chunk")


def pnet_in_chunk(var_name, file_name, ifrmd, var, np_, mp, lp, ih, stream=None):
    """Frame ifrmd of a netCDF classic variable into the interior of var."""
    lib = _native.load()
    dev = torch is not None and isinstance(var, torch.Tensor)
    if dev:
        ptr = _ptr(var, var.dtype, shapes(np_, mp, lp, ih)["psi"], "var")
        f64 = var.dtype == torch.float64
    else:
        ptr = var.ctypes.data
        f64 = var.dtype == np.float64
    fn = lib.mpdata_pnet_in_chunk_f64 if f64 else lib.mpdata_pnet_in_chunk_f32
    check(fn(var_name.encode(), str(file_name).encode(), int(ifrmd), ptr, np_, mp, lp, ih, 1 if dev else 0,
             _stream(stream) if dev else None), "mpdata_pnet_in_chunk")


def mass(psi, h, rhr=None, ibc=(1, 1, 1), ih=1, stream=None):
    """FP64 Neumaier-compensated sum(h*psi[/rhr]) over the interior."""
    import ctypes
    n = [d - 2 * ih for d in psi.shape]
    g = _native.MpdataGrid(n[0], n[1], n[2], ih, *ibc)
    lib = _native.load()
    out = ctypes.c_double(0.0)
    fn = lib.mpdata_mass_f64 if psi.dtype == torch.float64 else lib.mpdata_mass_f32
    d = psi.dtype
    check(fn(g, _ptr(psi, d, None, "psi"), _ptr(h, d, tuple(psi.shape), "h"),
             _ptr(rhr, d, tuple(psi.shape), "rhr"), out, _stream(stream)), "mpdata_mass")
    return out.value


def error_norms(a, b, ibc=(1, 1, 1), ih=1, stream=None):
    """(max|a-b|, ||a-b||_2, max|b|, ||b||_2) over the interior, FP64."""
    import ctypes
    if tuple(a.shape) != tuple(b.shape):
        raise ValueError("a and b must have the same shape")
    n = [d - 2 * ih for d in a.shape]
    g = _native.MpdataGrid(n[0], n[1], n[2], ih, *ibc)
    out = (ctypes.c_double * 4)()
    check(_native.load().mpdata_error_norms(g, _ptr(a, a.dtype, None, "a"), int(a.dtype == torch.float64),
                                            _ptr(b, b.dtype, None, "b"), int(b.dtype == torch.float64), out,
                                            _stream(stream)), "mpdata_error_norms")
    return tuple(out)


def release_cached():
    check(_native.load().mpdata_release_cached(), "mpdata_release_cached")


def launch_count():
    return int(_native.load().mpdata_launch_count())


__all__ = ["Workspace", "Batch", "ce_advection", "advec_dwarf", "fortran_device", "fortran_empty", "to_numpy", "MpdataError",
           "release_cached", "launch_count", "shapes", "mass", "error_norms"]
