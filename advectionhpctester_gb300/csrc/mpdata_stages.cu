// Stage kernels of the MPDATA step (strict-IEEE path).
//
// One kernel per stage of the reference's antidiffusive iteration, one thread
// per cell, with every face quantity computed exactly once (the reference
// recomputes shared faces per cell).  Scratch fields are interior-shaped;
// boundary conditions are index maps applied when a neighbour is read, so no
// halo-fill kernels run:
//   psi halo     Dirichlet bcx/bcy (putbcinxh, mpdataoperators.inc:253-287) or wrap
//   xant halo    reflection x(0)=x(2) (cp_scnd_last_to_halo_xy_fulld, :479-513) or wrap
//   x_in halo    zero gradient x(0)=x(1) (cp_last_to_halo_xy, :551-584) or wrap
//   face fields  0 on open x/y walls (flux_x_bcd/flux_y_bcd type 0, :673-811),
//                mirrored on z walls (flux_z_bc_nohalod type 2, :903-947), or wrap
// Built with --fmad=false and IEEE division so results are bit-identical to
// a strict-IEEE CPU evaluation of the reference's expressions.
#include "mpdata_common.cuh"
#include "mpdata_stages.cuh"

namespace mpdata {

// ---- read helpers -------------------------------------------------------
__device__ __forceinline__ int cx(const Geo& g, int i) { return g.bx ? wrapi(i, g.np) : clampi(i, g.np); }
__device__ __forceinline__ int cy(const Geo& g, int j) { return g.by ? wrapi(j, g.mp) : clampi(j, g.mp); }
__device__ __forceinline__ int cz(const Geo& g, int k) { return g.bz ? wrapi(k, g.lp) : clampi(k, g.lp); }

// the current (antidiffused) field with the xant halo rule
template <class R>
__device__ __forceinline__ R xr(const Geo& g, const Arr<R>& X, int i, int j, int k) {
  return X.ld(g.bx ? wrapi(i, g.np) : refl(i, g.np), g.by ? wrapi(j, g.mp) : refl(j, g.mp), cz(g, k));
}

// Face fields.  AIN = the caller's C-grid Courant numbers (faces 1..n+1 are
// data on open axes); otherwise an antidiffusive field stored for faces 1..n
// with the wall rule applied on read.
template <class R, bool AIN>
__device__ __forceinline__ R fx(const Geo& g, const Arr<R>& A, int f, int j, int k) {
  j = cy(g, j);
  k = cz(g, k);
  if (g.bx) return A.ld(wrapi(f, g.np), j, k);
  if (AIN) return A.ld(f, j, k);
  return (f <= 1 || f > g.np) ? R(0) : A.ld(f, j, k);
}
template <class R, bool AIN>
__device__ __forceinline__ R fy(const Geo& g, const Arr<R>& A, int i, int f, int k) {
  i = cx(g, i);
  k = cz(g, k);
  if (g.by) return A.ld(i, wrapi(f, g.mp), k);
  if (AIN) return A.ld(i, f, k);
  return (f <= 1 || f > g.mp) ? R(0) : A.ld(i, f, k);
}
template <class R, bool AIN>
__device__ __forceinline__ R fz(const Geo& g, const Arr<R>& A, int i, int j, int f) {
  i = cx(g, i);
  j = cy(g, j);
  if (g.bz) return A.ld(i, j, wrapi(f, g.lp));
  if (AIN) return A.ld(i, j, f);
  if (f <= 1) return -A.ld(i, j, 2);
  if (f > g.lp) return -A.ld(i, j, g.lp);
  return A.ld(i, j, f);
}

#define CELL_INDEX                                          \
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1; \
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1; \
  const int k = blockIdx.z + 1;                             \
  if (i > g.np || j > g.mp) return;

// ---- upwind3d_gpubc (upwind3d-gpubc.f90:101-198) -------------------------
// ANTIDIFF: an antidiffusive pass follows, so psi's open-wall halo ends the
// step holding the zero-gradient copy of the old boundary values (written by
// cp_last_to_halo_xy in the antidiffusion); otherwise it keeps bcx/bcy.
template <class R, bool ANTIDIFF>
__global__ void __launch_bounds__(128) k_upwind(Geo g, Arr<R> psi, Arr<R> u1, Arr<R> u2, Arr<R> u3,
                                                Arr<R> h, Arr<R> rhr, const R* __restrict__ bcx,
                                                const R* __restrict__ bcy, Arr<R> xant, Arr<R> hinv) {
  CELL_INDEX
  const R x = psi.ld(i, j, k);
  const long bx0 = (long)(j - 1) + (long)g.mp * (k - 1), bxs = (long)g.mp * g.lp;
  const long by0 = (long)(i - 1) + (long)g.np * (k - 1), bys = (long)g.np * g.lp;
  const R xim = i > 1 ? psi.ld(i - 1, j, k) : (g.bx ? psi.ld(g.np, j, k) : bcx[bx0]);
  const R xip = i < g.np ? psi.ld(i + 1, j, k) : (g.bx ? psi.ld(1, j, k) : bcx[bx0 + bxs]);
  const R xjm = j > 1 ? psi.ld(i, j - 1, k) : (g.by ? psi.ld(i, g.mp, k) : bcy[by0]);
  const R xjp = j < g.mp ? psi.ld(i, j + 1, k) : (g.by ? psi.ld(i, 1, k) : bcy[by0 + bys]);
  const R hi = R(1) / h.ld(i, j, k);
  const R f1p = donor(x, xip, fx<R, true>(g, u1, i + 1, j, k));
  const R f1 = donor(xim, x, u1.ld(i, j, k));
  const R f2p = donor(x, xjp, fy<R, true>(g, u2, i, j + 1, k));
  const R f2 = donor(xjm, x, u2.ld(i, j, k));
  R f3p, f3;
  if (!g.bz && k == 1) {  // :134-135
    f3p = donor(x, psi.ld(i, j, k + 1), u3.ld(i, j, k + 1));
    f3 = -f3p;
  } else if (!g.bz && k == g.lp) {  // :164-165
    f3 = donor(psi.ld(i, j, k - 1), x, u3.ld(i, j, k));
    f3p = -f3;
  } else {
    f3p = donor(x, psi.ld(i, j, cz(g, k + 1)), fz<R, true>(g, u3, i, j, k + 1));
    f3 = donor(psi.ld(i, j, cz(g, k - 1)), x, u3.ld(i, j, k));
  }
  xant.at(i, j, k) = rhr.ld(i, j, k) * (x - (f1p - f1 + f2p - f2 + f3p - f3) * hi);
  hinv.at(i, j, k) = hi;
  if (!g.bx) {
    if (i == 1) psi.at(0, j, k) = ANTIDIFF ? x : xim;
    if (i == g.np) psi.at(g.np + 1, j, k) = ANTIDIFF ? x : xip;
  }
  if (!g.by) {
    if (j == 1) psi.at(i, 0, k) = ANTIDIFF ? x : xjm;
    if (j == g.mp) psi.at(i, g.mp + 1, k) = ANTIDIFF ? x : xjp;
  }
}

template <class R>
__global__ void __launch_bounds__(128) k_copy(Geo g, Arr<R> src, Arr<R> dst) {
  CELL_INDEX
  dst.at(i, j, k) = src.ld(i, j, k);
}

// ---- antidiffusive pseudo-velocities --------------------------------------
// standard form: antidiff3d-standard-gpubc.f90:72-203; gauge form:
// antidiff3d-gauge-gpubc.f90:89-203.  The k=1 and k=lp planes of a z wall
// drop the z cross terms of v1/v2, as the reference's boundary kernels do.
// Each cell computes its lower faces; wall faces follow the read rules.
template <class R, bool STD, bool AIN>
__global__ void __launch_bounds__(128) k_pseudo(Geo g, Arr<R> X, Arr<R> A1, Arr<R> A2, Arr<R> A3,
                                                Arr<R> h, Arr<R> v1, Arr<R> v2, Arr<R> v3,
                                                Arr<R> fn1, Arr<R> fn2, Arr<R> fn3) {
  CELL_INDEX
  const R ep = Eps<R>::v;
  const bool zt = g.bz || (k > 1 && k < g.lp);
  const R hc = h.ld(i, j, k);
#define XX(a, b, c) xr<R>(g, X, (a), (b), (c))
#define AX(f, b, c) fx<R, AIN>(g, A1, (f), (b), (c))
#define AY(a, f, c) fy<R, AIN>(g, A2, (a), (f), (c))
#define AZ(a, b, f) fz<R, AIN>(g, A3, (a), (b), (f))
  if (g.bx || i > 1) {
    const R hmx = R(1) / (R(0.5) * (h.ld(cx(g, i - 1), j, k) + hc));
    const R a = AX(i, j, k);
    R v;
    if (STD) {
      v = vdyfa(XX(i - 1, j, k), XX(i, j, k), a, hmx, ep) +
          vcorra(a, AY(i - 1, j, k) + AY(i - 1, j + 1, k) + AY(i, j + 1, k) + AY(i, j, k),
                 (fabs(XX(i - 1, j + 1, k)) + fabs(XX(i, j + 1, k))) -
                     (fabs(XX(i - 1, j - 1, k)) + fabs(XX(i, j - 1, k))),
                 fabs(XX(i - 1, j + 1, k)) + fabs(XX(i, j + 1, k)) + fabs(XX(i - 1, j - 1, k)) +
                     fabs(XX(i, j - 1, k)) + ep,
                 hmx);
      if (zt)
        v = v + vcorra(a, AZ(i - 1, j, k) + AZ(i - 1, j, k + 1) + AZ(i, j, k + 1) + AZ(i, j, k),
                       (fabs(XX(i - 1, j, k + 1)) + fabs(XX(i, j, k + 1))) -
                           (fabs(XX(i - 1, j, k - 1)) + fabs(XX(i, j, k - 1))),
                       fabs(XX(i - 1, j, k + 1)) + fabs(XX(i, j, k + 1)) + fabs(XX(i - 1, j, k - 1)) +
                           fabs(XX(i, j, k - 1)) + ep,
                       hmx);
      fn1.at(i, j, k) = donor(XX(i - 1, j, k), XX(i, j, k), v);
    } else {
      const R c2 = (AY(i - 1, j, k) + AY(i - 1, j + 1, k) + AY(i, j + 1, k) + AY(i, j, k)) *
                   rat4(XX(i - 1, j - 1, k), XX(i, j - 1, k), XX(i - 1, j + 1, k), XX(i, j + 1, k));
      R cr = c2;
      if (zt)
        cr = c2 + (AZ(i - 1, j, k) + AZ(i - 1, j, k + 1) + AZ(i, j, k + 1) + AZ(i, j, k)) *
                      rat4(XX(i - 1, j, k - 1), XX(i, j, k - 1), XX(i - 1, j, k + 1), XX(i, j, k + 1));
      v = vdyf(XX(i - 1, j, k), XX(i, j, k), a, hmx) - R(0.125) * a * hmx * cr;
    }
    v1.at(i, j, k) = v;
  }
  if (g.by || j > 1) {
    const R hmy = R(1) / (R(0.5) * (h.ld(i, cy(g, j - 1), k) + hc));
    const R a = AY(i, j, k);
    R v;
    if (STD) {
      v = vdyfa(XX(i, j - 1, k), XX(i, j, k), a, hmy, ep) +
          vcorra(a, AX(i, j - 1, k) + AX(i, j, k) + AX(i + 1, j, k) + AX(i + 1, j - 1, k),
                 (fabs(XX(i + 1, j - 1, k)) + fabs(XX(i + 1, j, k))) -
                     (fabs(XX(i - 1, j - 1, k)) + fabs(XX(i - 1, j, k))),
                 fabs(XX(i + 1, j - 1, k)) + fabs(XX(i + 1, j, k)) + fabs(XX(i - 1, j - 1, k)) +
                     fabs(XX(i - 1, j, k)) + ep,
                 hmy);
      if (zt)
        v = v + vcorra(a, AZ(i, j - 1, k) + AZ(i, j, k) + AZ(i, j, k + 1) + AZ(i, j - 1, k + 1),
                       (fabs(XX(i, j - 1, k + 1)) + fabs(XX(i, j, k + 1))) -
                           (fabs(XX(i, j - 1, k - 1)) + fabs(XX(i, j, k - 1))),
                       fabs(XX(i, j - 1, k + 1)) + fabs(XX(i, j, k + 1)) + fabs(XX(i, j - 1, k - 1)) +
                           fabs(XX(i, j, k - 1)) + ep,
                       hmy);
      fn2.at(i, j, k) = donor(XX(i, j - 1, k), XX(i, j, k), v);
    } else {
      const R c1 = (AX(i, j - 1, k) + AX(i, j, k) + AX(i + 1, j, k) + AX(i + 1, j - 1, k)) *
                   rat4(XX(i - 1, j - 1, k), XX(i - 1, j, k), XX(i + 1, j - 1, k), XX(i + 1, j, k));
      R cr = c1;
      if (zt)
        cr = c1 + (AZ(i, j - 1, k) + AZ(i, j, k) + AZ(i, j, k + 1) + AZ(i, j - 1, k + 1)) *
                      rat4(XX(i, j - 1, k - 1), XX(i, j, k - 1), XX(i, j - 1, k + 1), XX(i, j, k + 1));
      v = vdyf(XX(i, j - 1, k), XX(i, j, k), a, hmy) - R(0.125) * a * hmy * cr;
    }
    v2.at(i, j, k) = v;
  }
  if (g.bz || k > 1) {
    const R hmz = R(1) / (R(0.5) * (h.ld(i, j, cz(g, k - 1)) + hc));
    const R a = AZ(i, j, k);
    R v;
    if (STD) {
      v = vdyfa(XX(i, j, k - 1), XX(i, j, k), a, hmz, ep) +
          vcorra(a, AX(i, j, k - 1) + AX(i, j, k) + AX(i + 1, j, k) + AX(i + 1, j, k - 1),
                 (fabs(XX(i + 1, j, k - 1)) + fabs(XX(i + 1, j, k))) -
                     (fabs(XX(i - 1, j, k - 1)) + fabs(XX(i - 1, j, k))),
                 fabs(XX(i + 1, j, k - 1)) + fabs(XX(i + 1, j, k)) + fabs(XX(i - 1, j, k - 1)) +
                     fabs(XX(i - 1, j, k)) + ep,
                 hmz) +
          vcorra(a, AY(i, j, k - 1) + AY(i, j + 1, k - 1) + AY(i, j + 1, k) + AY(i, j, k),
                 (fabs(XX(i, j + 1, k - 1)) + fabs(XX(i, j + 1, k))) -
                     (fabs(XX(i, j - 1, k - 1)) + fabs(XX(i, j - 1, k))),
                 fabs(XX(i, j + 1, k - 1)) + fabs(XX(i, j + 1, k)) + fabs(XX(i, j - 1, k - 1)) +
                     fabs(XX(i, j - 1, k)) + ep,
                 hmz);
      fn3.at(i, j, k) = donor(XX(i, j, k - 1), XX(i, j, k), v);
    } else {
      const R cr = (AX(i, j, k - 1) + AX(i, j, k) + AX(i + 1, j, k) + AX(i + 1, j, k - 1)) *
                       rat4(XX(i - 1, j, k - 1), XX(i - 1, j, k), XX(i + 1, j, k - 1), XX(i + 1, j, k)) +
                   (AY(i, j, k - 1) + AY(i, j + 1, k - 1) + AY(i, j + 1, k) + AY(i, j, k)) *
                       rat4(XX(i, j - 1, k - 1), XX(i, j - 1, k), XX(i, j + 1, k - 1), XX(i, j + 1, k));
      v = vdyf(XX(i, j, k - 1), XX(i, j, k), a, hmz) - R(0.125) * a * hmz * cr;
    }
    v3.at(i, j, k) = v;
  }
#undef XX
#undef AX
#undef AY
#undef AZ
}

// ---- limiter bounds and ratios (std :256-348, gauge :238-324) -------------
// FIRST folds the star of the step's input field x_in (zero-gradient halo)
// into the bounds, as every first corrective pass does; later passes start
// from the stored running extrema.  The gauge k=1 minimum over x_in, which the
// reference leaves unset (antidiff3d-gauge-gpubc.f90:249), is computed as in
// mpdata3d-rho-gauge-gpubc.f90:365-368.  Also stores q = x/rhr, the ratio every
// later stage divides out.
template <class R, bool NONOS, bool FIRST, bool KEEP>
__global__ void __launch_bounds__(128) k_bounds(Geo g, Arr<R> X, Arr<R> xin, Arr<R> mx, Arr<R> mn,
                                                Arr<R> h, Arr<R> rhr, Arr<R> F1, Arr<R> F2, Arr<R> F3,
                                                Arr<R> cp, Arr<R> cn, Arr<R> q) {
  CELL_INDEX
  const R x = X.ld(i, j, k);
  q.at(i, j, k) = x / rhr.ld(i, j, k);
  if (!NONOS) return;
  const bool lo = g.bz || k > 1, hi = g.bz || k < g.lp;
  R ma, mi;
  if (FIRST) {
    const int im = g.bx ? wrapi(i - 1, g.np) : clampi(i - 1, g.np);
    const int ip = g.bx ? wrapi(i + 1, g.np) : clampi(i + 1, g.np);
    const int jm = g.by ? wrapi(j - 1, g.mp) : clampi(j - 1, g.mp);
    const int jp = g.by ? wrapi(j + 1, g.mp) : clampi(j + 1, g.mp);
    const R a0 = xin.ld(im, j, k), a1 = xin.ld(i, j, k), a2 = xin.ld(ip, j, k), a3 = xin.ld(i, jm, k),
            a4 = xin.ld(i, jp, k);
    ma = mx2(mx2(mx2(a0, a1), mx2(a2, a3)), a4);
    mi = mn2(mn2(mn2(a0, a1), mn2(a2, a3)), a4);
    if (lo) { const R t = xin.ld(i, j, cz(g, k - 1)); ma = mx2(ma, t); mi = mn2(mi, t); }
    if (hi) { const R t = xin.ld(i, j, cz(g, k + 1)); ma = mx2(ma, t); mi = mn2(mi, t); }
  } else {
    ma = mx.ld(i, j, k);
    mi = mn.ld(i, j, k);
  }
  {
    const R b0 = xr<R>(g, X, i - 1, j, k), b2 = xr<R>(g, X, i + 1, j, k), b3 = xr<R>(g, X, i, j - 1, k),
            b4 = xr<R>(g, X, i, j + 1, k);
    ma = mx2(mx2(mx2(ma, b0), mx2(x, b2)), mx2(b3, b4));
    mi = mn2(mn2(mn2(mi, b0), mn2(x, b2)), mn2(b3, b4));
    if (lo) { const R t = X.ld(i, j, cz(g, k - 1)); ma = mx2(ma, t); mi = mn2(mi, t); }
    if (hi) { const R t = X.ld(i, j, cz(g, k + 1)); ma = mx2(ma, t); mi = mn2(mi, t); }
  }
  if (KEEP) {
    mx.at(i, j, k) = ma;
    mn.at(i, j, k) = mi;
  }
  const R ep = Eps<R>::v;
  const R e1 = fx<R, false>(g, F1, i + 1, j, k), w1 = fx<R, false>(g, F1, i, j, k);
  const R e2 = fy<R, false>(g, F2, i, j + 1, k), w2 = fy<R, false>(g, F2, i, j, k);
  const R e3 = fz<R, false>(g, F3, i, j, k + 1), w3 = fz<R, false>(g, F3, i, j, k);
  const R hc = h.ld(i, j, k);
  cp.at(i, j, k) = (ma - x) * hc / (pn(e1) + pp(w1) + pn(e2) + pp(w2) + pn(e3) + pp(w3) + ep);
  cn.at(i, j, k) = (x - mi) * hc / (pp(e1) + pn(w1) + pp(e2) + pn(w2) + pp(e3) + pn(w3) + ep);
}

// ---- limited antidiffusive velocities and fluxes --------------------------
// std: antidiff3d-standard-gpubc.f90:372-407 (sign-aware limited velocity,
// donor flux of x/rhr); gauge: antidiff3d-gauge-gpubc.f90:343-363 (the
// limited velocity is the flux).  Lower faces of each cell.
template <class R>
__device__ __forceinline__ R vlim_std(R v, R a1, R a2, R xl, R xrr) {
  return pp(v) * (a1 * possign(xl) + a2 * possign(-xl)) - pn(v) * (a2 * possign(xrr) + a1 * possign(-xrr));
}

template <class R, bool STD, bool NONOS>
__global__ void __launch_bounds__(128) k_limit(Geo g, Arr<R> X, Arr<R> v1, Arr<R> v2, Arr<R> v3,
                                               Arr<R> cp, Arr<R> cn, Arr<R> q, Arr<R> w1, Arr<R> w2,
                                               Arr<R> w3, Arr<R> f1, Arr<R> f2, Arr<R> f3) {
  CELL_INDEX
  const R cpc = NONOS ? cp.ld(i, j, k) : R(0), cnc = NONOS ? cn.ld(i, j, k) : R(0);
  const R xc = X.ld(i, j, k), qc = STD ? q.ld(i, j, k) : R(0);
  if (g.bx || i > 1) {
    const int im = wrapi(i - 1, g.np);
    const R v = v1.ld(i, j, k);
    R w = v;
    if (NONOS) {
      const R cpm = cp.ld(im, j, k), cnm = cn.ld(im, j, k);
      w = STD ? vlim_std(v, min3(cpc, cnm), min3(cpm, cnc), X.ld(im, j, k), xc)
              : pp(v) * min3(cpc, cnm) - pn(v) * min3(cpm, cnc);
    }
    w1.at(i, j, k) = w;
    if (STD) f1.at(i, j, k) = donor(q.ld(im, j, k), qc, w);
  }
  if (g.by || j > 1) {
    const int jm = wrapi(j - 1, g.mp);
    const R v = v2.ld(i, j, k);
    R w = v;
    if (NONOS) {
      const R cpm = cp.ld(i, jm, k), cnm = cn.ld(i, jm, k);
      w = STD ? vlim_std(v, min3(cpc, cnm), min3(cpm, cnc), X.ld(i, jm, k), xc)
              : pp(v) * min3(cpc, cnm) - pn(v) * min3(cpm, cnc);
    }
    w2.at(i, j, k) = w;
    if (STD) f2.at(i, j, k) = donor(q.ld(i, jm, k), qc, w);
  }
  if (g.bz || k > 1) {
    const int km = wrapi(k - 1, g.lp);
    const R v = v3.ld(i, j, k);
    R w = v;
    if (NONOS) {
      const R cpm = cp.ld(i, j, km), cnm = cn.ld(i, j, km);
      w = STD ? vlim_std(v, min3(cpc, cnm), min3(cpm, cnc), X.ld(i, j, km), xc)
              : pp(v) * min3(cpc, cnm) - pn(v) * min3(cpm, cnc);
    }
    w3.at(i, j, k) = w;
    if (STD) f3.at(i, j, k) = donor(q.ld(i, j, km), qc, w);
  }
}

// ---- corrective update (std :431-459, gauge :364-368/396-400/423-427) -----
template <class R, bool STD>
__global__ void __launch_bounds__(128) k_update(Geo g, Arr<R> q, Arr<R> rhr, Arr<R> h, Arr<R> hinv,
                                                Arr<R> F1, Arr<R> F2, Arr<R> F3, Arr<R> out) {
  CELL_INDEX
  const R d = fx<R, false>(g, F1, i + 1, j, k) - fx<R, false>(g, F1, i, j, k) +
              fy<R, false>(g, F2, i, j + 1, k) - fy<R, false>(g, F2, i, j, k) +
              fz<R, false>(g, F3, i, j, k + 1) - fz<R, false>(g, F3, i, j, k);
  if (STD)
    out.at(i, j, k) = rhr.ld(i, j, k) * (q.ld(i, j, k) - d * hinv.ld(i, j, k));
  else
    out.at(i, j, k) = rhr.ld(i, j, k) * (q.ld(i, j, k) - d / h.ld(i, j, k));
}

// ---- host-side launch sequence -------------------------------------------
static unsigned long long g_launches = 0;
unsigned long long launch_count() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
void add_launches(int n) { __atomic_add_fetch(&g_launches, (unsigned long long)n, __ATOMIC_RELAXED); }
static inline void count(int n) { add_launches(n); }

// launch wrapper: optional event pair around the kernel, launch accounting
#define LAUNCH(stage, ...)                          \
  do {                                              \
    if (P.prof) P.prof->begin(stage, s);            \
    __VA_ARGS__;                                    \
    if (P.prof) P.prof->end(stage, s);              \
    count(1);                                       \
  } while (0)

template <class R>
int run_step(const StepPlan<R>& P, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 grd((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  const bool stdf = !P.gauge;
  if (P.iord >= 2)
    LAUNCH(ST_UPWIND, k_upwind<R, true><<<grd, blk, 0, s>>>(g, P.psi, P.u1, P.u2, P.u3, P.h, P.rhr, P.bcx, P.bcy, P.xant, P.hinv));
  else
    LAUNCH(ST_UPWIND, k_upwind<R, false><<<grd, blk, 0, s>>>(g, P.psi, P.u1, P.u2, P.u3, P.h, P.rhr, P.bcx, P.bcy, P.xant, P.hinv));
  if (P.iord < 2) {
    LAUNCH(ST_COPY, k_copy<R><<<grd, blk, 0, s>>>(g, P.xant, P.psi));
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
  }
  const bool keep = P.iord > 2;
  for (int pass = 2; pass <= P.iord; pass++) {
    const bool ain = (pass == 2);
    const Arr<R> A1 = ain ? P.u1 : P.w1, A2 = ain ? P.u2 : P.w2, A3 = ain ? P.u3 : P.w3;
    // fluxes for the bounds: std -> donor fluxes (stored in f*), gauge -> v itself
    if (stdf) {
      if (ain) LAUNCH(ST_PSEUDO, k_pseudo<R, true, true><<<grd, blk, 0, s>>>(g, P.xant, A1, A2, A3, P.h, P.v1, P.v2, P.v3, P.f1, P.f2, P.f3));
      else LAUNCH(ST_PSEUDO, k_pseudo<R, true, false><<<grd, blk, 0, s>>>(g, P.xant, A1, A2, A3, P.h, P.v1, P.v2, P.v3, P.f1, P.f2, P.f3));
    } else {
      if (ain) LAUNCH(ST_PSEUDO, k_pseudo<R, false, true><<<grd, blk, 0, s>>>(g, P.xant, A1, A2, A3, P.h, P.v1, P.v2, P.v3, P.f1, P.f2, P.f3));
      else LAUNCH(ST_PSEUDO, k_pseudo<R, false, false><<<grd, blk, 0, s>>>(g, P.xant, A1, A2, A3, P.h, P.v1, P.v2, P.v3, P.f1, P.f2, P.f3));
    }
    const Arr<R> F1 = stdf ? P.f1 : P.v1, F2 = stdf ? P.f2 : P.v2, F3 = stdf ? P.f3 : P.v3;
    if (!P.nonos)
      LAUNCH(ST_BOUNDS, k_bounds<R, false, true, false><<<grd, blk, 0, s>>>(g, P.xant, P.psi, P.mx, P.mn, P.h, P.rhr, F1, F2, F3, P.cp, P.cn, P.q));
    else if (ain && keep)
      LAUNCH(ST_BOUNDS, k_bounds<R, true, true, true><<<grd, blk, 0, s>>>(g, P.xant, P.psi, P.mx, P.mn, P.h, P.rhr, F1, F2, F3, P.cp, P.cn, P.q));
    else if (ain)
      LAUNCH(ST_BOUNDS, k_bounds<R, true, true, false><<<grd, blk, 0, s>>>(g, P.xant, P.psi, P.mx, P.mn, P.h, P.rhr, F1, F2, F3, P.cp, P.cn, P.q));
    else
      LAUNCH(ST_BOUNDS, k_bounds<R, true, false, true><<<grd, blk, 0, s>>>(g, P.xant, P.psi, P.mx, P.mn, P.h, P.rhr, F1, F2, F3, P.cp, P.cn, P.q));
    if (stdf) {
      if (P.nonos) LAUNCH(ST_LIMIT, k_limit<R, true, true><<<grd, blk, 0, s>>>(g, P.xant, P.v1, P.v2, P.v3, P.cp, P.cn, P.q, P.w1, P.w2, P.w3, P.f1, P.f2, P.f3));
      else LAUNCH(ST_LIMIT, k_limit<R, true, false><<<grd, blk, 0, s>>>(g, P.xant, P.v1, P.v2, P.v3, P.cp, P.cn, P.q, P.w1, P.w2, P.w3, P.f1, P.f2, P.f3));
    } else {
      if (P.nonos) LAUNCH(ST_LIMIT, k_limit<R, false, true><<<grd, blk, 0, s>>>(g, P.xant, P.v1, P.v2, P.v3, P.cp, P.cn, P.q, P.w1, P.w2, P.w3, P.f1, P.f2, P.f3));
      else LAUNCH(ST_LIMIT, k_limit<R, false, false><<<grd, blk, 0, s>>>(g, P.xant, P.v1, P.v2, P.v3, P.cp, P.cn, P.q, P.w1, P.w2, P.w3, P.f1, P.f2, P.f3));
    }
    // the update reads q (not x), so the pass result may overwrite xant in place
    const Arr<R> out = (pass == P.iord) ? P.psi : P.xant;
    if (stdf) LAUNCH(ST_UPDATE, k_update<R, true><<<grd, blk, 0, s>>>(g, P.q, P.rhr, P.h, P.hinv, P.f1, P.f2, P.f3, out));
    else LAUNCH(ST_UPDATE, k_update<R, false><<<grd, blk, 0, s>>>(g, P.q, P.rhr, P.h, P.hinv, P.w1, P.w2, P.w3, out));
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template int run_step<double>(const StepPlan<double>&, cudaStream_t);
template int run_step<float>(const StepPlan<float>&, cudaStream_t);

}  // namespace mpdata
