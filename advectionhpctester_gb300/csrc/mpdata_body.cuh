// Per-cell bodies of the MPDATA stage kernels.
//
// One problem (a field on a grid, with its velocity, densities and scratch)
// is described by Prob<R>; every stage body computes one cell (i,j,k) of one
// problem.  The single-problem kernels pass Prob by value; the batched
// kernels read it from a device table (many tracers sharing one velocity,
// many independent domains), so both paths run the same arithmetic.
//
// Boundary conditions are index maps applied when a neighbour is read:
//   psi halo     Dirichlet bcx/bcy (putbcinxh, mpdataoperators.inc:253-287) or wrap
//   xant halo    reflection x(0)=x(2) (cp_scnd_last_to_halo_xy_fulld, :479-513) or wrap
//   x_in halo    zero gradient x(0)=x(1) (cp_last_to_halo_xy, :551-584) or wrap
//   face fields  0 on open x/y walls (flux_x_bcd/flux_y_bcd type 0, :673-811),
//                mirrored on z walls (flux_z_bc_nohalod type 2, :903-947), or wrap
// Face fields store the faces 1..n of their own axis; face n+1 is face 1
// (periodic), zero (open wall) or minus face n (z wall).
#pragma once
#include "mpdata_common.cuh"

namespace mpdata {

template <class R>
struct Prob {
  Geo g;
  int stdf;     // 1 = standard form (t_adv=2), 0 = infinite gauge (t_adv=1)
  int own_vel;  // 1 = this problem writes the velocity-derived scratch (hinv, hm*)
  int rho;      // density step of mpdata3d_rho_gauge_gpubc: no rhr, upwind fluxes kept
  int pairs;    // gauge pseudo-velocity: 1 = pair sums of xant in cp, cn, q
                // (k_pairs); 2 = also the pass velocities' cell-centred pairs
                // in f1..f3, which lets full warps at a boundary take the pair path
  int gv;       // batch velocity group: the velocity-only terms of the first
                // pass's pseudo-velocities, stored by the group owner's upwind:
                // bit 0 the gauge form's (gvf), bit 1 the standard form's (gvs)
  Arr<R> psi, u1, u2, u3, h, rhr;
  const R* bcx;
  const R* bcy;
  Arr<R> hinv, hmx, hmy, hmz;  // may be shared by problems with one velocity
  Arr<R> gvf[12];               // per face direction d = x, y, z (index 4d): the two
                                // 4-face sums of the cross terms, (|a|-a*a*hm)/2 and
                                // 0.03125*a*hm (velocity group, shared)
  Arr<R> gvs[9];                // standard form, per face direction (index 3d):
                                // |a|-a*a*hm and (0.125*a)*b of the two cross terms
  Arr<R> xant, v1, v2, v3, f1, f2, f3, w1, w2, w3, cp, cn, mx, mn, q;
  // density step only: outputs and the upwind fluxes of the faces n+1
  Arr<R> x_incomp, rhoadv, rhr_out, pexe, pexr1, pexr2;
  R* f1hi;  // (mp,lp)
  R* f2hi;  // (np,lp)
  R* f3hi;  // (np,mp)
};

// ---- read helpers -------------------------------------------------------
// IN: the caller guarantees that every index is inside [1, n] and every face
// inside [2, n] (a cell in [2, n-1] on every axis reading its +-1
// neighbours), where every boundary map is the identity.
template <bool IN = false>
__device__ __forceinline__ int cx(const Geo& g, int i) { return IN ? i : (g.bx ? wrapi(i, g.np) : clampi(i, g.np)); }
template <bool IN = false>
__device__ __forceinline__ int cy(const Geo& g, int j) { return IN ? j : (g.by ? wrapi(j, g.mp) : clampi(j, g.mp)); }
template <bool IN = false>
__device__ __forceinline__ int cz(const Geo& g, int k) { return IN ? k : (g.bz ? wrapi(k, g.lp) : clampi(k, g.lp)); }

// the xant halo rule's x and y maps: a wrap, or the reflection of a wall
template <bool IN = false>
__device__ __forceinline__ int xmx(const Geo& g, int i) { return IN ? i : (g.bx ? wrapi(i, g.np) : refl(i, g.np)); }
template <bool IN = false>
__device__ __forceinline__ int xmy(const Geo& g, int j) { return IN ? j : (g.by ? wrapi(j, g.mp) : refl(j, g.mp)); }

// the current (antidiffused) field with the xant halo rule
template <class R, bool IN = false>
__device__ __forceinline__ R xr(const Geo& g, const Arr<R>& X, int i, int j, int k) {
  if (IN) return X.ld(i, j, k);
  return X.ld(xmx(g, i), xmy(g, j), cz(g, k));
}

// Face fields.  AIN = the caller's C-grid Courant numbers (faces 1..n+1 are
// data on open axes); otherwise an antidiffusive field with the wall rule.
template <class R, bool AIN, bool IN = false>
__device__ __forceinline__ R fx(const Geo& g, const Arr<R>& A, int f, int j, int k) {
  if (IN) return A.ld(f, j, k);
  j = cy(g, j);
  k = cz(g, k);
  if (g.bx) return A.ld(wrapi(f, g.np), j, k);
  if (AIN) return A.ld(f, j, k);
  return (f <= 1 || f > g.np) ? R(0) : A.ld(f, j, k);
}
template <class R, bool AIN, bool IN = false>
__device__ __forceinline__ R fy(const Geo& g, const Arr<R>& A, int i, int f, int k) {
  if (IN) return A.ld(i, f, k);
  i = cx(g, i);
  k = cz(g, k);
  if (g.by) return A.ld(i, wrapi(f, g.mp), k);
  if (AIN) return A.ld(i, f, k);
  return (f <= 1 || f > g.mp) ? R(0) : A.ld(i, f, k);
}
template <class R, bool AIN, bool IN = false>
__device__ __forceinline__ R fz(const Geo& g, const Arr<R>& A, int i, int j, int f) {
  if (IN) return A.ld(i, j, f);
  i = cx(g, i);
  j = cy(g, j);
  if (g.bz) return A.ld(i, j, wrapi(f, g.lp));
  if (AIN) return A.ld(i, j, f);
  if (f <= 1) return -A.ld(i, j, 2);
  if (f > g.lp) return -A.ld(i, j, g.lp);
  return A.ld(i, j, f);
}

// Warp-uniform choice of the interior path: true when every lane of the warp
// holds a cell in [2, n-1] on every axis, where the bodies' reads (all within
// +-1 of the cell) need no boundary map.  Every lane of a full warp calls it,
// before any lane returns.
__device__ __forceinline__ bool warp_interior(const Geo& g, int i, int j, int k) {
  const bool in = i >= 2 && i < g.np && j >= 2 && j < g.mp && k >= 2 && k < g.lp;
  return __all_sync(0xffffffffu, in);
}

// Warp-uniform: every lane holds a cell of the grid.  Such a warp may take
// the precomputed pair sums outside the interior too: it reads them through
// the same boundary maps as the values they sum (pairs_body fills the wrapped
// pairs of periodic axes; a wall needs no pair beyond [1, n]).  Every lane of
// a full warp calls it, before any lane returns.
__device__ __forceinline__ bool warp_on_grid(const Geo& g, int i, int j) {
  return __all_sync(0xffffffffu, i <= g.np && j <= g.mp);
}

// The standard form's pseudo-velocity pieces with their velocity-only
// factors precomputed (a batch velocity group, gvs): vdyfa with
// ka = |a|-a*a*hm, vcorra with bc = (0.125*a)*b.  Same operations, same order.
template <class R>
__device__ __forceinline__ R vdyfa_k(R x1, R x2, R ka, R ep) {
  return ka * (fabs(x2) - fabs(x1)) / (fabs(x2) + fabs(x1) + ep);
}
template <bool U, class R>
__device__ __forceinline__ R vcorra_b(R bc, R y1, R y2, R hm) {
  return -(hmul<U>(bc * y1, hm) / y2);
}

// True when hmx, hmy and hmz are exactly 1 at every cell of the warp (FP64
// only; FP32 kernels are bound by instruction issue and keep the products).
template <class R>
__device__ __forceinline__ bool warp_unit_faces(const Prob<R>& P, int i, int j, int k) {
  if constexpr (sizeof(R) == 8) {
    const bool u = is_one(P.hmx.ld(i, j, k)) && is_one(P.hmy.ld(i, j, k)) && is_one(P.hmz.ld(i, j, k));
    return __all_sync(0xffffffffu, u);
  } else {
    return false;
  }
}

// True when h (and rhr, outside the density step) is exactly 1 at every cell
// of the warp (FP64 only).  Bodies instantiated with U drop the products and
// quotients by these densities: exact, as x*1 == x/1 == x.
template <class R>
__device__ __forceinline__ bool warp_unit_cell(const Prob<R>& P, int i, int j, int k) {
  if constexpr (sizeof(R) == 8) {
    const bool u = is_one(P.h.ld(i, j, k)) && (P.rho || is_one(P.rhr.ld(i, j, k)));
    return __all_sync(0xffffffffu, u);
  } else {
    return false;
  }
}

// The 4-face velocity sums of the cross terms as two cell-centred pairs, the
// lower cell first: the oracle's fixed order for the reference's
// unparenthesised sums (antidiff3d-gauge-gpubc.f90:163-203).  The pair of
// cell c along the velocity's own axis is, for the y velocity, a2(c)+a2(c+y).
// The user defines the face accessors AX, AY, AZ and the cell (i, j, k).
#define VSUM_2X ((AY(i - 1, j, k) + AY(i - 1, j + 1, k)) + (AY(i, j, k) + AY(i, j + 1, k)))
#define VSUM_3X ((AZ(i - 1, j, k) + AZ(i - 1, j, k + 1)) + (AZ(i, j, k) + AZ(i, j, k + 1)))
#define VSUM_1Y ((AX(i, j - 1, k) + AX(i + 1, j - 1, k)) + (AX(i, j, k) + AX(i + 1, j, k)))
#define VSUM_3Y ((AZ(i, j - 1, k) + AZ(i, j - 1, k + 1)) + (AZ(i, j, k) + AZ(i, j, k + 1)))
#define VSUM_1Z ((AX(i, j, k - 1) + AX(i + 1, j, k - 1)) + (AX(i, j, k) + AX(i + 1, j, k)))
#define VSUM_2Z ((AY(i, j, k - 1) + AY(i, j + 1, k - 1)) + (AY(i, j, k) + AY(i, j + 1, k)))

// Velocity-only terms of the first corrective pass's gauge pseudo-velocities
// (pseudo_form with AIN), stored by a velocity group's owner for all of the
// group's fields: per face, the 4-face sums of the two cross terms in
// pseudo_form's order, (|a| - a*a*hm)*0.5 and 0.03125*a*hm.  The half is
// applied before the product with (x2-x1) instead of after it, which gives
// the same bits unless a value is subnormal (scaling by a power of two
// commutes with rounding).
template <class R, bool IN>
__device__ __forceinline__ void velgroup_body(const Prob<R>& P, int i, int j, int k, R hx, R hy, R hz) {
  const Geo& g = P.g;
#define AX(f, b, c) fx<R, true, IN>(g, P.u1, (f), (b), (c))
#define AY(a, f, c) fy<R, true, IN>(g, P.u2, (a), (f), (c))
#define AZ(a, b, f) fz<R, true, IN>(g, P.u3, (a), (b), (f))
  // the standard form's vdyfa factor |a|-a*a*hm and vcorra's (0.125*a)*b
  // keep their own operation order (no scaling is moved)
  const bool gg = P.gv & 1, gs = P.gv & 2;
  if (IN || g.bx || i > 1) {
    const R a = AX(i, j, k);
    const R b1 = VSUM_2X;
    const R b2 = VSUM_3X;
    const R ka = fabs(a) - a * a * hx;
    if (gg) {
      P.gvf[0].at(i, j, k) = b1;
      P.gvf[1].at(i, j, k) = b2;
      P.gvf[2].at(i, j, k) = scale_down<1>(ka);
      P.gvf[3].at(i, j, k) = scale_down<5>(a) * hx;
    }
    if (gs) {
      P.gvs[0].at(i, j, k) = ka;
      P.gvs[1].at(i, j, k) = scale_down<3>(a) * b1;
      P.gvs[2].at(i, j, k) = scale_down<3>(a) * b2;
    }
  }
  if (IN || g.by || j > 1) {
    const R a = AY(i, j, k);
    const R b1 = VSUM_1Y;
    const R b2 = VSUM_3Y;
    const R ka = fabs(a) - a * a * hy;
    if (gg) {
      P.gvf[4].at(i, j, k) = b1;
      P.gvf[5].at(i, j, k) = b2;
      P.gvf[6].at(i, j, k) = scale_down<1>(ka);
      P.gvf[7].at(i, j, k) = scale_down<5>(a) * hy;
    }
    if (gs) {
      P.gvs[3].at(i, j, k) = ka;
      P.gvs[4].at(i, j, k) = scale_down<3>(a) * b1;
      P.gvs[5].at(i, j, k) = scale_down<3>(a) * b2;
    }
  }
  if (IN || g.bz || k > 1) {
    const R a = AZ(i, j, k);
    const R b1 = VSUM_1Z;
    const R b2 = VSUM_2Z;
    const R ka = fabs(a) - a * a * hz;
    if (gg) {
      P.gvf[8].at(i, j, k) = b1;
      P.gvf[9].at(i, j, k) = b2;
      P.gvf[10].at(i, j, k) = scale_down<1>(ka);
      P.gvf[11].at(i, j, k) = scale_down<5>(a) * hz;
    }
    if (gs) {
      P.gvs[6].at(i, j, k) = ka;
      P.gvs[7].at(i, j, k) = scale_down<3>(a) * b1;
      P.gvs[8].at(i, j, k) = scale_down<3>(a) * b2;
    }
  }
#undef AX
#undef AY
#undef AZ
}

// ---- upwind3d_gpubc (upwind3d-gpubc.f90:101-198) -------------------------
// ANTIDIFF: an antidiffusive pass follows, so psi's open-wall halo ends the
// step holding the zero-gradient copy of the old boundary values (written by
// cp_last_to_halo_xy in the antidiffusion); otherwise it keeps bcx/bcy.
// HALO: write psi's halo at all (off while autotuning).
template <class R, bool ANTIDIFF, bool HALO, bool IN = false, bool U = false, bool DEFER = true>
__device__ __forceinline__ void upwind_body(const Prob<R>& P, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& psi = P.psi;
  const R x = psi.ld(i, j, k);
  const long bx0 = (long)(j - 1) + (long)g.mp * (k - 1), bxs = (long)g.mp * g.lp;
  const long by0 = (long)(i - 1) + (long)g.np * (k - 1), bys = (long)g.np * g.lp;
  const R xim = (IN || i > 1) ? psi.ld(i - 1, j, k) : (g.bx ? psi.ld(g.np, j, k) : P.bcx[bx0]);
  const R xip = (IN || i < g.np) ? psi.ld(i + 1, j, k) : (g.bx ? psi.ld(1, j, k) : P.bcx[bx0 + bxs]);
  const R xjm = (IN || j > 1) ? psi.ld(i, j - 1, k) : (g.by ? psi.ld(i, g.mp, k) : P.bcy[by0]);
  const R xjp = (IN || j < g.mp) ? psi.ld(i, j + 1, k) : (g.by ? psi.ld(i, 1, k) : P.bcy[by0 + bys]);
  const R hc = P.h.ld(i, j, k);
  const R hi = U ? R(1) : rcp1(hc);
  const R f1p = donor(x, xip, fx<R, true, IN>(g, P.u1, i + 1, j, k));
  const R f1 = donor(xim, x, P.u1.ld(i, j, k));
  const R f2p = donor(x, xjp, fy<R, true, IN>(g, P.u2, i, j + 1, k));
  const R f2 = donor(xjm, x, P.u2.ld(i, j, k));
  R f3p, f3;
  if (!IN && !g.bz && k == 1) {  // :134-135
    f3p = donor(x, psi.ld(i, j, k + 1), P.u3.ld(i, j, k + 1));
    f3 = -f3p;
  } else if (!IN && !g.bz && k == g.lp) {  // :164-165
    f3 = donor(psi.ld(i, j, k - 1), x, P.u3.ld(i, j, k));
    f3p = -f3;
  } else {
    f3p = donor(x, psi.ld(i, j, cz<IN>(g, k + 1)), fz<R, true, IN>(g, P.u3, i, j, k + 1));
    f3 = donor(psi.ld(i, j, cz<IN>(g, k - 1)), x, P.u3.ld(i, j, k));
  }
  // the loads of the face reciprocals' neighbour densities and of rhr come
  // before the first store (see limit_form)
  const bool hv = ANTIDIFF && P.own_vel;
  const bool fxe = IN || g.bx || i > 1, fye = IN || g.by || j > 1, fze = IN || g.bz || k > 1;
  R hxm = R(0), hym = R(0), hzm = R(0);
  if (DEFER) {
    hxm = hv && fxe ? P.h.ld(cx<IN>(g, i - 1), j, k) : R(0);
    hym = hv && fye ? P.h.ld(i, cy<IN>(g, j - 1), k) : R(0);
    hzm = hv && fze ? P.h.ld(i, j, cz<IN>(g, k - 1)) : R(0);
  }
  const R rh = (P.rho || U) ? R(1) : P.rhr.ld(i, j, k);
  if (P.rho) {
    // mpdata3d-rho-gauge-gpubc.f90:137-210: no rhr, division by h, fluxes kept;
    // rhoadv takes the input x_incomp (:121-123)
    const R sum = f1p - f1 + f2p - f2 + f3p - f3;
    P.xant.at(i, j, k) = x - (U ? sum : div1(sum, hc));
    P.f1.at(i, j, k) = f1;
    P.f2.at(i, j, k) = f2;
    P.f3.at(i, j, k) = f3;
    if (i == g.np) P.f1hi[(j - 1) + (long)g.mp * (k - 1)] = f1p;
    if (j == g.mp) P.f2hi[(i - 1) + (long)g.np * (k - 1)] = f2p;
    if (k == g.lp) P.f3hi[(i - 1) + (long)g.np * (j - 1)] = f3p;
    P.rhoadv.at(i, j, k) = P.x_incomp.ld(i, j, k);
  } else {
    const R sum = f1p - f1 + f2p - f2 + f3p - f3;
    P.xant.at(i, j, k) = U ? x - sum : (x - sum * hi) * rh;
  }
  if (hv) {
    if (!DEFER) {  // the batch kernels load these after the first store (fewer registers)
      hxm = fxe ? P.h.ld(cx<IN>(g, i - 1), j, k) : R(0);
      hym = fye ? P.h.ld(i, cy<IN>(g, j - 1), k) : R(0);
      hzm = fze ? P.h.ld(i, j, cz<IN>(g, k - 1)) : R(0);
    }
    P.hinv.at(i, j, k) = hi;
    // reciprocal mean densities of the cell's lower faces, used by every
    // corrective pass of this step (hmx/hmy/hmz of antidiff3d-*-gpubc.f90)
    R hx = R(0), hy = R(0), hz = R(0);
    if (fxe) P.hmx.at(i, j, k) = hx = rhm(hxm, hc);
    if (fye) P.hmy.at(i, j, k) = hy = rhm(hym, hc);
    if (fze) P.hmz.at(i, j, k) = hz = rhm(hzm, hc);
    if (P.gv) velgroup_body<R, IN>(P, i, j, k, hx, hy, hz);
  }
  if (HALO && !IN) {
    if (!g.bx) {
      if (i == 1) psi.at(0, j, k) = ANTIDIFF ? x : xim;
      if (i == g.np) psi.at(g.np + 1, j, k) = ANTIDIFF ? x : xip;
    }
    if (!g.by) {
      if (j == 1) psi.at(i, 0, k) = ANTIDIFF ? x : xjm;
      if (j == g.mp) psi.at(i, g.mp + 1, k) = ANTIDIFF ? x : xjp;
    }
  }
}

// ---- antidiffusive pseudo-velocities --------------------------------------
// standard form: antidiff3d-standard-gpubc.f90:72-203; gauge form:
// antidiff3d-gauge-gpubc.f90:89-203.  The k=1 and k=lp planes of a z wall
// drop the z cross terms of v1/v2, as the reference's boundary kernels do.
// Each cell computes its lower faces.  AIN: the first corrective pass, whose
// "a" velocities are the caller's Courant numbers; later passes use the
// previous pass's limited velocities w1..w3.  U: the three face reciprocal
// densities of every cell of the warp are exactly 1 (warp_unit_faces).  PS
// (gauge, interior warps): the pair sums of xant the rat4 terms start with
// are read from cp, cn and q, where k_pairs stored them.  GV (gauge, first
// pass, interior warps of a batch velocity group): the velocity-only terms
// are read from gvf (velgroup_body).  PV (gauge, with PS): the velocities'
// cell-centred pairs of the 4-face sums are read from f1..f3, where k_pairs
// stored them.  Without IN (a full warp at a boundary), PS reads the xant
// pairs through the xant halo maps and PV the velocity pairs through the
// face maps, so each stored pair is the sum the generic body forms there.
template <class R, bool STD, bool AIN, bool IN = false, bool U = false, bool PS = false, bool GV = false,
          bool DEFER = true, bool PV = false>
__device__ __forceinline__ void pseudo_form(const Prob<R>& P, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& X = P.xant;
  const Arr<R>& A1 = AIN ? P.u1 : P.w1;
  const Arr<R>& A2 = AIN ? P.u2 : P.w2;
  const Arr<R>& A3 = AIN ? P.u3 : P.w3;
  const R ep = Eps<R>::v;
  const bool zt = IN || g.bz || (k > 1 && k < g.lp);
#define XX(a, b, c) xr<R, IN>(g, X, (a), (b), (c))
#define AX(f, b, c) fx<R, AIN, IN>(g, A1, (f), (b), (c))
#define AY(a, f, c) fy<R, AIN, IN>(g, A2, (a), (f), (c))
#define AZ(a, b, f) fz<R, AIN, IN>(g, A3, (a), (b), (f))
#define MX(a) cx<IN>(g, (a))
#define MY(a) cy<IN>(g, (a))
#define MZ(a) cz<IN>(g, (a))
#define QX(a) xmx<IN>(g, (a))
#define QY(a) xmy<IN>(g, (a))
#define S2X (PV ? P.f2.ld(MX(i - 1), j, k) + P.f2.ld(i, j, k) : VSUM_2X)
#define S3X (PV ? P.f3.ld(MX(i - 1), j, k) + P.f3.ld(i, j, k) : VSUM_3X)
#define S1Y (PV ? P.f1.ld(i, MY(j - 1), k) + P.f1.ld(i, j, k) : VSUM_1Y)
#define S3Y (PV ? P.f3.ld(i, MY(j - 1), k) + P.f3.ld(i, j, k) : VSUM_3Y)
#define S1Z (PV ? P.f1.ld(i, j, MZ(k - 1)) + P.f1.ld(i, j, k) : VSUM_1Z)
#define S2Z (PV ? P.f2.ld(i, j, MZ(k - 1)) + P.f2.ld(i, j, k) : VSUM_2Z)
  // DEFER: results held until every load is issued (see limit_form); the
  // batch kernels, whose launch bound admits 256 threads, store each face at
  // once, which keeps their register count (and occupancy) lower
  R vo[3] = {R(0), R(0), R(0)}, fo[3] = {R(0), R(0), R(0)};
  Arr<R> const* const va[3] = {&P.v1, &P.v2, &P.v3};
  Arr<R> const* const fa[3] = {&P.f1, &P.f2, &P.f3};
  auto put = [&](int d, R v, R f) {
    if (DEFER) {
      vo[d] = v;
      fo[d] = f;
    } else {
      va[d]->at(i, j, k) = v;
      if (STD) fa[d]->at(i, j, k) = f;
    }
  };
  const bool fxe = IN || g.bx || i > 1, fye = IN || g.by || j > 1, fze = IN || g.bz || k > 1;
  if (fxe) {
    const R hmx = P.hmx.ld(i, j, k);
    const R a = AX(i, j, k);
    R v;
    if (STD) {
      const R y1 = (fabs(XX(i - 1, j + 1, k)) + fabs(XX(i, j + 1, k))) -
                   (fabs(XX(i - 1, j - 1, k)) + fabs(XX(i, j - 1, k)));
      const R y2 = fabs(XX(i - 1, j + 1, k)) + fabs(XX(i, j + 1, k)) + fabs(XX(i - 1, j - 1, k)) +
                   fabs(XX(i, j - 1, k)) + ep;
      if (GV)
        v = vdyfa_k(XX(i - 1, j, k), XX(i, j, k), P.gvs[0].ld(i, j, k), ep) +
            vcorra_b<U>(P.gvs[1].ld(i, j, k), y1, y2, hmx);
      else
        v = vdyfa_u<U>(XX(i - 1, j, k), XX(i, j, k), a, hmx, ep) +
            vcorra_u<U>(a, S2X, y1, y2, hmx);
      if (zt) {
        const R z1 = (fabs(XX(i - 1, j, k + 1)) + fabs(XX(i, j, k + 1))) -
                     (fabs(XX(i - 1, j, k - 1)) + fabs(XX(i, j, k - 1)));
        const R z2 = fabs(XX(i - 1, j, k + 1)) + fabs(XX(i, j, k + 1)) + fabs(XX(i - 1, j, k - 1)) +
                     fabs(XX(i, j, k - 1)) + ep;
        v = v + (GV ? vcorra_b<U>(P.gvs[2].ld(i, j, k), z1, z2, hmx)
                    : vcorra_u<U>(a, S3X, z1, z2,
                                  hmx));
      }
      put(0, v, donor(XX(i - 1, j, k), XX(i, j, k), v));
    } else {
      const R d2 = PS ? P.cp.ld(i, QY(j + 1), k) - P.cp.ld(i, QY(j - 1), k)
                      : dif4(XX(i - 1, j - 1, k), XX(i, j - 1, k), XX(i - 1, j + 1, k), XX(i, j + 1, k));
      const R c2 = (GV ? P.gvf[0].ld(i, j, k) : S2X) * d2;
      R cr = c2;
      if (zt) {
        const R d3 = PS ? P.cp.ld(i, j, MZ(k + 1)) - P.cp.ld(i, j, MZ(k - 1))
                        : dif4(XX(i - 1, j, k - 1), XX(i, j, k - 1), XX(i - 1, j, k + 1), XX(i, j, k + 1));
        cr = c2 + (GV ? P.gvf[1].ld(i, j, k) : S3X) * d3;
      }
      if (GV)
        v = P.gvf[2].ld(i, j, k) * (XX(i, j, k) - XX(i - 1, j, k)) - P.gvf[3].ld(i, j, k) * cr;
      else
        v = vdyf_u<U>(XX(i - 1, j, k), XX(i, j, k), a, hmx) - hmul<U>(scale_down<5>(a), hmx) * cr;
    }
    if (!STD) put(0, v, R(0));
  }
  if (fye) {
    const R hmy = P.hmy.ld(i, j, k);
    const R a = AY(i, j, k);
    R v;
    if (STD) {
      const R y1 = (fabs(XX(i + 1, j - 1, k)) + fabs(XX(i + 1, j, k))) -
                   (fabs(XX(i - 1, j - 1, k)) + fabs(XX(i - 1, j, k)));
      const R y2 = fabs(XX(i + 1, j - 1, k)) + fabs(XX(i + 1, j, k)) + fabs(XX(i - 1, j - 1, k)) +
                   fabs(XX(i - 1, j, k)) + ep;
      if (GV)
        v = vdyfa_k(XX(i, j - 1, k), XX(i, j, k), P.gvs[3].ld(i, j, k), ep) +
            vcorra_b<U>(P.gvs[4].ld(i, j, k), y1, y2, hmy);
      else
        v = vdyfa_u<U>(XX(i, j - 1, k), XX(i, j, k), a, hmy, ep) +
            vcorra_u<U>(a, S1Y, y1, y2, hmy);
      if (zt) {
        const R z1 = (fabs(XX(i, j - 1, k + 1)) + fabs(XX(i, j, k + 1))) -
                     (fabs(XX(i, j - 1, k - 1)) + fabs(XX(i, j, k - 1)));
        const R z2 = fabs(XX(i, j - 1, k + 1)) + fabs(XX(i, j, k + 1)) + fabs(XX(i, j - 1, k - 1)) +
                     fabs(XX(i, j, k - 1)) + ep;
        v = v + (GV ? vcorra_b<U>(P.gvs[5].ld(i, j, k), z1, z2, hmy)
                    : vcorra_u<U>(a, S3Y, z1, z2,
                                  hmy));
      }
      put(1, v, donor(XX(i, j - 1, k), XX(i, j, k), v));
    } else {
      const R d1 = PS ? P.cn.ld(QX(i + 1), j, k) - P.cn.ld(QX(i - 1), j, k)
                      : dif4(XX(i - 1, j - 1, k), XX(i - 1, j, k), XX(i + 1, j - 1, k), XX(i + 1, j, k));
      const R c1 = (GV ? P.gvf[4].ld(i, j, k) : S1Y) * d1;
      R cr = c1;
      if (zt) {
        const R d3 = PS ? P.cn.ld(i, j, MZ(k + 1)) - P.cn.ld(i, j, MZ(k - 1))
                        : dif4(XX(i, j - 1, k - 1), XX(i, j, k - 1), XX(i, j - 1, k + 1), XX(i, j, k + 1));
        cr = c1 + (GV ? P.gvf[5].ld(i, j, k) : S3Y) * d3;
      }
      if (GV)
        v = P.gvf[6].ld(i, j, k) * (XX(i, j, k) - XX(i, j - 1, k)) - P.gvf[7].ld(i, j, k) * cr;
      else
        v = vdyf_u<U>(XX(i, j - 1, k), XX(i, j, k), a, hmy) - hmul<U>(scale_down<5>(a), hmy) * cr;
    }
    if (!STD) put(1, v, R(0));
  }
  if (fze) {
    const R hmz = P.hmz.ld(i, j, k);
    const R a = AZ(i, j, k);
    R v;
    if (STD) {
      const R x1 = (fabs(XX(i + 1, j, k - 1)) + fabs(XX(i + 1, j, k))) -
                   (fabs(XX(i - 1, j, k - 1)) + fabs(XX(i - 1, j, k)));
      const R x2 = fabs(XX(i + 1, j, k - 1)) + fabs(XX(i + 1, j, k)) + fabs(XX(i - 1, j, k - 1)) +
                   fabs(XX(i - 1, j, k)) + ep;
      const R y1 = (fabs(XX(i, j + 1, k - 1)) + fabs(XX(i, j + 1, k))) -
                   (fabs(XX(i, j - 1, k - 1)) + fabs(XX(i, j - 1, k)));
      const R y2 = fabs(XX(i, j + 1, k - 1)) + fabs(XX(i, j + 1, k)) + fabs(XX(i, j - 1, k - 1)) +
                   fabs(XX(i, j - 1, k)) + ep;
      if (GV)
        v = vdyfa_k(XX(i, j, k - 1), XX(i, j, k), P.gvs[6].ld(i, j, k), ep) +
            vcorra_b<U>(P.gvs[7].ld(i, j, k), x1, x2, hmz) + vcorra_b<U>(P.gvs[8].ld(i, j, k), y1, y2, hmz);
      else
        v = vdyfa_u<U>(XX(i, j, k - 1), XX(i, j, k), a, hmz, ep) +
            vcorra_u<U>(a, S1Z, x1, x2, hmz) +
            vcorra_u<U>(a, S2Z, y1, y2, hmz);
      put(2, v, donor(XX(i, j, k - 1), XX(i, j, k), v));
    } else {
      const R d1 = PS ? P.q.ld(QX(i + 1), j, k) - P.q.ld(QX(i - 1), j, k)
                      : dif4(XX(i - 1, j, k - 1), XX(i - 1, j, k), XX(i + 1, j, k - 1), XX(i + 1, j, k));
      const R d2 = PS ? P.q.ld(i, QY(j + 1), k) - P.q.ld(i, QY(j - 1), k)
                      : dif4(XX(i, j - 1, k - 1), XX(i, j - 1, k), XX(i, j + 1, k - 1), XX(i, j + 1, k));
      const R cr = (GV ? P.gvf[8].ld(i, j, k) : S1Z) * d1 +
                   (GV ? P.gvf[9].ld(i, j, k) : S2Z) * d2;
      if (GV)
        v = P.gvf[10].ld(i, j, k) * (XX(i, j, k) - XX(i, j, k - 1)) - P.gvf[11].ld(i, j, k) * cr;
      else
        v = vdyf_u<U>(XX(i, j, k - 1), XX(i, j, k), a, hmz) - hmul<U>(scale_down<5>(a), hmz) * cr;
    }
    if (!STD) put(2, v, R(0));
  }
  if (DEFER) {
    if (fxe) {
      P.v1.at(i, j, k) = vo[0];
      if (STD) P.f1.at(i, j, k) = fo[0];
    }
    if (fye) {
      P.v2.at(i, j, k) = vo[1];
      if (STD) P.f2.at(i, j, k) = fo[1];
    }
    if (fze) {
      P.v3.at(i, j, k) = vo[2];
      if (STD) P.f3.at(i, j, k) = fo[2];
    }
  }
#undef MX
#undef MY
#undef MZ
#undef QX
#undef QY
#undef S2X
#undef S3X
#undef S1Y
#undef S3Y
#undef S1Z
#undef S2Z
#undef XX
#undef AX
#undef AY
#undef AZ
}

template <class R, bool AIN, bool IN = false, bool U = false, bool PS = false, bool GV = false, bool DEFER = true,
          bool PV = false>
__device__ __forceinline__ void pseudo_body(const Prob<R>& P, int i, int j, int k) {
  if (P.stdf)
    pseudo_form<R, true, AIN, IN, U, false, GV, DEFER>(P, i, j, k);
  else
    pseudo_form<R, false, AIN, IN, U, PS, GV, DEFER, PV>(P, i, j, k);
}

// ---- limiter bounds and ratios (std :256-348, gauge :238-324) -------------
// FIRST folds the star of the step's input field x_in (zero-gradient halo)
// into the bounds, as every first corrective pass does; later passes start
// from the stored running extrema (KEEP stores them).  The gauge k=1 minimum
// over x_in, which the reference leaves unset (antidiff3d-gauge-gpubc.f90:249),
// is computed as in mpdata3d-rho-gauge-gpubc.f90:365-368.  Also stores
// q = x/rhr, the ratio every later stage divides out.  cp and cn are read
// only through min3 by the forward limiter, so a ratio >= 1 may be stored as 1.
// CLM 0: exact quotients (the adjoint's records); 1: lim_ratio per cell;
// 2: nothing stored, the four operands returned for the caller to divide.
template <class R>
struct RatioOps {
  R np, dp, nn, dn;
};
// The limiter's star extrema folded with the reference's compare-and-select
// in its tree order, whose ties between +0 and -0 keep the earlier operand
// (bounds_body: FP32 always, FP64 where its key-order extrema may differ).
template <class R>
struct MaMi {
  R ma, mi;
};
template <class R, bool FIRST, bool IN>
__device__ __forceinline__ MaMi<R> tree_extrema(const Geo& g, const Arr<R>& xin, const Arr<R>& X,
                                                const Arr<R>& mxa, const Arr<R>& mna, int i, int j, int k, R x,
                                                bool lo, bool hi) {
  R ma, mi;
  if (FIRST) {
    const int im = cx<IN>(g, i - 1), ip = cx<IN>(g, i + 1);
    const int jm = cy<IN>(g, j - 1), jp = cy<IN>(g, j + 1);
    const R a0 = xin.ld(im, j, k), a1 = xin.ld(i, j, k), a2 = xin.ld(ip, j, k), a3 = xin.ld(i, jm, k),
            a4 = xin.ld(i, jp, k);
    ma = mx2(mx2(mx2(a0, a1), mx2(a2, a3)), a4);
    mi = mn2(mn2(mn2(a0, a1), mn2(a2, a3)), a4);
    if (lo) {
      const R a5 = xin.ld(i, j, cz<IN>(g, k - 1));
      ma = mx2(ma, a5);
      mi = mn2(mi, a5);
    }
    if (hi) {
      const R a6 = xin.ld(i, j, cz<IN>(g, k + 1));
      ma = mx2(ma, a6);
      mi = mn2(mi, a6);
    }
  } else {
    ma = mxa.ld(i, j, k);
    mi = mna.ld(i, j, k);
  }
  const R b0 = xr<R, IN>(g, X, i - 1, j, k), b2 = xr<R, IN>(g, X, i + 1, j, k),
          b3 = xr<R, IN>(g, X, i, j - 1, k), b4 = xr<R, IN>(g, X, i, j + 1, k);
  ma = mx2(mx2(mx2(ma, b0), mx2(x, b2)), mx2(b3, b4));
  mi = mn2(mn2(mn2(mi, b0), mn2(x, b2)), mn2(b3, b4));
  if (lo) {
    const R b5 = X.ld(i, j, cz<IN>(g, k - 1));
    ma = mx2(ma, b5);
    mi = mn2(mi, b5);
  }
  if (hi) {
    const R b6 = X.ld(i, j, cz<IN>(g, k + 1));
    ma = mx2(ma, b6);
    mi = mn2(mi, b6);
  }
  return MaMi<R>{ma, mi};
}
// The same behind a call: the FP64 kernels branch around it.
template <class R, bool FIRST, bool IN>
static __device__ __noinline__ MaMi<R> tree_extrema_call(Geo g, Arr<R> xin, Arr<R> X, Arr<R> mxa, Arr<R> mna,
                                                         int i, int j, int k, R x, bool lo, bool hi) {
  return tree_extrema<R, FIRST, IN>(g, xin, X, mxa, mna, i, j, k, x, lo, hi);
}
template <class R, bool NONOS, bool FIRST, bool KEEP, bool IN = false, int CLM = 0, bool U = false,
          bool DEFER = true>
__device__ __forceinline__ RatioOps<R> bounds_body(const Prob<R>& P, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& X = P.xant;
  const R x = X.ld(i, j, k);
  const R qv = (P.rho || U) ? x : div1(x, P.rhr.ld(i, j, k));  // x/1 == x for the density step
  if (!NONOS || !DEFER) P.q.at(i, j, k) = qv;
  if (!NONOS) return {};
  const bool lo = IN || g.bz || k > 1, hi = IN || g.bz || k < g.lp;
  R ma, mi;
  if constexpr (sizeof(R) == 4) {
    const MaMi<R> t = tree_extrema<R, FIRST, IN>(g, P.psi, X, P.mx, P.mn, i, j, k, x, lo, hi);
    ma = t.ma;
    mi = t.mi;
  } else {
    // FP64: key order on the integer pipe, then the tree where an extremum
    // may be a zero or a NaN, the only cases in which the two can differ
    if (FIRST) {
      const Arr<R>& xin = P.psi;
      const int im = cx<IN>(g, i - 1), ip = cx<IN>(g, i + 1);
      const int jm = cy<IN>(g, j - 1), jp = cy<IN>(g, j + 1);
      Extrema<R> e(xin.ld(i, j, k));
      e.add(xin.ld(im, j, k));
      e.add(xin.ld(ip, j, k));
      e.add(xin.ld(i, jm, k));
      e.add(xin.ld(i, jp, k));
      if (lo) e.add(xin.ld(i, j, cz<IN>(g, k - 1)));
      if (hi) e.add(xin.ld(i, j, cz<IN>(g, k + 1)));
      e.add(x);
      e.add(xr<R, IN>(g, X, i - 1, j, k));
      e.add(xr<R, IN>(g, X, i + 1, j, k));
      e.add(xr<R, IN>(g, X, i, j - 1, k));
      e.add(xr<R, IN>(g, X, i, j + 1, k));
      if (lo) e.add(X.ld(i, j, cz<IN>(g, k - 1)));
      if (hi) e.add(X.ld(i, j, cz<IN>(g, k + 1)));
      ma = e.max();
      mi = e.min();
    } else {
      Extrema<R> e(x);
      e.add(xr<R, IN>(g, X, i - 1, j, k));
      e.add(xr<R, IN>(g, X, i + 1, j, k));
      e.add(xr<R, IN>(g, X, i, j - 1, k));
      e.add(xr<R, IN>(g, X, i, j + 1, k));
      if (lo) e.add(X.ld(i, j, cz<IN>(g, k - 1)));
      if (hi) e.add(X.ld(i, j, cz<IN>(g, k + 1)));
      ma = mx2k(P.mx.ld(i, j, k), e.max());
      mi = mn2k(P.mn.ld(i, j, k), e.min());
    }
    if (zero_nan_hi(ma) || zero_nan_hi(mi)) {
      const MaMi<R> t = tree_extrema_call<R, FIRST, IN>(g, P.psi, X, P.mx, P.mn, i, j, k, x, lo, hi);
      ma = t.ma;
      mi = t.mi;
    }
  }
  if (KEEP && !DEFER) {
    P.mx.at(i, j, k) = ma;
    P.mn.at(i, j, k) = mi;
  }
  // fluxes for the bounds: std -> donor fluxes f*ns, gauge -> v itself
  const Arr<R>& F1 = P.stdf ? P.f1 : P.v1;
  const Arr<R>& F2 = P.stdf ? P.f2 : P.v2;
  const Arr<R>& F3 = P.stdf ? P.f3 : P.v3;
  const R ep = Eps<R>::v;
  const R e1 = fx<R, false, IN>(g, F1, i + 1, j, k), w1 = fx<R, false, IN>(g, F1, i, j, k);
  const R e2 = fy<R, false, IN>(g, F2, i, j + 1, k), w2 = fy<R, false, IN>(g, F2, i, j, k);
  const R e3 = fz<R, false, IN>(g, F3, i, j, k + 1), w3 = fz<R, false, IN>(g, F3, i, j, k);
  const R hc = U ? R(1) : P.h.ld(i, j, k);
  // DEFER: the stores follow every load (see limit_form); the batch kernels
  // store early, which keeps their register count lower
  if (DEFER) {
    P.q.at(i, j, k) = qv;
    if (KEEP) {
      P.mx.at(i, j, k) = ma;
      P.mn.at(i, j, k) = mi;
    }
  }
  const R np_ = U ? ma - x : (ma - x) * hc, nn = U ? x - mi : (x - mi) * hc;
  R dp, dn;
  if constexpr (sizeof(R) == 8) {
    // dp = pn(e1)+pp(w1)+pn(e2)+pp(w2)+pn(e3)+pp(w3)+ep and dn, its mirror,
    // left to right.  Each flux f is nonzero in at most one of the two sums,
    // as |f|, and adding +0 to a sum of non-negative terms changes no bit, so
    // each |f| is added to its own sum only, in the same order: 6 FP64 adds
    // instead of 12.
    dp = R(0);
    dn = R(0);
    const R f[6] = {e1, w1, e2, w2, e3, w3};
#pragma unroll
    for (int t = 0; t < 6; t++) {
      const bool to_p = (t & 1) ? !sgn(f[t]) : sgn(f[t]);  // e: pn into dp; w: pp into dp
      const R a = (to_p ? dp : dn) + fabs(f[t]);
      dp = to_p ? a : dp;
      dn = to_p ? dn : a;
    }
    dp = dp + ep;
    dn = dn + ep;
  } else {
    dp = pn(e1) + pp(w1) + pn(e2) + pp(w2) + pn(e3) + pp(w3) + ep;
    dn = pp(e1) + pn(w1) + pp(e2) + pn(w2) + pp(e3) + pn(w3) + ep;
  }
  if (CLM == 2) return {np_, dp, nn, dn};
  P.cp.at(i, j, k) = CLM ? lim_ratio(np_, dp) : np_ / dp;
  P.cn.at(i, j, k) = CLM ? lim_ratio(nn, dn) : nn / dn;
  return {};
}

// The FP64 limiter ratios of a block (whole warps, at most 256 threads),
// divided together.  Only the ratios below 1 need a quotient (a larger one
// is stored as RATIO_CAP, see lim_ratio), and they are a few percent of the
// cells, scattered: a
// warp dividing its own would run the division sequence (about ten FP64-pipe
// instructions) whenever any of its lanes needs one.  Here the block packs its
// operand pairs into shared memory, the first warps divide them, 32 at a time,
// and every cell stores its two ratios.  Every thread of the block, inside
// the domain or not, reaches the barriers.
template <class R>
__device__ __forceinline__ void block_ratios(const Prob<R>& P, int i, int j, int k, bool valid,
                                             const RatioOps<R>& r) {
  __shared__ int s_cnt[8];
  __shared__ R s_n[512], s_d[512];
  const int nt = blockDim.x * blockDim.y, tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, w = tid >> 5, nw = nt >> 5;
  const bool dp = valid && !ratio_ge1(r.np, r.dp), dn = valid && !ratio_ge1(r.nn, r.dn);
  const unsigned bp = __ballot_sync(0xffffffffu, dp), bn = __ballot_sync(0xffffffffu, dn);
  if (lane == 0) s_cnt[w] = __popc(bp) + __popc(bn);
  __syncthreads();
  int off = 0, total = 0;
  for (int v = 0; v < nw; v++) {
    const int c = s_cnt[v];
    off += v < w ? c : 0;
    total += c;
  }
  const unsigned lt = (1u << lane) - 1u;
  const int ip = off + __popc(bp & lt), in = off + __popc(bp) + __popc(bn & lt);
  if (dp) {
    s_n[ip] = r.np;
    s_d[ip] = r.dp;
  }
  if (dn) {
    s_n[in] = r.nn;
    s_d[in] = r.dn;
  }
  __syncthreads();
  // a zero numerator is its own quotient: on a zero background whole warps
  // of the packed list skip the division
  for (int it = tid; it < total; it += nt) {
    const R n = s_n[it], d = s_d[it];
    if (!ratio_zero(n, d)) s_n[it] = n / d;
  }
  __syncthreads();
  if (valid) {
    P.cp.at(i, j, k) = dp ? s_n[ip] : R(RATIO_CAP);
    P.cn.at(i, j, k) = dn ? s_n[in] : R(RATIO_CAP);
  }
}

// Pair sums of xant for the gauge pseudo-velocities of interior warps, which
// read each of them from four faces: Sx = x(i)+x(i-1) into cp, Sy =
// x(j)+x(j-1) into cn, Sz = x(k)+x(k-1) into q.  The operand order is that of
// the rat4 sums (antidiff3d-gauge-gpubc.f90:89-203), so every difference of
// two of them is the value rat4's own sums give.  cp, cn and q are free
// until the limiter bounds stage rewrites them.  A periodic axis also gets
// the wrapped pair of its first cell (x(1)+x(n)).  PV: also the pass
// velocities' cell-centred pairs of the 4-face sums (VSUM_*), a1(i)+a1(i+1)
// into f1, a2(j)+a2(j+1) into f2, a3(k)+a3(k+1) into f3, which the gauge form
// leaves unused outside the density step.  The face reads take the boundary
// rules, so the pairs interior warps read are the sums their faces give.
template <class R, bool AIN = true, bool PV = false>
__device__ __forceinline__ void pairs_body(const Prob<R>& P, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& X = P.xant;
  const R x = X.ld(i, j, k);
  R a1 = R(0), a2 = R(0), a3 = R(0);
  if (PV) {
    const Arr<R>& A1 = AIN ? P.u1 : P.w1;
    const Arr<R>& A2 = AIN ? P.u2 : P.w2;
    const Arr<R>& A3 = AIN ? P.u3 : P.w3;
    a1 = fx<R, AIN>(g, A1, i, j, k) + fx<R, AIN>(g, A1, i + 1, j, k);
    a2 = fy<R, AIN>(g, A2, i, j, k) + fy<R, AIN>(g, A2, i, j + 1, k);
    a3 = fz<R, AIN>(g, A3, i, j, k) + fz<R, AIN>(g, A3, i, j, k + 1);
  }
  if (i > 1 || g.bx) P.cp.at(i, j, k) = x + X.ld(i > 1 ? i - 1 : g.np, j, k);
  if (j > 1 || g.by) P.cn.at(i, j, k) = x + X.ld(i, j > 1 ? j - 1 : g.mp, k);
  if (k > 1 || g.bz) P.q.at(i, j, k) = x + X.ld(i, j, k > 1 ? k - 1 : g.lp);
  if (PV) {
    P.f1.at(i, j, k) = a1;
    P.f2.at(i, j, k) = a2;
    P.f3.at(i, j, k) = a3;
  }
}

// ---- limited antidiffusive velocities and fluxes --------------------------
// std: antidiff3d-standard-gpubc.f90:372-407 (sign-aware limited velocity,
// donor flux of x/rhr); gauge: antidiff3d-gauge-gpubc.f90:343-363 (the
// limited velocity is the flux).  Lower faces of each cell.
// The reference's factors a1*possign(xl) + a2*possign(-xl) and
// a2*possign(xrr) + a1*possign(-xrr) multiply by 1 and 0.  a1 and a2 are min3
// values of non-negative ratios (never -0), so each factor is exactly a1 + +0
// or +0 + a2, that is one of a1, a2 chosen by a sign bit.
template <class R>
__device__ __forceinline__ R vlim_std(R v, R a1, R a2, R xl, R xrr) {
  return donor(sgn(xl) ? a2 : a1, sgn(xrr) ? a1 : a2, v);
}

template <class R, bool STD, bool NONOS, bool IN = false, bool DEFER = true>
__device__ __forceinline__ void limit_form(const Prob<R>& P, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& X = P.xant;
  // every load before the first store: the arrays may alias as far as the
  // compiler knows, and a store would otherwise fence the next face's loads
  const R cpc = NONOS ? P.cp.ld(i, j, k) : R(0), cnc = NONOS ? P.cn.ld(i, j, k) : R(0);
  const R xc = X.ld(i, j, k), qc = STD ? P.q.ld(i, j, k) : R(0);
  const bool fx_ = IN || g.bx || i > 1, fy_ = IN || g.by || j > 1, fz_ = IN || g.bz || k > 1;
  const int im = IN ? i - 1 : wrapi(i - 1, g.np), jm = IN ? j - 1 : wrapi(j - 1, g.mp),
            km = IN ? k - 1 : wrapi(k - 1, g.lp);
  R w[3] = {R(0), R(0), R(0)}, f[3] = {R(0), R(0), R(0)};
#define LIMIT_FACE(d, V, WA, FA, I, J, K)                                              \
  {                                                                                    \
    const R v = V.ld(i, j, k);                                                         \
    R ww = v;                                                                          \
    if (NONOS) {                                                                       \
      const R cpm = P.cp.ld(I, J, K), cnm = P.cn.ld(I, J, K);                          \
      ww = STD ? vlim_std(v, min3(cpc, cnm), min3(cpm, cnc), X.ld(I, J, K), xc)         \
               : donor(min3(cpc, cnm), min3(cpm, cnc), v);                             \
    }                                                                                  \
    w[d] = ww;                                                                         \
    if (STD) f[d] = donor(P.q.ld(I, J, K), qc, ww);                                    \
    if (!DEFER) {                                                                      \
      WA.at(i, j, k) = ww;                                                             \
      if (STD) FA.at(i, j, k) = f[d];                                                  \
    }                                                                                  \
  }
  if (fx_) LIMIT_FACE(0, P.v1, P.w1, P.f1, im, j, k)
  if (fy_) LIMIT_FACE(1, P.v2, P.w2, P.f2, i, jm, k)
  if (fz_) LIMIT_FACE(2, P.v3, P.w3, P.f3, i, j, km)
#undef LIMIT_FACE
  if (!DEFER) return;
  if (fx_) {
    P.w1.at(i, j, k) = w[0];
    if (STD) P.f1.at(i, j, k) = f[0];
  }
  if (fy_) {
    P.w2.at(i, j, k) = w[1];
    if (STD) P.f2.at(i, j, k) = f[1];
  }
  if (fz_) {
    P.w3.at(i, j, k) = w[2];
    if (STD) P.f3.at(i, j, k) = f[2];
  }
}

template <class R, bool NONOS, bool IN = false, bool DEFER = true>
__device__ __forceinline__ void limit_body(const Prob<R>& P, int i, int j, int k) {
  if (P.stdf)
    limit_form<R, true, NONOS, IN, DEFER>(P, i, j, k);
  else
    limit_form<R, false, NONOS, IN, DEFER>(P, i, j, k);
}

// ---- corrective update (std :431-459, gauge :364-368/396-400/423-427) -----
// LAST: the last pass writes psi; earlier passes overwrite xant in place (the
// update reads q, not x).
template <class R, bool LAST, bool IN = false, bool U = false>
__device__ __forceinline__ void update_body(const Prob<R>& P, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& out = LAST ? P.psi : P.xant;
  if (P.stdf) {
    const R d = fx<R, false, IN>(g, P.f1, i + 1, j, k) - fx<R, false, IN>(g, P.f1, i, j, k) +
                fy<R, false, IN>(g, P.f2, i, j + 1, k) - fy<R, false, IN>(g, P.f2, i, j, k) +
                fz<R, false, IN>(g, P.f3, i, j, k + 1) - fz<R, false, IN>(g, P.f3, i, j, k);
    out.at(i, j, k) = U ? P.q.ld(i, j, k) - d : (P.q.ld(i, j, k) - d * P.hinv.ld(i, j, k)) * P.rhr.ld(i, j, k);
  } else {
    const R d = fx<R, false, IN>(g, P.w1, i + 1, j, k) - fx<R, false, IN>(g, P.w1, i, j, k) +
                fy<R, false, IN>(g, P.w2, i, j + 1, k) - fy<R, false, IN>(g, P.w2, i, j, k) +
                fz<R, false, IN>(g, P.w3, i, j, k + 1) - fz<R, false, IN>(g, P.w3, i, j, k);
    const R t = P.q.ld(i, j, k) - (U ? d : div1(d, P.h.ld(i, j, k)));
    out.at(i, j, k) = (P.rho || U) ? t : t * P.rhr.ld(i, j, k);  // rhr == 1 in the density step
  }
}

// ---- outputs of the density step (mpdata3d-rho-gauge-gpubc.f90:486-606) ----
// x_incomp = x*h, pexr1 = x_incomp*pexe, pexr2 = x_incomp, rhr = rhoadv/x_incomp,
// and the mass fluxes u = upwind flux + limited antidiffusive flux on the
// cell's lower faces (and the faces n+1 on the last cells).  LINER: the
// upwind-only branch (:594-606), where psi still has to take xant.
template <class R, bool LINER>
__device__ __forceinline__ void rho_out_body(const Prob<R>& P, int i, int j, int k) {
  const Geo& g = P.g;
  if (LINER) P.psi.at(i, j, k) = P.xant.ld(i, j, k);
  const R xv = LINER ? P.xant.ld(i, j, k) : P.psi.ld(i, j, k);
  const R xc = xv * P.h.ld(i, j, k);
  P.x_incomp.at(i, j, k) = xc;
  P.pexr1.at(i, j, k) = xc * P.pexe.ld(i, j, k);
  P.pexr2.at(i, j, k) = xc;
  P.rhr_out.at(i, j, k) = P.rhoadv.ld(i, j, k) / xc;
  P.u1.at(i, j, k) = P.f1.ld(i, j, k) + (LINER ? R(0) : fx<R, false>(g, P.w1, i, j, k));
  P.u2.at(i, j, k) = P.f2.ld(i, j, k) + (LINER ? R(0) : fy<R, false>(g, P.w2, i, j, k));
  P.u3.at(i, j, k) = P.f3.ld(i, j, k) + (LINER ? R(0) : fz<R, false>(g, P.w3, i, j, k));
  if (i == g.np)
    P.u1.at(g.np + 1, j, k) = P.f1hi[(j - 1) + (long)g.mp * (k - 1)] + (LINER ? R(0) : fx<R, false>(g, P.w1, g.np + 1, j, k));
  if (j == g.mp)
    P.u2.at(i, g.mp + 1, k) = P.f2hi[(i - 1) + (long)g.np * (k - 1)] + (LINER ? R(0) : fy<R, false>(g, P.w2, i, g.mp + 1, k));
  if (k == g.lp)
    P.u3.at(i, j, g.lp + 1) = P.f3hi[(i - 1) + (long)g.np * (j - 1)] + (LINER ? R(0) : fz<R, false>(g, P.w3, i, j, g.lp + 1));
}

template <class R>
__device__ __forceinline__ void copy_body(const Prob<R>& P, int i, int j, int k) {
  P.psi.at(i, j, k) = P.xant.ld(i, j, k);
}

}  // namespace mpdata
