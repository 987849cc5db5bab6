// Adjoint of the MPDATA step (infinite-gauge and standard forms, iord >= 2
// corrective passes, nonoscillatory limiter on or off).  No reference code exists for
// it; it differentiates the forward step of mpdata_body.cuh exactly, with
// every branch (pp, pn, min3, the limiter's max/min over the 7-point stars
// and over the running extrema of earlier passes, abs) taken at the forward
// values ("piecewise at the forward branch").
//
// Given psi at the start of a step, the velocities and lambda = dJ/dpsi_new,
// the step adjoint first records the forward step pass by pass (upwind field,
// face reciprocals; per pass its input field, pseudo-velocities, limiter
// ratios, limited velocities and running extrema), then runs one reverse
// kernel per forward stage, last pass first:
//   update    x_out = rhr*(q - div(w)/h)           -> lambda_x, lambda_w
//             (standard: rhr*(q - div(g)*hinv), g the limited donor fluxes of q)
//   limiter   w = pp(v)*A1 - pn(v)*A2              -> lambda_v, lambda_cp, lambda_cn
//             (standard: the sign-aware vlim_std and g = donor(q, w))
//   bounds    cp,cn from the extrema and v         -> lambda_x, lambda_v, and lambda of
//                                                     the step input (first pass) or of
//                                                     the previous pass's extrema
//   pseudo    v(x, a)                              -> lambda_x, and lambda_a: the
//                                                     velocity gradient (first pass) or
//                                                     the previous pass's lambda_w
//   upwind    xant(psi, u)                         -> lambda_psi, lambda_u
// Each reverse kernel walks the forward stage's reads (with the same boundary
// index maps) and scatters the products of the local partial derivatives
// with atomic adds, so wall faces (constant zero), mirrored z faces and
// periodic wraps are transposed exactly as the forward reads them.  The
// summation order of the atomics is not fixed: results agree with the FP64
// AD oracle to rounding, not bit for bit.
#include "mpdata_body.cuh"
#include "mpdata_stages.cuh"

namespace mpdata {

// Launch bounds of the reverse kernels: minimum resident 128-thread blocks
// per SM (0: no explicit bound).  Build-time overridable for tuning sweeps;
// a sweep of 6-16 blocks per kernel measured within 0.5% of no bound.
#ifndef MPDATA_MINB_KA_PSEUDO
#define MPDATA_MINB_KA_PSEUDO 0
#endif
#ifndef MPDATA_MINB_KA_BOUNDS
#define MPDATA_MINB_KA_BOUNDS 0
#endif
#ifndef MPDATA_MINB_KA_UPWIND
#define MPDATA_MINB_KA_UPWIND 0
#endif
#ifndef MPDATA_MINB_KA_LIMIT
#define MPDATA_MINB_KA_LIMIT 0
#endif
#ifndef MPDATA_MINB_KA_UPDATE
#define MPDATA_MINB_KA_UPDATE 0
#endif
#define KA_BOUND_(n) __launch_bounds__(128, n)
#define KA_BOUND0 __launch_bounds__(128)
#if MPDATA_MINB_KA_PSEUDO > 0
#define KA_LB_PSEUDO KA_BOUND_(MPDATA_MINB_KA_PSEUDO)
#else
#define KA_LB_PSEUDO KA_BOUND0
#endif
#if MPDATA_MINB_KA_BOUNDS > 0
#define KA_LB_BOUNDS KA_BOUND_(MPDATA_MINB_KA_BOUNDS)
#else
#define KA_LB_BOUNDS KA_BOUND0
#endif
#if MPDATA_MINB_KA_UPWIND > 0
#define KA_LB_UPWIND KA_BOUND_(MPDATA_MINB_KA_UPWIND)
#else
#define KA_LB_UPWIND KA_BOUND0
#endif
#if MPDATA_MINB_KA_LIMIT > 0
#define KA_LB_LIMIT KA_BOUND_(MPDATA_MINB_KA_LIMIT)
#else
#define KA_LB_LIMIT KA_BOUND0
#endif
#if MPDATA_MINB_KA_UPDATE > 0
#define KA_LB_UPDATE KA_BOUND_(MPDATA_MINB_KA_UPDATE)
#else
#define KA_LB_UPDATE KA_BOUND0
#endif
// The record kernels run the forward stage bodies: the forward stage
// kernels' bounds (FP64 / FP32).
template <class R, int N64, int N32>
struct KfMinBlocks {
  static constexpr int v = sizeof(R) == 8 ? N64 : N32;
};

// ---- adjoints of the read maps --------------------------------------------
// Adding a zero changes no accumulator (they start at +0), so zero
// contributions, frequent where the limiter is inactive, skip the atomic; the
// test is an integer one on the FP64 bit pattern.
__device__ __forceinline__ bool nonzero(double v) { return nonzero_bits(v); }
__device__ __forceinline__ bool nonzero(float v) { return v != 0.0f; }
template <class R>
__device__ __forceinline__ void addat(const Arr<R>& A, int i, int j, int k, R v) {
  if (nonzero(v)) atomicAdd(&A.at(i, j, k), v);
}
// xr(): the field with the xant halo rule (reflection or wrap).  IN: the
// index is inside the grid (a cell in [2, n-1] reading +-1), the map is the
// identity.
template <class R, bool IN = false>
__device__ __forceinline__ void xr_add(const Geo& g, const Arr<R>& L, int i, int j, int k, R v) {
  if (IN) { addat(L, i, j, k, v); return; }
  addat(L, g.bx ? wrapi(i, g.np) : refl(i, g.np), g.by ? wrapi(j, g.mp) : refl(j, g.mp), cz(g, k), v);
}
// fx/fy/fz<AIN>()
template <class R, bool AIN, bool IN = false>
__device__ __forceinline__ void fx_add(const Geo& g, const Arr<R>& A, int f, int j, int k, R v) {
  if (IN) { addat(A, f, j, k, v); return; }
  j = cy(g, j);
  k = cz(g, k);
  if (g.bx) { addat(A, wrapi(f, g.np), j, k, v); return; }
  if (AIN) { addat(A, f, j, k, v); return; }
  if (f <= 1 || f > g.np) return;  // wall faces are the constant 0
  addat(A, f, j, k, v);
}
template <class R, bool AIN, bool IN = false>
__device__ __forceinline__ void fy_add(const Geo& g, const Arr<R>& A, int i, int f, int k, R v) {
  if (IN) { addat(A, i, f, k, v); return; }
  i = cx(g, i);
  k = cz(g, k);
  if (g.by) { addat(A, i, wrapi(f, g.mp), k, v); return; }
  if (AIN) { addat(A, i, f, k, v); return; }
  if (f <= 1 || f > g.mp) return;
  addat(A, i, f, k, v);
}
template <class R, bool AIN, bool IN = false>
__device__ __forceinline__ void fz_add(const Geo& g, const Arr<R>& A, int i, int j, int f, R v) {
  if (IN) { addat(A, i, j, f, v); return; }
  i = cx(g, i);
  j = cy(g, j);
  if (g.bz) { addat(A, i, j, wrapi(f, g.lp), v); return; }
  if (AIN) { addat(A, i, j, f, v); return; }
  if (f <= 1) { addat(A, i, j, 2, -v); return; }       // face 1 reads -face 2
  if (f > g.lp) { addat(A, i, j, g.lp, -v); return; }  // face lp+1 reads -face lp
  addat(A, i, j, f, v);
}

// derivative conventions of the branches (forward values decide); the
// tests are integer ones on the sign bit and the magnitude bits
template <class R> __device__ __forceinline__ R dpp(R y) { return (!sgn(y) && nonzero(y)) ? R(1) : R(0); }
template <class R> __device__ __forceinline__ R dpn(R y) { return (sgn(y) && nonzero(y)) ? R(-1) : R(0); }
template <class R> __device__ __forceinline__ R dabs(R y) { return sgn(y) ? R(-1) : R(1); }


// Reverse kernels: the body is a device function of (i,j,k) templated on
// IN; warps away from every wall take IN = true.
#define ADISPATCH(CALL)                                      \
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;  \
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;  \
  const int k = blockIdx.z + 1;                              \
  const bool win = warp_interior(P.g, i, j, k);              \
  if (i > P.g.np || j > P.g.mp) return;                      \
  if (win) {                                                 \
    CALL(true);                                              \
  } else {                                                   \
    CALL(false);                                             \
  }

#define ACELL                                                \
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;  \
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;  \
  const int k = blockIdx.z + 1;                              \
  if (i > P.g.np || j > P.g.mp) return;                      \
  const Geo& g = P.g;

// ---- update: x_new = rhr*(q - D/h), D = sum of signed limited fluxes -------
template <class R, bool IN>
__device__ __forceinline__ void ka_update_cell(const Prob<R>& P, const AdjArr<R>& A, int i, int j, int k) {
  const Geo& g = P.g;
  const R ln = A.lam.ld(i, j, k);
  const R rh = P.rhr.ld(i, j, k);
  const R lt = rh * ln;                 // d x_new / d t, t = q - D/h
  A.lxant.at(i, j, k) = lt / rh;        // q = xant/rhr
  const R lD = -lt / P.h.ld(i, j, k);
  fx_add<R, false, IN>(g, A.lw1, i + 1, j, k, lD);
  fx_add<R, false, IN>(g, A.lw1, i, j, k, -lD);
  fy_add<R, false, IN>(g, A.lw2, i, j + 1, k, lD);
  fy_add<R, false, IN>(g, A.lw2, i, j, k, -lD);
  fz_add<R, false, IN>(g, A.lw3, i, j, k + 1, lD);
  fz_add<R, false, IN>(g, A.lw3, i, j, k, -lD);
}
template <class R>
__global__ void KA_LB_UPDATE ka_update(const Prob<R> P, const AdjArr<R> A) {
#define C(IN) ka_update_cell<R, IN>(P, A, i, j, k)
  ADISPATCH(C)
#undef C
}

// ---- limiter: w = pp(v)*min3(cp(c),cn(c-1)) - pn(v)*min3(cp(c-1),cn(c)) -------
// min3(a,b) = mn2(mn2(1,a),b): b is taken when b <= t, else a when a <= 1.
// The ratios are non-negative (or RATIO_CAP), so for doubles their bit
// patterns order as their values and the compares run on the integer pipe.
__device__ __forceinline__ bool lt_nonneg(double a, double b) {
  return __double_as_longlong(a) < __double_as_longlong(b);
}
__device__ __forceinline__ bool lt_nonneg(float a, float b) { return a < b; }
template <class R>
__device__ __forceinline__ void min3_adj(R a, R b, R lam, const Arr<R>& La, int ia, int ja, int ka,
                                         const Arr<R>& Lb, int ib, int jb, int kb) {
  const bool a_over = lt_nonneg(R(1), a);
  const R t = a_over ? R(1) : a;
  if (!lt_nonneg(t, b)) { addat(Lb, ib, jb, kb, lam); return; }
  if (!a_over) addat(La, ia, ja, ka, lam);
}

template <class R, bool NONOS, bool IN>
__device__ __forceinline__ void ka_limit_cell(const Prob<R>& P, const AdjArr<R>& A, int i, int j, int k) {
  const Geo& g = P.g;
  const R cpc = NONOS ? P.cp.ld(i, j, k) : R(0), cnc = NONOS ? P.cn.ld(i, j, k) : R(0);
#define LIMIT_FACE(V, LV, LW, IM, JM, KM)                                                  \
  {                                                                                        \
    const R v = V.ld(i, j, k);                                                             \
    const R lw = LW.ld(i, j, k);                                                           \
    if (!NONOS) {                                                                          \
      addat(LV, i, j, k, lw);                                                              \
    } else {                                                                               \
      const R cpm = P.cp.ld(IM, JM, KM), cnm = P.cn.ld(IM, JM, KM);                        \
      /* dw/dv = a1 (v > 0), a2 (v < 0), 0; dw/da1 = pp(v), dw/da2 = -pn(v): */          \
      /* one of them is v, the other zero */                                              \
      const bool vz = !nonzero(v), vn = sgn(v);                                             \
      const R m = lw * v;                                                                   \
      if (!vz) addat(LV, i, j, k, lw * (vn ? min3(cpm, cnc) : min3(cpc, cnm)));             \
      if (!vz && !vn) min3_adj(cpc, cnm, m, A.lcp, i, j, k, A.lcn, IM, JM, KM);             \
      if (!vz && vn) min3_adj(cpm, cnc, m, A.lcp, IM, JM, KM, A.lcn, i, j, k);              \
    }                                                                                      \
  }
  if (IN || g.bx || i > 1) LIMIT_FACE(P.v1, A.lv1, A.lw1, (IN ? i - 1 : wrapi(i - 1, g.np)), j, k)
  if (IN || g.by || j > 1) LIMIT_FACE(P.v2, A.lv2, A.lw2, i, (IN ? j - 1 : wrapi(j - 1, g.mp)), k)
  if (IN || g.bz || k > 1) LIMIT_FACE(P.v3, A.lv3, A.lw3, i, j, (IN ? k - 1 : wrapi(k - 1, g.lp)))
#undef LIMIT_FACE
}
template <class R, bool NONOS>
__global__ void KA_LB_LIMIT ka_limit(const Prob<R> P, const AdjArr<R> A) {
#define C(IN) ka_limit_cell<R, NONOS, IN>(P, A, i, j, k)
  ADISPATCH(C)
#undef C
}

// ---- bounds: cp = (mx-x)h/Dp, cn = (x-mn)h/Dn -------------------------------
// The extrema are re-folded in the oracle's order (mx2/mn2 trees) with the
// compare-and-select's own semantics (ties, +0 == -0 included, keep the
// second operand), so each goes to the same operand: element ids 0..6 are
// x_in, 7..13 xant.  FP64 values compare on the integer pipe (ieee_gt).
__device__ __forceinline__ bool arg_gt(double a, double b) { return ieee_gt(a, b); }
__device__ __forceinline__ bool arg_gt(float a, float b) { return a > b; }
template <class R>
struct Arg {
  R v;
  int id;
};
template <class R> __device__ __forceinline__ Arg<R> mkarg(R v, int id) { return Arg<R>{v, id}; }
template <class R> __device__ __forceinline__ Arg<R> amax(Arg<R> a, Arg<R> b) { return arg_gt(a.v, b.v) ? a : b; }
template <class R> __device__ __forceinline__ Arg<R> amin(Arg<R> a, Arg<R> b) { return arg_gt(b.v, a.v) ? a : b; }

// Adjoint of the bounds' denominators onto one flux f: Dp holds pn(f) and
// Dn pp(f) for an outflow face (e), the reverse for an inflow face (w); a
// zero flux contributes to neither.
template <class R>
__device__ __forceinline__ R lflux(R f, R lDp, R lDn, bool inflow) {
  if (!nonzero(f)) return R(0);
  const bool neg = sgn(f);
  if (inflow) return neg ? -lDn : lDp;
  return neg ? -lDp : lDn;
}

// FIRST: the fold starts from the step input's star (ids 0..6); later passes
// start from the previous pass's running extrema (id 14).  The current
// field's star is ids 7..13.  The adjoint of this pass's extrema is the
// cp/cn part plus what the next pass carried back (lmx, lmn).
// STD: the fluxes of the bounds are the unlimited donor fluxes f*ns (their
// adjoint goes to lf); gauge: the pseudo-velocities themselves (lv).
template <class R, bool FIRST, bool STD, bool IN>
__device__ __forceinline__ void ka_bounds_cell(const Prob<R>& P, const AdjArr<R>& A, int i, int j, int k) {
  const Geo& g = P.g;
  const bool lo = IN || g.bz || k > 1, hi = IN || g.bz || k < g.lp;
  const Arr<R>& X = P.xant;
  const Arr<R>& xin = P.psi;
  // star cells: x_in with the zero-gradient map, the current field with the reflection map
  const int im = IN ? i - 1 : (g.bx ? wrapi(i - 1, g.np) : clampi(i - 1, g.np));
  const int ip = IN ? i + 1 : (g.bx ? wrapi(i + 1, g.np) : clampi(i + 1, g.np));
  const int jm = IN ? j - 1 : (g.by ? wrapi(j - 1, g.mp) : clampi(j - 1, g.mp));
  const int jp = IN ? j + 1 : (g.by ? wrapi(j + 1, g.mp) : clampi(j + 1, g.mp));
  const int km = cz<IN>(g, k - 1), kp = cz<IN>(g, k + 1);
  const int ri_m = IN ? i - 1 : (g.bx ? wrapi(i - 1, g.np) : refl(i - 1, g.np)), ri_p = IN ? i + 1 : (g.bx ? wrapi(i + 1, g.np) : refl(i + 1, g.np));
  const int rj_m = IN ? j - 1 : (g.by ? wrapi(j - 1, g.mp) : refl(j - 1, g.mp)), rj_p = IN ? j + 1 : (g.by ? wrapi(j + 1, g.mp) : refl(j + 1, g.mp));
  // element table: (i,j,k) of ids 0..13; id 14 is the previous extremum at (i,j,k)
  const int ci[15] = {im, i, ip, i, i, i, i, ri_m, i, ri_p, i, i, i, i, i};
  const int cj[15] = {j, j, j, jm, jp, j, j, j, j, j, rj_m, rj_p, j, j, j};
  const int ck[15] = {k, k, k, k, k, km, kp, k, k, k, k, k, km, kp, k};
  Arg<R> e[14];
  for (int n = 7; n < 14; n++) e[n] = mkarg(X.ld(ci[n], cj[n], ck[n]), n);
  Arg<R> ma, mi;
  if (FIRST) {
    for (int n = 0; n < 7; n++) e[n] = mkarg(xin.ld(ci[n], cj[n], ck[n]), n);
    ma = amax(amax(amax(e[0], e[1]), amax(e[2], e[3])), e[4]);
    mi = amin(amin(amin(e[0], e[1]), amin(e[2], e[3])), e[4]);
    if (lo) { ma = amax(ma, e[5]); mi = amin(mi, e[5]); }
    if (hi) { ma = amax(ma, e[6]); mi = amin(mi, e[6]); }
  } else {
    ma = mkarg(A.mxp.ld(i, j, k), 14);
    mi = mkarg(A.mnp.ld(i, j, k), 14);
  }
  ma = amax(amax(amax(ma, e[7]), amax(e[8], e[9])), amax(e[10], e[11]));
  mi = amin(amin(amin(mi, e[7]), amin(e[8], e[9])), amin(e[10], e[11]));
  if (lo) { ma = amax(ma, e[12]); mi = amin(mi, e[12]); }
  if (hi) { ma = amax(ma, e[13]); mi = amin(mi, e[13]); }

  const R x = X.ld(i, j, k), hc = P.h.ld(i, j, k);
  const R lcp = A.lcp.ld(i, j, k), lcn = A.lcn.ld(i, j, k);
  const Arr<R>& F1 = STD ? P.f1 : P.v1;
  const Arr<R>& F2 = STD ? P.f2 : P.v2;
  const Arr<R>& F3 = STD ? P.f3 : P.v3;
  const Arr<R>& LF1 = STD ? A.lf1 : A.lv1;
  const Arr<R>& LF2 = STD ? A.lf2 : A.lv2;
  const Arr<R>& LF3 = STD ? A.lf3 : A.lv3;
  const R e1 = fx<R, false, IN>(g, F1, i + 1, j, k), w1 = fx<R, false, IN>(g, F1, i, j, k);
  const R e2 = fy<R, false, IN>(g, F2, i, j + 1, k), w2 = fy<R, false, IN>(g, F2, i, j, k);
  const R e3 = fz<R, false, IN>(g, F3, i, j, k + 1), w3 = fz<R, false, IN>(g, F3, i, j, k);
  // d cp/d mx, d cn/d mn (plus the carried adjoints of the extrema), d/d x,
  // and d/dD = -c/D.  cp = num/Dp: lnum = lcp*h/Dp, lDp = -lnum*(mx-x)/Dp,
  // with one reciprocal per denominator; both vanish where the limiter did
  // not select the ratio (lcp = 0), as they mostly do.
  R lnum_p = R(0), lnum_n = R(0), lDp = R(0), lDn = R(0);
  if (nonzero(lcp) || nonzero(lcn)) {
    const R ep = Eps<R>::v;
    const R Dp = pn(e1) + pp(w1) + pn(e2) + pp(w2) + pn(e3) + pp(w3) + ep;
    const R Dn = pp(e1) + pn(w1) + pp(e2) + pn(w2) + pp(e3) + pn(w3) + ep;
    const R rp = R(1) / Dp, rn = R(1) / Dn;
    lnum_p = lcp * hc * rp;
    lnum_n = lcn * hc * rn;
    lDp = -(lnum_p * (ma.v - x)) * rp;
    lDn = -(lnum_n * (x - mi.v)) * rn;
  }
  const R lma = lnum_p + A.lmx.ld(i, j, k), lmi = -lnum_n + A.lmn.ld(i, j, k);
  if (ma.id == 14) addat(A.lmxp, i, j, k, lma);
  else addat(ma.id < 7 ? A.lx : A.lxant, ci[ma.id], cj[ma.id], ck[ma.id], lma);
  if (mi.id == 14) addat(A.lmnp, i, j, k, lmi);
  else addat(mi.id < 7 ? A.lx : A.lxant, ci[mi.id], cj[mi.id], ck[mi.id], lmi);
  addat(A.lxant, i, j, k, lnum_n - lnum_p);
  // Dp = pn(e)+pp(w)+..., Dn = pp(e)+pn(w)+... over the six faces
  fx_add<R, false, IN>(g, LF1, i + 1, j, k, lflux(e1, lDp, lDn, false));
  fx_add<R, false, IN>(g, LF1, i, j, k, lflux(w1, lDp, lDn, true));
  fy_add<R, false, IN>(g, LF2, i, j + 1, k, lflux(e2, lDp, lDn, false));
  fy_add<R, false, IN>(g, LF2, i, j, k, lflux(w2, lDp, lDn, true));
  fz_add<R, false, IN>(g, LF3, i, j, k + 1, lflux(e3, lDp, lDn, false));
  fz_add<R, false, IN>(g, LF3, i, j, k, lflux(w3, lDp, lDn, true));
}
template <class R, bool FIRST, bool STD>
__global__ void KA_LB_BOUNDS ka_bounds(const Prob<R> P, const AdjArr<R> A) {
#define C(IN) ka_bounds_cell<R, FIRST, STD, IN>(P, A, i, j, k)
  ADISPATCH(C)
#undef C
}

// ---- pseudo-velocity (gauge): v = vdyf(xl,xr,a,hm) - 0.125*a*hm*cr ------------
// cr = S2*rat4(y0,y1,y2,y3) [+ S3*rat4(z0,z1,z2,z3)], S = sums of four a faces.
// AIN: a = the caller's Courant numbers (gradient into gu); otherwise a = the
// previous pass's limited velocities, read with the wall rule (gradient into
// that pass's lambda_w).
template <class R> __device__ __forceinline__ R negv(R x) { return -x; }
template <> __device__ __forceinline__ double negv<double>(double x) { return neg_bits(x); }

// The adjoint of one face's v = K*(xr-xl) - 0.03125*a*hm*cr4, with
// K = (|a| - a*a*hm)/2 and cr4 = S*D [+ S'*D'], the 4-face sums S times the
// unscaled rat4 differences D (4*cr of the forward's form).  U: hm == 1.
template <class R, bool U>
struct FaceAdj {
  R la, lK, lcr4;
  __device__ __forceinline__ FaceAdj(R lv, R a, R hm, R xl, R xrr, R cr4) {
    // the products by powers of two run on the integer pipe (scale_down/up)
    const R K = scale_down<1>(fabs(a) - hmul<U>(a * a, hm));
    la = lv * (scale_down<1>((dabs(a) - hmul<U>(scale_up<1>(a), hm)) * (xrr - xl)) -
               hmul<U>(scale_down<5>(cr4), hm));
    lK = lv * K;
    lcr4 = negv(lv * hmul<U>(scale_down<5>(a), hm));
  }
};

// U: the warp's face densities are all exactly 1.  PS: the pair sums of the
// pass's input field are in cp/cn/q (kf_pairs), as in the forward stage.
// PV (with PS): the velocities' cell-centred pairs are in f1..f3.  Without IN
// (a full warp at a boundary) the stored pairs are read through the boundary
// maps of the values they sum, as in pseudo_form.
template <class R, bool AIN, bool IN, bool U = false, bool PS = false, bool PV = false>
__device__ __forceinline__ void ka_pseudo_cell(const Prob<R>& P, const AdjArr<R>& A, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& X = P.xant;
  const Arr<R>& U1 = AIN ? P.u1 : P.w1;
  const Arr<R>& U2 = AIN ? P.u2 : P.w2;
  const Arr<R>& U3 = AIN ? P.u3 : P.w3;
  const bool zt = IN || g.bz || (k > 1 && k < g.lp);
#define XX(a, b, c) xr<R, IN>(g, X, (a), (b), (c))
#define LX(a, b, c, v) xr_add<R, IN>(g, A.lxant, (a), (b), (c), (v))
#define AX(f, b, c) fx<R, AIN, IN>(g, U1, (f), (b), (c))
#define AY(a, f, c) fy<R, AIN, IN>(g, U2, (a), (f), (c))
#define AZ(a, b, f) fz<R, AIN, IN>(g, U3, (a), (b), (f))
#define MX(a) cx<IN>(g, (a))
#define MY(a) cy<IN>(g, (a))
#define MZ(a) cz<IN>(g, (a))
#define QX(a) xmx<IN>(g, (a))
#define QY(a) xmy<IN>(g, (a))
#define S2X_ (PV ? P.f2.ld(MX(i - 1), j, k) + P.f2.ld(i, j, k) : VSUM_2X)
#define S3X_ (PV ? P.f3.ld(MX(i - 1), j, k) + P.f3.ld(i, j, k) : VSUM_3X)
#define S1Y_ (PV ? P.f1.ld(i, MY(j - 1), k) + P.f1.ld(i, j, k) : VSUM_1Y)
#define S3Y_ (PV ? P.f3.ld(i, MY(j - 1), k) + P.f3.ld(i, j, k) : VSUM_3Y)
#define S1Z_ (PV ? P.f1.ld(i, j, MZ(k - 1)) + P.f1.ld(i, j, k) : VSUM_1Z)
#define S2Z_ (PV ? P.f2.ld(i, j, MZ(k - 1)) + P.f2.ld(i, j, k) : VSUM_2Z)
  // x faces
  if (IN || g.bx || i > 1) {
    const R lv = A.lv1.ld(i, j, k);
    const R hm = U ? R(1) : P.hmx.ld(i, j, k), a = fx<R, AIN, IN>(g, U1, i, j, k);
    const R xl = XX(i - 1, j, k), xrr = XX(i, j, k);
    const R S2 = S2X_;
    const R D2 = PS ? P.cp.ld(i, QY(j + 1), k) - P.cp.ld(i, QY(j - 1), k)
                    : dif4(XX(i - 1, j - 1, k), XX(i, j - 1, k), XX(i - 1, j + 1, k), XX(i, j + 1, k));
    R cr4 = S2 * D2, S3 = R(0), D3 = R(0);
    if (zt) {
      S3 = S3X_;
      D3 = PS ? P.cp.ld(i, j, MZ(k + 1)) - P.cp.ld(i, j, MZ(k - 1))
              : dif4(XX(i - 1, j, k - 1), XX(i, j, k - 1), XX(i - 1, j, k + 1), XX(i, j, k + 1));
      cr4 = cr4 + S3 * D3;
    }
    const FaceAdj<R, U> f(lv, a, hm, xl, xrr, cr4);
    fx_add<R, AIN, IN>(g, A.la1, i, j, k, f.la);
    LX(i, j, k, f.lK);
    LX(i - 1, j, k, negv(f.lK));
    const R lS2 = f.lcr4 * D2, lR2 = f.lcr4 * S2, nR2 = negv(lR2);
    fy_add<R, AIN, IN>(g, A.la2, i - 1, j, k, lS2);
    fy_add<R, AIN, IN>(g, A.la2, i - 1, j + 1, k, lS2);
    fy_add<R, AIN, IN>(g, A.la2, i, j + 1, k, lS2);
    fy_add<R, AIN, IN>(g, A.la2, i, j, k, lS2);
    LX(i, j + 1, k, lR2); LX(i - 1, j + 1, k, lR2); LX(i, j - 1, k, nR2); LX(i - 1, j - 1, k, nR2);
    if (zt) {
      const R lS3 = f.lcr4 * D3, lR3 = f.lcr4 * S3, nR3 = negv(lR3);
      fz_add<R, AIN, IN>(g, A.la3, i - 1, j, k, lS3);
      fz_add<R, AIN, IN>(g, A.la3, i - 1, j, k + 1, lS3);
      fz_add<R, AIN, IN>(g, A.la3, i, j, k + 1, lS3);
      fz_add<R, AIN, IN>(g, A.la3, i, j, k, lS3);
      LX(i, j, k + 1, lR3); LX(i - 1, j, k + 1, lR3); LX(i, j, k - 1, nR3); LX(i - 1, j, k - 1, nR3);
    }
  }
  // y faces
  if (IN || g.by || j > 1) {
    const R lv = A.lv2.ld(i, j, k);
    const R hm = U ? R(1) : P.hmy.ld(i, j, k), a = fy<R, AIN, IN>(g, U2, i, j, k);
    const R xl = XX(i, j - 1, k), xrr = XX(i, j, k);
    const R S1 = S1Y_;
    const R D1 = PS ? P.cn.ld(QX(i + 1), j, k) - P.cn.ld(QX(i - 1), j, k)
                    : dif4(XX(i - 1, j - 1, k), XX(i - 1, j, k), XX(i + 1, j - 1, k), XX(i + 1, j, k));
    R cr4 = S1 * D1, S3 = R(0), D3 = R(0);
    if (zt) {
      S3 = S3Y_;
      D3 = PS ? P.cn.ld(i, j, MZ(k + 1)) - P.cn.ld(i, j, MZ(k - 1))
              : dif4(XX(i, j - 1, k - 1), XX(i, j, k - 1), XX(i, j - 1, k + 1), XX(i, j, k + 1));
      cr4 = cr4 + S3 * D3;
    }
    const FaceAdj<R, U> f(lv, a, hm, xl, xrr, cr4);
    fy_add<R, AIN, IN>(g, A.la2, i, j, k, f.la);
    LX(i, j, k, f.lK);
    LX(i, j - 1, k, negv(f.lK));
    const R lS1 = f.lcr4 * D1, lR1 = f.lcr4 * S1, nR1 = negv(lR1);
    fx_add<R, AIN, IN>(g, A.la1, i, j - 1, k, lS1);
    fx_add<R, AIN, IN>(g, A.la1, i, j, k, lS1);
    fx_add<R, AIN, IN>(g, A.la1, i + 1, j, k, lS1);
    fx_add<R, AIN, IN>(g, A.la1, i + 1, j - 1, k, lS1);
    LX(i + 1, j, k, lR1); LX(i + 1, j - 1, k, lR1); LX(i - 1, j, k, nR1); LX(i - 1, j - 1, k, nR1);
    if (zt) {
      const R lS3 = f.lcr4 * D3, lR3 = f.lcr4 * S3, nR3 = negv(lR3);
      fz_add<R, AIN, IN>(g, A.la3, i, j - 1, k, lS3);
      fz_add<R, AIN, IN>(g, A.la3, i, j, k, lS3);
      fz_add<R, AIN, IN>(g, A.la3, i, j, k + 1, lS3);
      fz_add<R, AIN, IN>(g, A.la3, i, j - 1, k + 1, lS3);
      LX(i, j, k + 1, lR3); LX(i, j - 1, k + 1, lR3); LX(i, j, k - 1, nR3); LX(i, j - 1, k - 1, nR3);
    }
  }
  // z faces
  if (IN || g.bz || k > 1) {
    const R lv = A.lv3.ld(i, j, k);
    const R hm = U ? R(1) : P.hmz.ld(i, j, k), a = fz<R, AIN, IN>(g, U3, i, j, k);
    const R xl = XX(i, j, k - 1), xrr = XX(i, j, k);
    const R S1 = S1Z_;
    const R D1 = PS ? P.q.ld(QX(i + 1), j, k) - P.q.ld(QX(i - 1), j, k)
                    : dif4(XX(i - 1, j, k - 1), XX(i - 1, j, k), XX(i + 1, j, k - 1), XX(i + 1, j, k));
    const R S2 = S2Z_;
    const R D2 = PS ? P.q.ld(i, QY(j + 1), k) - P.q.ld(i, QY(j - 1), k)
                    : dif4(XX(i, j - 1, k - 1), XX(i, j - 1, k), XX(i, j + 1, k - 1), XX(i, j + 1, k));
    const R cr4 = S1 * D1 + S2 * D2;
    const FaceAdj<R, U> f(lv, a, hm, xl, xrr, cr4);
    fz_add<R, AIN, IN>(g, A.la3, i, j, k, f.la);
    LX(i, j, k, f.lK);
    LX(i, j, k - 1, negv(f.lK));
    const R lS1 = f.lcr4 * D1, lR1 = f.lcr4 * S1, nR1 = negv(lR1);
    fx_add<R, AIN, IN>(g, A.la1, i, j, k - 1, lS1);
    fx_add<R, AIN, IN>(g, A.la1, i, j, k, lS1);
    fx_add<R, AIN, IN>(g, A.la1, i + 1, j, k, lS1);
    fx_add<R, AIN, IN>(g, A.la1, i + 1, j, k - 1, lS1);
    LX(i + 1, j, k, lR1); LX(i + 1, j, k - 1, lR1); LX(i - 1, j, k, nR1); LX(i - 1, j, k - 1, nR1);
    const R lS2 = f.lcr4 * D2, lR2 = f.lcr4 * S2, nR2 = negv(lR2);
    fy_add<R, AIN, IN>(g, A.la2, i, j, k - 1, lS2);
    fy_add<R, AIN, IN>(g, A.la2, i, j + 1, k - 1, lS2);
    fy_add<R, AIN, IN>(g, A.la2, i, j + 1, k, lS2);
    fy_add<R, AIN, IN>(g, A.la2, i, j, k, lS2);
    LX(i, j + 1, k, lR2); LX(i, j + 1, k - 1, lR2); LX(i, j - 1, k, nR2); LX(i, j - 1, k - 1, nR2);
  }
#undef XX
#undef LX
#undef AX
#undef AY
#undef AZ
#undef MX
#undef MY
#undef MZ
#undef QX
#undef QY
#undef S2X_
#undef S3X_
#undef S1Y_
#undef S3Y_
#undef S1Z_
#undef S2Z_
}
template <class R, bool AIN>
__global__ void KA_LB_PSEUDO ka_pseudo(const Prob<R> P, const AdjArr<R> A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  const bool win = warp_interior(P.g, i, j, k);
  // every pair sum stored (pairs 2): full warps at a boundary read them too
  bool pin = false;
  if (!win && P.pairs == 2) pin = warp_on_grid(P.g, i, j);
  if (i > P.g.np || j > P.g.mp) return;
  if (!win) {
    if (pin) {
      if (warp_unit_faces(P, i, j, k))
        ka_pseudo_cell<R, AIN, false, true, true, true>(P, A, i, j, k);
      else
        ka_pseudo_cell<R, AIN, false, false, true, true>(P, A, i, j, k);
      return;
    }
    ka_pseudo_cell<R, AIN, false>(P, A, i, j, k);
  } else if constexpr (sizeof(R) == 8) {
    const bool unit = warp_unit_faces(P, i, j, k);
    if (P.pairs == 2) {
      if (unit)
        ka_pseudo_cell<R, AIN, true, true, true, true>(P, A, i, j, k);
      else
        ka_pseudo_cell<R, AIN, true, false, true, true>(P, A, i, j, k);
    } else if (P.pairs) {
      if (unit)
        ka_pseudo_cell<R, AIN, true, true, true>(P, A, i, j, k);
      else
        ka_pseudo_cell<R, AIN, true, false, true>(P, A, i, j, k);
    } else {
      if (unit)
        ka_pseudo_cell<R, AIN, true, true>(P, A, i, j, k);
      else
        ka_pseudo_cell<R, AIN, true>(P, A, i, j, k);
    }
  } else if (P.pairs == 2) {  // FP32: the stored pairs save issue slots
    ka_pseudo_cell<R, AIN, true, false, true, true>(P, A, i, j, k);
  } else {
    ka_pseudo_cell<R, AIN, true>(P, A, i, j, k);
  }
}

// ---- standard form (antidiff3d-standard-gpubc.f90) ---------------------------
// update: x_out = rhr*(q - d*hinv), d = signed sum of the limited fluxes g
template <class R, bool IN>
__device__ __forceinline__ void ka_update_std_cell(const Prob<R>& P, const AdjArr<R>& A, int i, int j, int k) {
  const Geo& g = P.g;
  const R lt = P.rhr.ld(i, j, k) * A.lam.ld(i, j, k);
  addat(A.lq, i, j, k, lt);
  const R lD = -lt * P.hinv.ld(i, j, k);
  fx_add<R, false, IN>(g, A.lg1, i + 1, j, k, lD);
  fx_add<R, false, IN>(g, A.lg1, i, j, k, -lD);
  fy_add<R, false, IN>(g, A.lg2, i, j + 1, k, lD);
  fy_add<R, false, IN>(g, A.lg2, i, j, k, -lD);
  fz_add<R, false, IN>(g, A.lg3, i, j, k + 1, lD);
  fz_add<R, false, IN>(g, A.lg3, i, j, k, -lD);
}
template <class R>
__global__ void __launch_bounds__(128) ka_update_std(const Prob<R> P, const AdjArr<R> A) {
#define C(IN) ka_update_std_cell<R, IN>(P, A, i, j, k)
  ADISPATCH(C)
#undef C
}

// limiter: w = vlim_std(v, a1, a2, x(c-1), x(c)) with a1 = min3(cp(c), cn(c-1)),
// a2 = min3(cp(c-1), cn(c)); g = donor(q(c-1), q(c), w).  possign() is
// piecewise constant: only v, a1 and a2 carry a derivative through it.
template <class R, bool NONOS, bool IN>
__device__ __forceinline__ void ka_limit_std_cell(const Prob<R>& P, const AdjArr<R>& A, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& X = P.xant;
  const R cpc = NONOS ? P.cp.ld(i, j, k) : R(0), cnc = NONOS ? P.cn.ld(i, j, k) : R(0);
  const R xc = X.ld(i, j, k), qc = P.q.ld(i, j, k);
#define LIMIT_STD_FACE(V, LV, LW, LG, IM, JM, KM)                                                       \
  {                                                                                                     \
    const R v = V.ld(i, j, k);                                                                          \
    const R xl = X.ld(IM, JM, KM), ql = P.q.ld(IM, JM, KM);                                             \
    R w = v, a1 = R(0), a2 = R(0), cpm = R(0), cnm = R(0);                                              \
    if (NONOS) {                                                                                        \
      cpm = P.cp.ld(IM, JM, KM);                                                                        \
      cnm = P.cn.ld(IM, JM, KM);                                                                        \
      a1 = min3(cpc, cnm);                                                                              \
      a2 = min3(cpm, cnc);                                                                              \
      w = vlim_std(v, a1, a2, xl, xc);                                                                  \
    }                                                                                                   \
    const R lg = LG.ld(i, j, k);                                                                        \
    addat(A.lq, IM, JM, KM, lg * pp(w));                                                                \
    addat(A.lq, i, j, k, -lg * pn(w));                                                                  \
    const R lw = LW.ld(i, j, k) + lg * (dpp(w) * ql - dpn(w) * qc);                                     \
    if (!NONOS) {                                                                                       \
      addat(LV, i, j, k, lw);                                                                           \
    } else {                                                                                            \
      const R sl = possign(xl), sml = possign(-xl), sr = possign(xc), smr = possign(-xc);              \
      addat(LV, i, j, k, lw * (dpp(v) * (a1 * sl + a2 * sml) - dpn(v) * (a2 * sr + a1 * smr)));         \
      min3_adj(cpc, cnm, lw * (pp(v) * sl - pn(v) * smr), A.lcp, i, j, k, A.lcn, IM, JM, KM);          \
      min3_adj(cpm, cnc, lw * (pp(v) * sml - pn(v) * sr), A.lcp, IM, JM, KM, A.lcn, i, j, k);          \
    }                                                                                                   \
  }
  if (IN || g.bx || i > 1) LIMIT_STD_FACE(P.v1, A.lv1, A.lw1, A.lg1, (IN ? i - 1 : wrapi(i - 1, g.np)), j, k)
  if (IN || g.by || j > 1) LIMIT_STD_FACE(P.v2, A.lv2, A.lw2, A.lg2, i, (IN ? j - 1 : wrapi(j - 1, g.mp)), k)
  if (IN || g.bz || k > 1) LIMIT_STD_FACE(P.v3, A.lv3, A.lw3, A.lg3, i, j, (IN ? k - 1 : wrapi(k - 1, g.lp)))
#undef LIMIT_STD_FACE
}
template <class R, bool NONOS>
__global__ void __launch_bounds__(128) ka_limit_std(const Prob<R> P, const AdjArr<R> A) {
#define C(IN) ka_limit_std_cell<R, NONOS, IN>(P, A, i, j, k)
  ADISPATCH(C)
#undef C
}

// vcorra(a, b, y1, y2, hm) = -(0.125*a*b*y1*hm/y2) with y1 = (|p1|+|p2|)-(|m1|+|m2|),
// y2 = |p1|+|p2|+|m1|+|m2|+ep; returns dv/da and dv/db, scatters dv/dx.
template <class R>
struct VcTerm {
  R lb;  // lambda of b
  R la;  // lambda of a
};
template <class R, bool IN>
__device__ __forceinline__ VcTerm<R> vcorra_adj(const Geo& g, const Arr<R>& X, const Arr<R>& LX, R lv, R a, R b,
                                                R hm, int pi1, int pj1, int pk1, int pi2, int pj2, int pk2,
                                                int mi1, int mj1, int mk1, int mi2, int mj2, int mk2) {
  const R p1 = xr<R, IN>(g, X, pi1, pj1, pk1), p2 = xr<R, IN>(g, X, pi2, pj2, pk2);
  const R m1 = xr<R, IN>(g, X, mi1, mj1, mk1), m2 = xr<R, IN>(g, X, mi2, mj2, mk2);
  const R y1 = (fabs(p1) + fabs(p2)) - (fabs(m1) + fabs(m2));
  const R y2 = fabs(p1) + fabs(p2) + fabs(m1) + fabs(m2) + Eps<R>::v;
  const R t = -R(0.125) * hm;
  const R dy1 = t * a * b / y2, dy2 = -t * a * b * y1 / (y2 * y2);
  xr_add<R, IN>(g, LX, pi1, pj1, pk1, lv * (dy1 + dy2) * dabs(p1));
  xr_add<R, IN>(g, LX, pi2, pj2, pk2, lv * (dy1 + dy2) * dabs(p2));
  xr_add<R, IN>(g, LX, mi1, mj1, mk1, lv * (dy2 - dy1) * dabs(m1));
  xr_add<R, IN>(g, LX, mi2, mj2, mk2, lv * (dy2 - dy1) * dabs(m2));
  return VcTerm<R>{lv * t * a * y1 / y2, lv * t * b * y1 / y2};
}

// pseudo-velocity: f*ns = donor(xl, xr, v) first, then
// v = vdyfa(xl, xr, a, hm) + vcorra(cross 1) [+ vcorra(cross 2)], and the
// q = x/rhr of the limiter's fluxes back into x.
template <class R, bool AIN, bool IN>
__device__ __forceinline__ void ka_pseudo_std_cell(const Prob<R>& P, const AdjArr<R>& A, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& X = P.xant;
  const Arr<R>& U1 = AIN ? P.u1 : P.w1;
  const Arr<R>& U2 = AIN ? P.u2 : P.w2;
  const Arr<R>& U3 = AIN ? P.u3 : P.w3;
  const R ep = Eps<R>::v;
  const bool zt = IN || g.bz || (k > 1 && k < g.lp);
  addat(A.lxant, i, j, k, A.lq.ld(i, j, k) / P.rhr.ld(i, j, k));
#define XX(a, b, c) xr<R, IN>(g, X, (a), (b), (c))
#define LX(a, b, c, v) xr_add<R, IN>(g, A.lxant, (a), (b), (c), (v))
#define AX(f, b, c) fx<R, AIN, IN>(g, U1, (f), (b), (c))
#define AY(a, f, c) fy<R, AIN, IN>(g, U2, (a), (f), (c))
#define AZ(a, b, f) fz<R, AIN, IN>(g, U3, (a), (b), (f))
  // the face's own velocity, donor flux and vdyfa; returns lambda of v after f*ns
#define FACE_HEAD(LV, LF, V, AF, HM, XLI, XLJ, XLK)                                                     \
  const R v = V.ld(i, j, k), hm = HM.ld(i, j, k), a = AF;                                           \
  const R xl = XX(XLI, XLJ, XLK), xrr = XX(i, j, k);                                                \
  const R lf = LF.ld(i, j, k);                                                                      \
  LX(XLI, XLJ, XLK, lf * pp(v));                                                                    \
  LX(i, j, k, -lf * pn(v));                                                                         \
  const R lv = LV.ld(i, j, k) + lf * (dpp(v) * xl - dpn(v) * xrr);                                  \
  const R K = fabs(a) - a * a * hm, N = fabs(xrr) - fabs(xl), Dd = fabs(xrr) + fabs(xl) + ep;       \
  R la = lv * (dabs(a) - R(2) * a * hm) * N / Dd;                                                   \
  LX(i, j, k, lv * K * dabs(xrr) * (Dd - N) / (Dd * Dd));                                           \
  LX(XLI, XLJ, XLK, -lv * K * dabs(xl) * (Dd + N) / (Dd * Dd));
  if (IN || g.bx || i > 1) {
    FACE_HEAD(A.lv1, A.lf1, P.v1, (fx<R, AIN, IN>(g, U1, i, j, k)), P.hmx, i - 1, j, k)
    {
      const R b = VSUM_2X;
      const VcTerm<R> c = vcorra_adj<R, IN>(g, X, A.lxant, lv, a, b, hm, i - 1, j + 1, k, i, j + 1, k, i - 1, j - 1, k,
                                        i, j - 1, k);
      la += c.la;
      fy_add<R, AIN, IN>(g, A.la2, i - 1, j, k, c.lb);
      fy_add<R, AIN, IN>(g, A.la2, i - 1, j + 1, k, c.lb);
      fy_add<R, AIN, IN>(g, A.la2, i, j + 1, k, c.lb);
      fy_add<R, AIN, IN>(g, A.la2, i, j, k, c.lb);
    }
    if (zt) {
      const R b = VSUM_3X;
      const VcTerm<R> c = vcorra_adj<R, IN>(g, X, A.lxant, lv, a, b, hm, i - 1, j, k + 1, i, j, k + 1, i - 1, j, k - 1,
                                        i, j, k - 1);
      la += c.la;
      fz_add<R, AIN, IN>(g, A.la3, i - 1, j, k, c.lb);
      fz_add<R, AIN, IN>(g, A.la3, i - 1, j, k + 1, c.lb);
      fz_add<R, AIN, IN>(g, A.la3, i, j, k + 1, c.lb);
      fz_add<R, AIN, IN>(g, A.la3, i, j, k, c.lb);
    }
    fx_add<R, AIN, IN>(g, A.la1, i, j, k, la);
  }
  if (IN || g.by || j > 1) {
    FACE_HEAD(A.lv2, A.lf2, P.v2, (fy<R, AIN, IN>(g, U2, i, j, k)), P.hmy, i, j - 1, k)
    {
      const R b = VSUM_1Y;
      const VcTerm<R> c = vcorra_adj<R, IN>(g, X, A.lxant, lv, a, b, hm, i + 1, j - 1, k, i + 1, j, k, i - 1, j - 1, k,
                                        i - 1, j, k);
      la += c.la;
      fx_add<R, AIN, IN>(g, A.la1, i, j - 1, k, c.lb);
      fx_add<R, AIN, IN>(g, A.la1, i, j, k, c.lb);
      fx_add<R, AIN, IN>(g, A.la1, i + 1, j, k, c.lb);
      fx_add<R, AIN, IN>(g, A.la1, i + 1, j - 1, k, c.lb);
    }
    if (zt) {
      const R b = VSUM_3Y;
      const VcTerm<R> c = vcorra_adj<R, IN>(g, X, A.lxant, lv, a, b, hm, i, j - 1, k + 1, i, j, k + 1, i, j - 1, k - 1,
                                        i, j, k - 1);
      la += c.la;
      fz_add<R, AIN, IN>(g, A.la3, i, j - 1, k, c.lb);
      fz_add<R, AIN, IN>(g, A.la3, i, j, k, c.lb);
      fz_add<R, AIN, IN>(g, A.la3, i, j, k + 1, c.lb);
      fz_add<R, AIN, IN>(g, A.la3, i, j - 1, k + 1, c.lb);
    }
    fy_add<R, AIN, IN>(g, A.la2, i, j, k, la);
  }
  if (IN || g.bz || k > 1) {
    FACE_HEAD(A.lv3, A.lf3, P.v3, (fz<R, AIN, IN>(g, U3, i, j, k)), P.hmz, i, j, k - 1)
    {
      const R b = VSUM_1Z;
      const VcTerm<R> c = vcorra_adj<R, IN>(g, X, A.lxant, lv, a, b, hm, i + 1, j, k - 1, i + 1, j, k, i - 1, j, k - 1,
                                        i - 1, j, k);
      la += c.la;
      fx_add<R, AIN, IN>(g, A.la1, i, j, k - 1, c.lb);
      fx_add<R, AIN, IN>(g, A.la1, i, j, k, c.lb);
      fx_add<R, AIN, IN>(g, A.la1, i + 1, j, k, c.lb);
      fx_add<R, AIN, IN>(g, A.la1, i + 1, j, k - 1, c.lb);
    }
    {
      const R b = VSUM_2Z;
      const VcTerm<R> c = vcorra_adj<R, IN>(g, X, A.lxant, lv, a, b, hm, i, j + 1, k - 1, i, j + 1, k, i, j - 1, k - 1,
                                        i, j - 1, k);
      la += c.la;
      fy_add<R, AIN, IN>(g, A.la2, i, j, k - 1, c.lb);
      fy_add<R, AIN, IN>(g, A.la2, i, j + 1, k - 1, c.lb);
      fy_add<R, AIN, IN>(g, A.la2, i, j + 1, k, c.lb);
      fy_add<R, AIN, IN>(g, A.la2, i, j, k, c.lb);
    }
    fz_add<R, AIN, IN>(g, A.la3, i, j, k, la);
  }
#undef FACE_HEAD
#undef XX
#undef LX
#undef AX
#undef AY
#undef AZ
}
template <class R, bool AIN>
__global__ void __launch_bounds__(128) ka_pseudo_std(const Prob<R> P, const AdjArr<R> A) {
#define C(IN) ka_pseudo_std_cell<R, AIN, IN>(P, A, i, j, k)
  ADISPATCH(C)
#undef C
}

// ---- upwind: xant = rhr*(x - D*hinv), D = signed sum of donor fluxes --------
// F = donor(xl, xr, u) = pp(u)*xl - pn(u)*xr; dF/du = [u>0]*xl + [u<0]*xr.
// Open-wall neighbours come from bcx/bcy (constants: no gradient).
template <class R>
__device__ __forceinline__ void flux_adj(R lF, R xl, R xr_, R u, bool l_var, const Arr<R>& Lx, int li, int lj,
                                         int lk, bool r_var, int ri, int rj, int rk, R* lu_out) {
  // F = pp(u)*xl - pn(u)*xr: dF/dxl = pp(u), dF/dxr = -pn(u) (one of them
  // is u, the other zero), dF/du = dpp(u)*xl - dpn(u)*xr
  const R m = lF * u;
  if (sgn(u)) {
    if (r_var) addat(Lx, ri, rj, rk, m);
  } else {
    if (l_var) addat(Lx, li, lj, lk, m);
  }
  *lu_out = nonzero(u) ? lF * (sgn(u) ? xr_ : xl) : R(0);
}

// MF (density step): the step also outputs each face's upwind flux as part
// of its mass flux: the lower face's flux of every cell (u1(i), u2(j), u3(k))
// and the upper face's of the last cell along each axis (u1(np+1), ...).
// Their cotangents add to the fluxes' own; at a z wall the flux stored for
// face 1 is -F3(2) and the one for face lp+1 is -F3(lp).
template <class R, bool IN, bool MF = false>
__device__ __forceinline__ void ka_upwind_cell(const Prob<R>& P, const AdjArr<R>& A, int i, int j, int k) {
  const Geo& g = P.g;
  const Arr<R>& psi = P.psi;
  const R lxa = A.lxant.ld(i, j, k);
  const R rh = P.rhr.ld(i, j, k);
  addat(A.lx, i, j, k, lxa * rh);
  const R lD = -lxa * rh * P.hinv.ld(i, j, k);
  const R x = psi.ld(i, j, k);
  const long bx0 = (long)(j - 1) + (long)g.mp * (k - 1), bxs = (long)g.mp * g.lp;
  const long by0 = (long)(i - 1) + (long)g.np * (k - 1), bys = (long)g.np * g.lp;
  const bool im_var = IN || i > 1 || g.bx, ip_var = IN || i < g.np || g.bx, jm_var = IN || j > 1 || g.by, jp_var = IN || j < g.mp || g.by;
  const int im = IN ? i - 1 : wrapi(i - 1, g.np), ip = IN ? i + 1 : wrapi(i + 1, g.np), jm = IN ? j - 1 : wrapi(j - 1, g.mp), jp = IN ? j + 1 : wrapi(j + 1, g.mp);
  const R xim = im_var ? psi.ld(im, j, k) : P.bcx[bx0];
  const R xip = ip_var ? psi.ld(ip, j, k) : P.bcx[bx0 + bxs];
  const R xjm = jm_var ? psi.ld(i, jm, k) : P.bcy[by0];
  const R xjp = jp_var ? psi.ld(i, jp, k) : P.bcy[by0 + bys];
  R lu;
  // the mass fluxes' cotangents of the fluxes this cell computes (MF)
  R m1 = R(0), m1p = R(0), m2 = R(0), m2p = R(0), m3 = R(0), m3p = R(0);
  if (MF) {
    m1 = A.lm1.ld(i, j, k);
    m2 = A.lm2.ld(i, j, k);
    m3 = A.lm3.ld(i, j, k);
    if (!IN && i == g.np) m1p = A.lm1.ld(g.np + 1, j, k);
    if (!IN && j == g.mp) m2p = A.lm2.ld(i, g.mp + 1, k);
    if (!IN && k == g.lp) m3p = A.lm3.ld(i, j, g.lp + 1);
  }
  // x faces: D = F1(i+1) - F1(i) + ...
  flux_adj(lD + m1p, x, xip, fx<R, true, IN>(g, P.u1, i + 1, j, k), true, A.lx, i, j, k, ip_var, ip, j, k, &lu);
  fx_add<R, true, IN>(g, A.gu1, i + 1, j, k, lu);
  flux_adj(-lD + m1, xim, x, P.u1.ld(i, j, k), im_var, A.lx, im, j, k, true, i, j, k, &lu);
  fx_add<R, true, IN>(g, A.gu1, i, j, k, lu);
  flux_adj(lD + m2p, x, xjp, fy<R, true, IN>(g, P.u2, i, j + 1, k), true, A.lx, i, j, k, jp_var, i, jp, k, &lu);
  fy_add<R, true, IN>(g, A.gu2, i, j + 1, k, lu);
  flux_adj(-lD + m2, xjm, x, P.u2.ld(i, j, k), jm_var, A.lx, i, jm, k, true, i, j, k, &lu);
  fy_add<R, true, IN>(g, A.gu2, i, j, k, lu);
  if (!IN && !g.bz && k == 1) {  // F3(1) = -F3(2): D = ... + 2*F3(2); the flux stored for face 1 is -F3(2)
    flux_adj(R(2) * lD - m3, x, psi.ld(i, j, k + 1), P.u3.ld(i, j, k + 1), true, A.lx, i, j, k, true, i, j, k + 1,
             &lu);
    addat(A.gu3, i, j, k + 1, lu);
  } else if (!IN && !g.bz && k == g.lp) {  // F3(lp+1) = -F3(lp): D = ... - 2*F3(lp); face lp+1 stores -F3(lp)
    flux_adj(-R(2) * lD + m3 - m3p, psi.ld(i, j, k - 1), x, P.u3.ld(i, j, k), true, A.lx, i, j, k - 1, true, i, j,
             k, &lu);
    addat(A.gu3, i, j, k, lu);
  } else {
    const int kp = cz<IN>(g, k + 1), km = cz<IN>(g, k - 1);
    flux_adj(lD + m3p, x, psi.ld(i, j, kp), fz<R, true, IN>(g, P.u3, i, j, k + 1), true, A.lx, i, j, k, true, i,
             j, kp, &lu);
    fz_add<R, true, IN>(g, A.gu3, i, j, k + 1, lu);
    flux_adj(-lD + m3, psi.ld(i, j, km), x, P.u3.ld(i, j, k), true, A.lx, i, j, km, true, i, j, k, &lu);
    fz_add<R, true, IN>(g, A.gu3, i, j, k, lu);
  }
}
template <class R, bool MF = false>
__global__ void KA_LB_UPWIND ka_upwind(const Prob<R> P, const AdjArr<R> A) {
#define C(IN) ka_upwind_cell<R, IN, MF>(P, A, i, j, k)
  ADISPATCH(C)
#undef C
}

// Density step: the mass flux of every face adds the last pass's limited
// flux as the forward reads it (fx/fy/fz of the stored faces: the periodic
// wrap, the zero open walls, the mirrored z faces), so its cotangent goes to
// that flux's adjoint through the same read maps.
template <class R>
__global__ void __launch_bounds__(128) ka_mass_to_w(const Prob<R> P, const AdjArr<R> A) {
  ACELL
  fx_add<R, false>(g, A.lw1, i, j, k, A.lm1.ld(i, j, k));
  fy_add<R, false>(g, A.lw2, i, j, k, A.lm2.ld(i, j, k));
  fz_add<R, false>(g, A.lw3, i, j, k, A.lm3.ld(i, j, k));
  if (i == g.np) fx_add<R, false>(g, A.lw1, g.np + 1, j, k, A.lm1.ld(g.np + 1, j, k));
  if (j == g.mp) fy_add<R, false>(g, A.lw2, i, g.mp + 1, k, A.lm2.ld(i, g.mp + 1, k));
  if (k == g.lp) fz_add<R, false>(g, A.lw3, i, j, g.lp + 1, A.lm3.ld(i, j, g.lp + 1));
}

// Reverse of the density step's outputs (rho_out_body): x_incomp = x*h,
// pexr1 = x_incomp*pexe, pexr2 = x_incomp, rhr = rhoadv/x_incomp with rhoadv
// the x_incomp input.  lam (dJ/dpsi after the step) gains h*dJ/dx_incomp;
// g_xinc and g_pexe receive dJ/d(x_incomp input) and dJ/dpexe.  Null
// cotangent arrays are zeros.
template <class R>
__global__ void __launch_bounds__(128) ka_rho_out(const Prob<R> P, const Arr<R> out, const Arr<R> lxc,
                                                  const Arr<R> lp1, const Arr<R> lp2, const Arr<R> lrh, Arr<R> lam,
                                                  Arr<R> g_xinc, Arr<R> g_pexe) {
  ACELL
  (void)g;
  const R h = P.h.ld(i, j, k);
  const R xc = out.ld(i, j, k) * h;
  const R pe = P.pexe.ld(i, j, k), ra = P.x_incomp.ld(i, j, k);
  const R a_xc = lxc.p ? lxc.ld(i, j, k) : R(0), a_p1 = lp1.p ? lp1.ld(i, j, k) : R(0),
          a_p2 = lp2.p ? lp2.ld(i, j, k) : R(0), a_rh = lrh.p ? lrh.ld(i, j, k) : R(0);
  const R l_xc = a_xc + a_p1 * pe + a_p2 - a_rh * (ra / xc) / xc;
  lam.at(i, j, k) = lam.ld(i, j, k) + l_xc * h;
  g_xinc.at(i, j, k) = a_rh / xc;
  g_pexe.at(i, j, k) = a_p1 * xc;
}

template <class R>
__global__ void __launch_bounds__(128) ka_store(const Prob<R> P, const AdjArr<R> A) {
  ACELL
  A.lam.at(i, j, k) = A.lx.ld(i, j, k);
}

// J's seed: lambda = psi_N - target on the interior, 0 on the halo.
template <class R>
__global__ void __launch_bounds__(128) ka_seed(const Prob<R> P, const Arr<R> psi, const Arr<R> target, Arr<R> lam) {
  ACELL
  lam.at(i, j, k) = psi.ld(i, j, k) - target.ld(i, j, k);
}

// forward record kernels (psi's halo is left untouched: HALO=false); warps
// away from every wall take the bodies without boundary maps, as the
// forward stage kernels do
#define FCELL(BODY)                                          \
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;  \
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;  \
  const int k = blockIdx.z + 1;                              \
  const bool win = warp_interior(P.g, i, j, k);              \
  if (i > P.g.np || j > P.g.mp) return;                      \
  if (win) {                                                 \
    BODY(true);                                              \
  } else {                                                   \
    BODY(false);                                             \
  }
// As FCELL, with the unit-density instantiation BODY(IN, U) for interior
// warps whose densities are all exactly 1 (FP64).
#define FCELL_U(BODY)                                        \
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;  \
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;  \
  const int k = blockIdx.z + 1;                              \
  const bool win = warp_interior(P.g, i, j, k);              \
  if (i > P.g.np || j > P.g.mp) return;                      \
  if (!win) {                                                \
    BODY(false, false);                                      \
  } else if (warp_unit_cell(P, i, j, k)) {                   \
    BODY(true, true);                                        \
  } else {                                                   \
    BODY(true, false);                                       \
  }
template <class R>
__global__ void __launch_bounds__(128, (KfMinBlocks<R, 8, 10>::v)) kf_upwind(const Prob<R> P) {
#define B(IN, U) upwind_body<R, true, false, IN, U>(P, i, j, k)
  FCELL_U(B)
#undef B
}
template <class R, bool AIN, bool PV>
__global__ void __launch_bounds__(128) kf_pairs(const Prob<R> P) {
  ACELL
  (void)g;
  pairs_body<R, AIN, PV>(P, i, j, k);
}
// the forward stage's dispatch: unit face densities and pair sums (FP64),
// and the stage kernel's seven resident blocks per SM for FP64
template <class R>
struct KfPseudoMinBlocks {
  static constexpr int v = sizeof(R) == 8 ? 7 : 1;
};
template <class R, bool AIN>
__global__ void __launch_bounds__(128, KfPseudoMinBlocks<R>::v) kf_pseudo(const Prob<R> P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  const bool win = warp_interior(P.g, i, j, k);
  bool pin = false;
  if constexpr (sizeof(R) == 8)
    if (!win && P.pairs == 2) pin = warp_on_grid(P.g, i, j);
  if (i > P.g.np || j > P.g.mp) return;
  if (!win) {
    if constexpr (sizeof(R) == 8) {
      if (pin) {
        if (warp_unit_faces(P, i, j, k))
          pseudo_body<R, AIN, false, true, true, false, true, true>(P, i, j, k);
        else
          pseudo_body<R, AIN, false, false, true, false, true, true>(P, i, j, k);
        return;
      }
    }
    pseudo_body<R, AIN, false>(P, i, j, k);
  } else if constexpr (sizeof(R) == 8) {
    const bool unit = warp_unit_faces(P, i, j, k);
    if (P.pairs == 2) {
      if (unit)
        pseudo_body<R, AIN, true, true, true, false, true, true>(P, i, j, k);
      else
        pseudo_body<R, AIN, true, false, true, false, true, true>(P, i, j, k);
    } else if (P.pairs) {
      if (unit)
        pseudo_body<R, AIN, true, true, true>(P, i, j, k);
      else
        pseudo_body<R, AIN, true, false, true>(P, i, j, k);
    } else {
      if (unit)
        pseudo_body<R, AIN, true, true>(P, i, j, k);
      else
        pseudo_body<R, AIN, true>(P, i, j, k);
    }
  } else {
    pseudo_body<R, AIN, true>(P, i, j, k);
  }
}
// Ratios of at least 1 are recorded as RATIO_CAP (lim_ratio): the reverse
// limiter's min3 selects neither form, and the reverse bounds kernel
// recomputes its quotients from the recorded extrema and fluxes.
template <class R, bool NONOS, bool FIRST, bool KEEP>
__global__ void __launch_bounds__(128, (KfMinBlocks<R, 12, 12>::v)) kf_bounds(const Prob<R> P) {
  if constexpr (NONOS && sizeof(R) == 8) {  // FP32: per-lane quotients are cheaper than the barriers
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    const bool win = warp_interior(P.g, i, j, k);
    const bool valid = i <= P.g.np && j <= P.g.mp;
    RatioOps<R> r{};
    if (valid) {
      if (!win)
        r = bounds_body<R, true, FIRST, KEEP, false, 2>(P, i, j, k);
      else if (warp_unit_cell(P, i, j, k))
        r = bounds_body<R, true, FIRST, KEEP, true, 2, true>(P, i, j, k);
      else
        r = bounds_body<R, true, FIRST, KEEP, true, 2>(P, i, j, k);
    }
    block_ratios(P, i, j, k, valid, r);
  } else {
#define B(IN, U) bounds_body<R, NONOS, FIRST, KEEP, IN, 1, U>(P, i, j, k)
    FCELL_U(B)
#undef B
  }
}
template <class R, bool NONOS>
__global__ void __launch_bounds__(128, (KfMinBlocks<R, 16, 16>::v)) kf_limit(const Prob<R> P) {
#define B(IN) limit_body<R, NONOS, IN>(P, i, j, k)
  FCELL(B)
#undef B
}
template <class R>
__global__ void __launch_bounds__(128) kf_update(const Prob<R> P) {
#define B(IN, U) update_body<R, false, IN, U>(P, i, j, k)
  FCELL_U(B)
#undef B
}
#undef FCELL
#undef FCELL_U

// The values of pass t: its input field, pseudo-velocities, ratios and
// extrema from the records; `a` selects the "a" velocities the pass's
// pseudo-velocity read (the previous pass's limited ones) or its own
// limited velocities (for the limiter's forward).
template <class R>
Prob<R> pass_prob(const Prob<R>& P, const AdjPlan<R>& A, int t, bool prev_w) {
  Prob<R> Q = P;
  Q.xant = A.x[t];
  Q.v1 = A.v[t][0];
  Q.v2 = A.v[t][1];
  Q.v3 = A.v[t][2];
  Q.cp = A.cp[t];
  Q.cn = A.cn[t];
  Q.mx = A.mx[t];
  Q.mn = A.mn[t];
  Q.q = A.q[t];
  Q.f1 = A.fns[t][0];  // standard form: the unlimited donor fluxes of the pass
  Q.f2 = A.fns[t][1];
  Q.f3 = A.fns[t][2];
  const int tw = prev_w ? (t > 0 ? t - 1 : 0) : t;
  Q.w1 = A.w[tw][0];
  Q.w2 = A.w[tw][1];
  Q.w3 = A.w[tw][2];
  return Q;
}

// The forward records of one step (every pass's input field, velocities,
// ratios and extrema) into A's record arrays.  out: when given, the last
// pass's update also writes the step's output field there (interior cells),
// so that a checkpointed reverse sweep rebuilds a segment and records it in
// one pass.
template <class R>
int run_step_record(const Prob<R>& P, const AdjPlan<R>& A, int nonos, const Arr<R>* out, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 grd((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  const int np_ = A.npass;
  const bool keep = np_ > 1;
  const size_t ncell = (size_t)g.np * g.mp * g.lp;
  int n = 0;
  Prob<R> F = P;
  F.xant = A.x[0];
  kf_upwind<R><<<grd, blk, 0, s>>>(F);
  n++;
  for (int t = 0; t < np_; t++) {
    Prob<R> Qa = pass_prob(P, A, t, true);
    // FP64 gauge: pair sums of the pass's input field into its cp/cn/q
    // records, which the bounds kernel fills afterwards, and the velocity
    // pairs into the workspace's f1..f3 (unused by the gauge form)
    Qa.pairs = (!P.stdf && sizeof(R) == 8) ? 2 : 0;
    if (Qa.pairs) {
      Qa.f1 = P.f1;
      Qa.f2 = P.f2;
      Qa.f3 = P.f3;
      if (t == 0) kf_pairs<R, true, true><<<grd, blk, 0, s>>>(Qa);
      else kf_pairs<R, false, true><<<grd, blk, 0, s>>>(Qa);
      n++;
    }
    if (t == 0) kf_pseudo<R, true><<<grd, blk, 0, s>>>(Qa);
    else kf_pseudo<R, false><<<grd, blk, 0, s>>>(Qa);
    const Prob<R> Q = pass_prob(P, A, t, false);
    if (nonos && keep && t > 0) {  // the running extrema continue from the previous pass
      if (cudaMemcpyAsync(A.mx[t].p, A.mx[t - 1].p, ncell * sizeof(R), cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
          cudaMemcpyAsync(A.mn[t].p, A.mn[t - 1].p, ncell * sizeof(R), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return -5;
    }
    if (!nonos) kf_bounds<R, false, true, false><<<grd, blk, 0, s>>>(Q);
    else if (!keep) kf_bounds<R, true, true, false><<<grd, blk, 0, s>>>(Q);
    else if (t == 0) kf_bounds<R, true, true, true><<<grd, blk, 0, s>>>(Q);
    else kf_bounds<R, true, false, true><<<grd, blk, 0, s>>>(Q);
    // the limited fluxes (standard form) go to the workspace scratch: only
    // the update reads them
    Prob<R> L = Q;
    L.f1 = P.f1;
    L.f2 = P.f2;
    L.f3 = P.f3;
    if (nonos) kf_limit<R, true><<<grd, blk, 0, s>>>(L);
    else kf_limit<R, false><<<grd, blk, 0, s>>>(L);
    n += 3;
    if (t < np_ - 1 || out) {
      Prob<R> U = L;
      U.xant = t < np_ - 1 ? A.x[t + 1] : *out;
      kf_update<R><<<grd, blk, 0, s>>>(U);
      n++;
    }
  }
  add_launches(n);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

// The reverse kernels of one recorded step: lambda of the step's output (A.lam)
// becomes lambda of its input; the velocity gradients accumulate into A.gu*.
template <class R>
int run_step_reverse(const Prob<R>& P, const AdjPlan<R>& A, int nonos, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 grd((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  const int np_ = A.npass;
  int n = 0;
  if (cudaMemsetAsync(A.acc, 0, A.acc_elems * sizeof(R), s) != cudaSuccess) return -5;
  if (A.rho && A.lm1.p) {  // the density step's mass fluxes read the last pass's limited fluxes
    AdjArr<R> m{};
    m.lw1 = A.lw[np_ - 1][0];
    m.lw2 = A.lw[np_ - 1][1];
    m.lw3 = A.lw[np_ - 1][2];
    m.lm1 = A.lm1;
    m.lm2 = A.lm2;
    m.lm3 = A.lm3;
    ka_mass_to_w<R><<<grd, blk, 0, s>>>(P, m);
    n++;
  }
  // ---- reverse, last pass first
  for (int t = np_ - 1; t >= 0; t--) {
    if (t < np_ - 1 && cudaMemsetAsync(A.pass_acc, 0, A.pass_acc_elems * sizeof(R), s) != cudaSuccess) return -5;
    const Prob<R> Q = pass_prob(P, A, t, true);
    AdjArr<R> a{};
    a.lxant = A.lx[t];
    a.lv1 = A.lv[0];
    a.lv2 = A.lv[1];
    a.lv3 = A.lv[2];
    a.lw1 = A.lw[t][0];
    a.lw2 = A.lw[t][1];
    a.lw3 = A.lw[t][2];
    a.lcp = A.lcp;
    a.lcn = A.lcn;
    a.lx = A.lxin;
    a.lam = t == np_ - 1 ? A.lam : A.lx[t + 1];
    a.gu1 = A.gu1;
    a.gu2 = A.gu2;
    a.gu3 = A.gu3;
    a.la1 = t == 0 ? A.gu1 : A.lw[t - 1][0];
    a.la2 = t == 0 ? A.gu2 : A.lw[t - 1][1];
    a.la3 = t == 0 ? A.gu3 : A.lw[t - 1][2];
    a.lmx = A.lmx[t];
    a.lmn = A.lmn[t];
    a.lmxp = A.lmx[t > 0 ? t - 1 : 0];
    a.lmnp = A.lmn[t > 0 ? t - 1 : 0];
    a.mxp = A.mx[t > 0 ? t - 1 : 0];
    a.mnp = A.mn[t > 0 ? t - 1 : 0];
    a.lg1 = A.lg[0];
    a.lg2 = A.lg[1];
    a.lg3 = A.lg[2];
    a.lf1 = A.lf[0];
    a.lf2 = A.lf[1];
    a.lf3 = A.lf[2];
    a.lq = A.lq;
    if (P.stdf) {
      ka_update_std<R><<<grd, blk, 0, s>>>(Q, a);
      if (nonos) {
        ka_limit_std<R, true><<<grd, blk, 0, s>>>(Q, a);
        if (t == 0) ka_bounds<R, true, true><<<grd, blk, 0, s>>>(Q, a);
        else ka_bounds<R, false, true><<<grd, blk, 0, s>>>(Q, a);
        n++;
      } else {
        ka_limit_std<R, false><<<grd, blk, 0, s>>>(Q, a);
      }
      if (t == 0) ka_pseudo_std<R, true><<<grd, blk, 0, s>>>(Q, a);
      else ka_pseudo_std<R, false><<<grd, blk, 0, s>>>(Q, a);
    } else {
      ka_update<R><<<grd, blk, 0, s>>>(Q, a);
      if (nonos) {
        ka_limit<R, true><<<grd, blk, 0, s>>>(Q, a);
        if (t == 0) ka_bounds<R, true, false><<<grd, blk, 0, s>>>(Q, a);
        else ka_bounds<R, false, false><<<grd, blk, 0, s>>>(Q, a);
        n++;
      } else {
        ka_limit<R, false><<<grd, blk, 0, s>>>(Q, a);
      }
      // the pass's cp/cn/q records are dead once the reverse bounds ran:
      // they take the pair sums of its input field, and the workspace's
      // f1..f3 the velocity pairs (FP64)
      Prob<R> Qp = Q;
      Qp.pairs = 2;
      if (Qp.pairs) {
        Qp.f1 = P.f1;
        Qp.f2 = P.f2;
        Qp.f3 = P.f3;
        if (t == 0) kf_pairs<R, true, true><<<grd, blk, 0, s>>>(Qp);
        else kf_pairs<R, false, true><<<grd, blk, 0, s>>>(Qp);
        n++;
      }
      if (t == 0) ka_pseudo<R, true><<<grd, blk, 0, s>>>(Qp, a);
      else ka_pseudo<R, false><<<grd, blk, 0, s>>>(Qp, a);
    }
    n += 3;
  }
  AdjArr<R> a0{};
  a0.lxant = A.lx[0];
  a0.lx = A.lxin;
  a0.gu1 = A.gu1;
  a0.gu2 = A.gu2;
  a0.gu3 = A.gu3;
  a0.lam = A.lam;
  if (A.rho && A.lm1.p) {
    a0.lm1 = A.lm1;
    a0.lm2 = A.lm2;
    a0.lm3 = A.lm3;
    ka_upwind<R, true><<<grd, blk, 0, s>>>(P, a0);
  } else {
    ka_upwind<R><<<grd, blk, 0, s>>>(P, a0);
  }
  ka_store<R><<<grd, blk, 0, s>>>(P, a0);
  n += 2;
  add_launches(n);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template <class R>
int run_step_adjoint(const Prob<R>& P, const AdjPlan<R>& A, int nonos, cudaStream_t s) {
  const int rc = run_step_record<R>(P, A, nonos, nullptr, s);
  return rc ? rc : run_step_reverse<R>(P, A, nonos, s);
}

template <class R>
int run_rho_out_adjoint(const Prob<R>& P, const Arr<R>& out, const Arr<R>& lxc, const Arr<R>& lp1,
                        const Arr<R>& lp2, const Arr<R>& lrh, const Arr<R>& lam, const Arr<R>& g_xinc,
                        const Arr<R>& g_pexe, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 grd((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  ka_rho_out<R><<<grd, blk, 0, s>>>(P, out, lxc, lp1, lp2, lrh, lam, g_xinc, g_pexe);
  add_launches(1);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template <class R>
int run_seed(const Prob<R>& P, const Arr<R>& psi, const Arr<R>& target, const Arr<R>& lam, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 grd((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  ka_seed<R><<<grd, blk, 0, s>>>(P, psi, target, lam);
  add_launches(1);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template int run_step_adjoint<double>(const Prob<double>&, const AdjPlan<double>&, int, cudaStream_t);
template int run_step_adjoint<float>(const Prob<float>&, const AdjPlan<float>&, int, cudaStream_t);
template int run_step_record<double>(const Prob<double>&, const AdjPlan<double>&, int, const Arr<double>*,
                                     cudaStream_t);
template int run_step_record<float>(const Prob<float>&, const AdjPlan<float>&, int, const Arr<float>*,
                                    cudaStream_t);
template int run_step_reverse<double>(const Prob<double>&, const AdjPlan<double>&, int, cudaStream_t);
template int run_step_reverse<float>(const Prob<float>&, const AdjPlan<float>&, int, cudaStream_t);
template int run_rho_out_adjoint<double>(const Prob<double>&, const Arr<double>&, const Arr<double>&,
                                         const Arr<double>&, const Arr<double>&, const Arr<double>&,
                                         const Arr<double>&, const Arr<double>&, const Arr<double>&, cudaStream_t);
template int run_rho_out_adjoint<float>(const Prob<float>&, const Arr<float>&, const Arr<float>&, const Arr<float>&,
                                        const Arr<float>&, const Arr<float>&, const Arr<float>&, const Arr<float>&,
                                        const Arr<float>&, cudaStream_t);
template int run_seed<double>(const Prob<double>&, const Arr<double>&, const Arr<double>&, const Arr<double>&, cudaStream_t);
template int run_seed<float>(const Prob<float>&, const Arr<float>&, const Arr<float>&, const Arr<float>&, cudaStream_t);

}  // namespace mpdata
