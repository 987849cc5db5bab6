// CPU oracle for the MPDATA advection step — TEST INFRASTRUCTURE ONLY.
// See mpdata_oracle.h for scope, pinning and conventions.  Built with
// -O2 -ffp-contract=off (no FMA contraction) so every expression rounds
// exactly as written, in the reference's left-to-right order.
#include "mpdata_oracle.h"

#include <cmath>
#include <limits>
#include <algorithm>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

int g_threads = 1;

// Fortran-ordered 3-D view with lower bound `lo` on every axis.
template <class R>
struct V3 {
  R* p;
  int lo;
  long sj, sk;
  inline R& operator()(int i, int j, int k) const {
    return p[(long)(i - lo) + (long)(j - lo) * sj + (long)(k - lo) * sk];
  }
};
template <class R>
inline V3<R> view(R* p, int ih, int n0, int n1) {
  return V3<R>{p, 1 - ih, (long)n0, (long)n0 * n1};
}

// Owned array with a 1-cell shell, extents (n0,n1,n2) including the shell.
template <class R>
struct Buf {
  std::vector<R> d;
  V3<R> v;
  Buf(int n0, int n1, int n2) : d((size_t)n0 * n1 * n2, R(0)) { v = view<R>(d.data(), 1, n0, n1); }
  inline R& operator()(int i, int j, int k) { return v(i, j, k); }
};

// abs and sign bit, generic so the step can also run on the AD scalar below
inline double absv(double x) { return std::fabs(x); }
inline float absv(float x) { return std::fabs(x); }
inline bool sgnb(double x) { return std::signbit(x); }
inline bool sgnb(float x) { return std::signbit(x); }

// ---- reverse-mode AD scalar (for the un-checkpointed FP64 adjoint) --------
// Every arithmetic result is a tape node with up to two parents and the
// local partial derivatives; branches (max/min/pp/pn/abs/sign) follow the
// forward values, so the derivative is taken piecewise at the forward branch.
struct Tape {
  std::vector<int> a, b;
  std::vector<double> da, db;
  int push(int ia, double pa, int ib, double pb) {
    a.push_back(ia); da.push_back(pa); b.push_back(ib); db.push_back(pb);
    return (int)a.size() - 1;
  }
};
Tape* g_tape = nullptr;
struct AD {
  double v;
  int id;  // < 0: constant
  AD() : v(0.0), id(-1) {}
  AD(double x) : v(x), id(-1) {}
};
inline AD mk(double v, int ia, double pa, int ib, double pb) {
  AD r(v);
  if (ia >= 0 || ib >= 0) r.id = g_tape->push(ia, pa, ib, pb);
  return r;
}
inline AD operator+(AD x, AD y) { return mk(x.v + y.v, x.id, 1.0, y.id, 1.0); }
inline AD operator-(AD x, AD y) { return mk(x.v - y.v, x.id, 1.0, y.id, -1.0); }
inline AD operator*(AD x, AD y) { return mk(x.v * y.v, x.id, y.v, y.id, x.v); }
inline AD operator/(AD x, AD y) {
  const double q = x.v / y.v;
  return mk(q, x.id, 1.0 / y.v, y.id, -q / y.v);
}
inline AD operator-(AD x) { return mk(-x.v, x.id, -1.0, -1, 0.0); }
inline bool operator>(AD x, AD y) { return x.v > y.v; }
inline bool operator<(AD x, AD y) { return x.v < y.v; }
inline AD absv(AD x) { return std::signbit(x.v) ? -x : x; }
inline bool sgnb(AD x) { return std::signbit(x.v); }

// ---- point operators: mpdataoperators.inc:50-96 (device versions) ----
template <class R> inline R pp(R y) { return y > R(0) ? y : R(0); }        // max(0,y)
template <class R> inline R pn(R y) { return y < R(0) ? -y : R(0); }       // -min(0,y)
template <class R> inline R mx2(R a, R b) { return a > b ? a : b; }
template <class R> inline R mn2(R a, R b) { return a < b ? a : b; }
template <class R> inline R donor(R y1, R y2, R a) { return pp(a) * y1 - pn(a) * y2; }
// vdyf: (abs(a)-a*a*rinv)*(x2-x1)*.5                            (:65-69)
template <class R> inline R vdyf(R x1, R x2, R a, R rinv) {
  return (absv(a) - a * a * rinv) * (x2 - x1) * R(0.5);
}
// rat4: ((z3+z2)-(z1+z0))*.25                                    (:80-84)
template <class R> inline R rat4(R z0, R z1, R z2, R z3) { return ((z3 + z2) - (z1 + z0)) * R(0.25); }
// vdyfa: (abs(a)-a*a*rinv)*(abs(x2)-abs(x1))/(abs(x2)+abs(x1)+ep) (:85-91)
template <class R> inline R vdyfa(R x1, R x2, R a, R rinv, R ep) {
  return (absv(a) - a * a * rinv) * (absv(x2) - absv(x1)) /
         (absv(x2) + absv(x1) + ep);
}
// vcorra: -0.125*a*b*y1*rinv/(y2)                                 (:92-96)
template <class R> inline R vcorra(R a, R b, R y1, R y2, R rinv) {
  return -(R(0.125) * a * b * y1 * rinv / y2);
}
// pp(sign(1,x)): 1 when x carries a + sign (IEEE signed zero aware), else 0
template <class R> inline R possign(R x) { return sgnb(x) ? R(0) : R(1); }

struct Dims {
  int np, mp, lp, ih;
  int bx, by, bz;  // 1 = periodic on that axis
};

// Periodic wrap of a 1-shell array along each periodic axis.  `fx/fy/fz` tell
// whether the array is face-centred along that axis (extent n+3, faces 0..n+2,
// face n+1 == face 1) or cell-centred (extent n+2, cells 0..n+1).
template <class R>
void wrap(Buf<R>& A, const Dims& d, bool fx, bool fy, bool fz) {
  const int n0 = d.np + (fx ? 3 : 2), n1 = d.mp + (fy ? 3 : 2), n2 = d.lp + (fz ? 3 : 2);
  if (d.by) {
    for (int k = 0; k < n2; k++)
      for (int i = 0; i < n0; i++) {
        A(i, 0, k) = A(i, d.mp, k);
        A(i, d.mp + 1, k) = A(i, 1, k);
        if (fy) A(i, d.mp + 2, k) = A(i, 2, k);
      }
  }
  if (d.bx) {
    for (int k = 0; k < n2; k++)
      for (int j = 0; j < n1; j++) {
        A(0, j, k) = A(d.np, j, k);
        A(d.np + 1, j, k) = A(1, j, k);
        if (fx) A(d.np + 2, j, k) = A(2, j, k);
      }
  }
  if (d.bz) {
    for (int j = 0; j < n1; j++)
      for (int i = 0; i < n0; i++) {
        A(i, j, 0) = A(i, j, d.lp);
        A(i, j, d.lp + 1) = A(i, j, 1);
        if (fz) A(i, j, d.lp + 2) = A(i, j, 2);
      }
  }
}

// xant-style halo: cp_scnd_last_to_halo_xy_fulld (mpdataoperators.inc:479-513):
// y walls first, then x walls, over the full halo range; periodic axes wrap.
template <class R>
void halo_second_last(Buf<R>& A, const Dims& d) {
  for (int k = 0; k <= d.lp + 1; k++)
    for (int i = 0; i <= d.np + 1; i++) {
      if (d.by) { A(i, 0, k) = A(i, d.mp, k); A(i, d.mp + 1, k) = A(i, 1, k); }
      else { A(i, 0, k) = A(i, 2, k); A(i, d.mp + 1, k) = A(i, d.mp - 1, k); }
    }
  for (int k = 0; k <= d.lp + 1; k++)
    for (int j = 0; j <= d.mp + 1; j++) {
      if (d.bx) { A(0, j, k) = A(d.np, j, k); A(d.np + 1, j, k) = A(1, j, k); }
      else { A(0, j, k) = A(2, j, k); A(d.np + 1, j, k) = A(d.np - 1, j, k); }
    }
  if (d.bz)
    for (int j = 0; j <= d.mp + 1; j++)
      for (int i = 0; i <= d.np + 1; i++) { A(i, j, 0) = A(i, j, d.lp); A(i, j, d.lp + 1) = A(i, j, 1); }
}

// x_in halo for the limiter bounds: cp_last_to_halo_xy (mpdataoperators.inc:551-584)
// zero-gradient copy on open x/y walls; periodic axes wrap.
template <class R>
void halo_last(Buf<R>& A, const Dims& d) {
  for (int k = 0; k <= d.lp + 1; k++)
    for (int i = 0; i <= d.np + 1; i++) {
      if (d.by) { A(i, 0, k) = A(i, d.mp, k); A(i, d.mp + 1, k) = A(i, 1, k); }
      else { A(i, 0, k) = A(i, 1, k); A(i, d.mp + 1, k) = A(i, d.mp, k); }
    }
  for (int k = 0; k <= d.lp + 1; k++)
    for (int j = 0; j <= d.mp + 1; j++) {
      if (d.bx) { A(0, j, k) = A(d.np, j, k); A(d.np + 1, j, k) = A(1, j, k); }
      else { A(0, j, k) = A(1, j, k); A(d.np + 1, j, k) = A(d.np, j, k); }
    }
  if (d.bz)
    for (int j = 0; j <= d.mp + 1; j++)
      for (int i = 0; i <= d.np + 1; i++) { A(i, j, 0) = A(i, j, d.lp); A(i, j, d.lp + 1) = A(i, j, 1); }
}

// cp/cn halo: zero_halo_xyd (mpdataoperators.inc:1034-1063) on open walls.
template <class R>
void halo_zero_or_wrap(Buf<R>& A, const Dims& d) {
  for (int k = 0; k <= d.lp + 1; k++)
    for (int i = 0; i <= d.np + 1; i++) {
      if (d.by) { A(i, 0, k) = A(i, d.mp, k); A(i, d.mp + 1, k) = A(i, 1, k); }
      else { A(i, 0, k) = R(0); A(i, d.mp + 1, k) = R(0); }
    }
  for (int k = 0; k <= d.lp + 1; k++)
    for (int j = 0; j <= d.mp + 1; j++) {
      if (d.bx) { A(0, j, k) = A(d.np, j, k); A(d.np + 1, j, k) = A(1, j, k); }
      else { A(0, j, k) = R(0); A(d.np + 1, j, k) = R(0); }
    }
  if (d.bz)
    for (int j = 0; j <= d.mp + 1; j++)
      for (int i = 0; i <= d.np + 1; i++) { A(i, j, 0) = A(i, j, d.lp); A(i, j, d.lp + 1) = A(i, j, 1); }
}

// Boundary rule on a face-centred field: open x/y walls zero the wall faces
// (flux_x_bcd / flux_y_bcd type 0, mpdataoperators.inc:673-811); z walls mirror
// (flux_z_bc_nohalod type 2, :903-947); periodic axes wrap (face n+1 == face 1).
template <class R>
void face_bc(Buf<R>& F, const Dims& d, int axis) {
  if (axis == 0) {
    if (!d.bx)
      for (int k = 1; k <= d.lp; k++)
        for (int j = 1; j <= d.mp; j++) { F(1, j, k) = R(0); F(d.np + 1, j, k) = R(0); }
    wrap(F, d, true, false, false);
  } else if (axis == 1) {
    if (!d.by)
      for (int k = 1; k <= d.lp; k++)
        for (int i = 1; i <= d.np; i++) { F(i, 1, k) = R(0); F(i, d.mp + 1, k) = R(0); }
    wrap(F, d, false, true, false);
  } else {
    if (!d.bz)
      for (int j = 1; j <= d.mp; j++)
        for (int i = 1; i <= d.np; i++) { F(i, j, 1) = -F(i, j, 2); F(i, j, d.lp + 1) = -F(i, j, d.lp); }
    wrap(F, d, false, false, true);
  }
}

// Copy a caller C-grid array into a 1-shell face buffer (interior faces only;
// on periodic axes face n+1 is taken from face 1).
template <class R>
void load_face(Buf<R>& F, const R* src, const Dims& d, int axis) {
  const int ih = d.ih;
  const int n0 = d.np + 2 * ih + (axis == 0), n1 = d.mp + 2 * ih + (axis == 1);
  V3<R> S = view<R>(const_cast<R*>(src), ih, n0, n1);
  const int ie = d.np + (axis == 0 && !d.bx), je = d.mp + (axis == 1 && !d.by),
            ke = d.lp + (axis == 2 && !d.bz);
  for (int k = 1; k <= ke; k++)
    for (int j = 1; j <= je; j++)
      for (int i = 1; i <= ie; i++) F(i, j, k) = S(i, j, k);
  wrap(F, d, axis == 0, axis == 1, axis == 2);
}

template <class R>
void load_cell(Buf<R>& C, const R* src, const Dims& d) {
  V3<R> S = view<R>(const_cast<R*>(src), d.ih, d.np + 2 * d.ih, d.mp + 2 * d.ih);
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) C(i, j, k) = S(i, j, k);
  wrap(C, d, false, false, false);
}

// ---- upwind3d_gpubc (upwind3d-gpubc.f90:101-198) ----
// xin: psi with its halo already set (putbcinxh / periodic wrap).
template <class R>
void upwind(const Dims& d, Buf<R>& xin, Buf<R>& u1, Buf<R>& u2, Buf<R>& u3, Buf<R>& h,
            Buf<R>& rhr, Buf<R>& xant) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        const R hinv = R(1) / h(i, j, k);
        const R x = xin(i, j, k);
        const R f1p = donor(x, xin(i + 1, j, k), u1(i + 1, j, k));
        const R f1 = donor(xin(i - 1, j, k), x, u1(i, j, k));
        const R f2p = donor(x, xin(i, j + 1, k), u2(i, j + 1, k));
        const R f2 = donor(xin(i, j - 1, k), x, u2(i, j, k));
        R f3p, f3;
        if (!d.bz && k == 1) {  // :134-135  f3(k) = -f3(k+1)
          f3p = donor(x, xin(i, j, k + 1), u3(i, j, k + 1));
          f3 = -f3p;
        } else if (!d.bz && k == d.lp) {  // :164-165  f3(k+1) = -f3(k)
          f3 = donor(xin(i, j, k - 1), x, u3(i, j, k));
          f3p = -f3;
        } else {
          f3p = donor(x, xin(i, j, k + 1), u3(i, j, k + 1));
          f3 = donor(xin(i, j, k - 1), x, u3(i, j, k));
        }
        xant(i, j, k) = rhr(i, j, k) * (x - (f1p - f1 + f2p - f2 + f3p - f3) * hinv);
      }
}

// The 4-face velocity sums of the cross terms (u2(i-1,j)+u2(i-1,j+1)+u2(i,j+1)
// +u2(i,j) and its five siblings) carry no parentheses in the reference, and
// Fortran may evaluate an unparenthesised sum in any mathematically equivalent
// order; the reference's own builds reassociate (-Ofast, -O3, CMakeLists.txt:
// 64-76).  This restatement fixes one order: the sum of two cell-centred pairs,
// (a(c) + a(c+e)) + (a(c') + a(c'+e)), lower cell first, where a(c)+a(c+e) is
// the cell's pair of faces along the velocity's own axis.  Every sum of the
// pass then shares those pairs.

// Literal mode (orc_set_literal_sums): the six sums are evaluated left to
// right in the order the reference writes their terms, ((t1+t2)+t3)+t4,
// which is the order an unoptimised Fortran build takes.  It exists to
// measure how far the fixed pair order moves a field; the default (0) is the
// pair order that the CUDA kernels reproduce bit for bit.
int g_literal_sums = 0;
// t1..t4 in the reference's written order.  s12: the pair form is
// (t1+t2)+(t3+t4); s14: the pair form is (t1+t4)+(t2+t3).
template <class R> inline R s12(R t1, R t2, R t3, R t4) {
  return g_literal_sums ? ((t1 + t2) + t3) + t4 : (t1 + t2) + (t3 + t4);
}
template <class R> inline R s14(R t1, R t2, R t3, R t4) {
  return g_literal_sums ? ((t1 + t2) + t3) + t4 : (t1 + t4) + (t2 + t3);
}

// Whether plane k carries the z cross terms in the x/y pseudo-velocities:
// the reference's k=1 and k=lp kernels drop them (antidiff3d-*-gpubc.f90).
inline bool zterm(const Dims& d, int k) { return d.bz || (k > 1 && k < d.lp); }

// ---- pseudo-velocities, standard form (antidiff3d-standard-gpubc.f90:72-203) ----
template <class R>
void pseudo_std(const Dims& d, Buf<R>& x, Buf<R>& a1, Buf<R>& a2, Buf<R>& a3, Buf<R>& h,
                Buf<R>& v1, Buf<R>& v2, Buf<R>& v3, Buf<R>& f1, Buf<R>& f2, Buf<R>& f3, R ep) {
  const int i0 = d.bx ? 1 : 2, j0 = d.by ? 1 : 2, k0 = d.bz ? 1 : 2;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++) {
    const bool zt = zterm(d, k);
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        if (i >= i0) {
          const R hmx = R(1) / (R(0.5) * (h(i - 1, j, k) + h(i, j, k)));
          R v = vdyfa(x(i - 1, j, k), x(i, j, k), a1(i, j, k), hmx, ep) +
                vcorra(a1(i, j, k), s12(a2(i - 1, j, k), a2(i - 1, j + 1, k), a2(i, j + 1, k), a2(i, j, k)),
                       (absv(x(i - 1, j + 1, k)) + absv(x(i, j + 1, k))) -
                           (absv(x(i - 1, j - 1, k)) + absv(x(i, j - 1, k))),
                       absv(x(i - 1, j + 1, k)) + absv(x(i, j + 1, k)) +
                           absv(x(i - 1, j - 1, k)) + absv(x(i, j - 1, k)) + ep,
                       hmx);
          if (zt)
            v = v + vcorra(a1(i, j, k), s12(a3(i - 1, j, k), a3(i - 1, j, k + 1), a3(i, j, k + 1), a3(i, j, k)),
                           (absv(x(i - 1, j, k + 1)) + absv(x(i, j, k + 1))) -
                               (absv(x(i - 1, j, k - 1)) + absv(x(i, j, k - 1))),
                           absv(x(i - 1, j, k + 1)) + absv(x(i, j, k + 1)) +
                               absv(x(i - 1, j, k - 1)) + absv(x(i, j, k - 1)) + ep,
                           hmx);
          v1(i, j, k) = v;
          f1(i, j, k) = donor(x(i - 1, j, k), x(i, j, k), v);
        }
        if (j >= j0) {
          const R hmy = R(1) / (R(0.5) * (h(i, j - 1, k) + h(i, j, k)));
          R v = vdyfa(x(i, j - 1, k), x(i, j, k), a2(i, j, k), hmy, ep) +
                vcorra(a2(i, j, k), s14(a1(i, j - 1, k), a1(i, j, k), a1(i + 1, j, k), a1(i + 1, j - 1, k)),
                       (absv(x(i + 1, j - 1, k)) + absv(x(i + 1, j, k))) -
                           (absv(x(i - 1, j - 1, k)) + absv(x(i - 1, j, k))),
                       absv(x(i + 1, j - 1, k)) + absv(x(i + 1, j, k)) +
                           absv(x(i - 1, j - 1, k)) + absv(x(i - 1, j, k)) + ep,
                       hmy);
          if (zt)
            v = v + vcorra(a2(i, j, k), s14(a3(i, j - 1, k), a3(i, j, k), a3(i, j, k + 1), a3(i, j - 1, k + 1)),
                           (absv(x(i, j - 1, k + 1)) + absv(x(i, j, k + 1))) -
                               (absv(x(i, j - 1, k - 1)) + absv(x(i, j, k - 1))),
                           absv(x(i, j - 1, k + 1)) + absv(x(i, j, k + 1)) +
                               absv(x(i, j - 1, k - 1)) + absv(x(i, j, k - 1)) + ep,
                           hmy);
          v2(i, j, k) = v;
          f2(i, j, k) = donor(x(i, j - 1, k), x(i, j, k), v);
        }
        if (k >= k0) {
          const R hmz = R(1) / (R(0.5) * (h(i, j, k - 1) + h(i, j, k)));
          const R v = vdyfa(x(i, j, k - 1), x(i, j, k), a3(i, j, k), hmz, ep) +
                      vcorra(a3(i, j, k), s14(a1(i, j, k - 1), a1(i, j, k), a1(i + 1, j, k), a1(i + 1, j, k - 1)),
                             (absv(x(i + 1, j, k - 1)) + absv(x(i + 1, j, k))) -
                                 (absv(x(i - 1, j, k - 1)) + absv(x(i - 1, j, k))),
                             absv(x(i + 1, j, k - 1)) + absv(x(i + 1, j, k)) +
                                 absv(x(i - 1, j, k - 1)) + absv(x(i - 1, j, k)) + ep,
                             hmz) +
                      vcorra(a3(i, j, k), s12(a2(i, j, k - 1), a2(i, j + 1, k - 1), a2(i, j + 1, k), a2(i, j, k)),
                             (absv(x(i, j + 1, k - 1)) + absv(x(i, j + 1, k))) -
                                 (absv(x(i, j - 1, k - 1)) + absv(x(i, j - 1, k))),
                             absv(x(i, j + 1, k - 1)) + absv(x(i, j + 1, k)) +
                                 absv(x(i, j - 1, k - 1)) + absv(x(i, j - 1, k)) + ep,
                             hmz);
          v3(i, j, k) = v;
          f3(i, j, k) = donor(x(i, j, k - 1), x(i, j, k), v);
        }
      }
  }
  face_bc(v1, d, 0); face_bc(v2, d, 1); face_bc(v3, d, 2);
  face_bc(f1, d, 0); face_bc(f2, d, 1); face_bc(f3, d, 2);
}

// ---- pseudo-velocities, gauge form (antidiff3d-gauge-gpubc.f90:89-203) ----
template <class R>
void pseudo_gauge(const Dims& d, Buf<R>& x, Buf<R>& a1, Buf<R>& a2, Buf<R>& a3, Buf<R>& h,
                  Buf<R>& v1, Buf<R>& v2, Buf<R>& v3) {
  const int i0 = d.bx ? 1 : 2, j0 = d.by ? 1 : 2, k0 = d.bz ? 1 : 2;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++) {
    const bool zt = zterm(d, k);
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        if (i >= i0) {
          const R hmx = R(1) / (R(0.5) * (h(i - 1, j, k) + h(i, j, k)));
          const R c2 = (s12(a2(i - 1, j, k), a2(i - 1, j + 1, k), a2(i, j + 1, k), a2(i, j, k))) *
                       rat4(x(i - 1, j - 1, k), x(i, j - 1, k), x(i - 1, j + 1, k), x(i, j + 1, k));
          R cr = c2;
          if (zt)
            cr = c2 + (s12(a3(i - 1, j, k), a3(i - 1, j, k + 1), a3(i, j, k + 1), a3(i, j, k))) *
                          rat4(x(i - 1, j, k - 1), x(i, j, k - 1), x(i - 1, j, k + 1), x(i, j, k + 1));
          v1(i, j, k) = vdyf(x(i - 1, j, k), x(i, j, k), a1(i, j, k), hmx) -
                        R(0.125) * a1(i, j, k) * hmx * cr;
        }
        if (j >= j0) {
          const R hmy = R(1) / (R(0.5) * (h(i, j - 1, k) + h(i, j, k)));
          const R c1 = (s14(a1(i, j - 1, k), a1(i, j, k), a1(i + 1, j, k), a1(i + 1, j - 1, k))) *
                       rat4(x(i - 1, j - 1, k), x(i - 1, j, k), x(i + 1, j - 1, k), x(i + 1, j, k));
          R cr = c1;
          if (zt)
            cr = c1 + (s14(a3(i, j - 1, k), a3(i, j, k), a3(i, j, k + 1), a3(i, j - 1, k + 1))) *
                          rat4(x(i, j - 1, k - 1), x(i, j, k - 1), x(i, j - 1, k + 1), x(i, j, k + 1));
          v2(i, j, k) = vdyf(x(i, j - 1, k), x(i, j, k), a2(i, j, k), hmy) -
                        R(0.125) * a2(i, j, k) * hmy * cr;
        }
        if (k >= k0) {
          const R hmz = R(1) / (R(0.5) * (h(i, j, k - 1) + h(i, j, k)));
          const R cr = (s14(a1(i, j, k - 1), a1(i, j, k), a1(i + 1, j, k), a1(i + 1, j, k - 1))) *
                           rat4(x(i - 1, j, k - 1), x(i - 1, j, k), x(i + 1, j, k - 1), x(i + 1, j, k)) +
                       (s12(a2(i, j, k - 1), a2(i, j + 1, k - 1), a2(i, j + 1, k), a2(i, j, k))) *
                           rat4(x(i, j - 1, k - 1), x(i, j - 1, k), x(i, j + 1, k - 1), x(i, j + 1, k));
          v3(i, j, k) = vdyf(x(i, j, k - 1), x(i, j, k), a3(i, j, k), hmz) -
                        R(0.125) * a3(i, j, k) * hmz * cr;
        }
      }
  }
  face_bc(v1, d, 0); face_bc(v2, d, 1); face_bc(v3, d, 2);
}

// ---- limiter bounds: std :256-348, gauge :238-324 (k=1 gauge bug fixed: the
// minimum over x_in is computed as in mpdata3d-rho-gauge-gpubc.f90:365-368) ----
// mx/mn carry the running extrema: on entry the x_in star (first corrective
// pass) or the previous pass's bounds; the star of the current field is folded in.
template <class R>
void bounds_fold(const Dims& d, Buf<R>& x, Buf<R>& mx, Buf<R>& mn, bool first, Buf<R>& xin) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++) {
    const bool lo = d.bz || k > 1, hi = d.bz || k < d.lp;
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        R ma, mi;
        if (first) {
          ma = mx2(mx2(mx2(xin(i - 1, j, k), xin(i, j, k)), mx2(xin(i + 1, j, k), xin(i, j - 1, k))), xin(i, j + 1, k));
          mi = mn2(mn2(mn2(xin(i - 1, j, k), xin(i, j, k)), mn2(xin(i + 1, j, k), xin(i, j - 1, k))), xin(i, j + 1, k));
          if (lo) { ma = mx2(ma, xin(i, j, k - 1)); mi = mn2(mi, xin(i, j, k - 1)); }
          if (hi) { ma = mx2(ma, xin(i, j, k + 1)); mi = mn2(mi, xin(i, j, k + 1)); }
        } else {
          ma = mx(i, j, k);
          mi = mn(i, j, k);
        }
        ma = mx2(mx2(mx2(ma, x(i - 1, j, k)), mx2(x(i, j, k), x(i + 1, j, k))), mx2(x(i, j - 1, k), x(i, j + 1, k)));
        mi = mn2(mn2(mn2(mi, x(i - 1, j, k)), mn2(x(i, j, k), x(i + 1, j, k))), mn2(x(i, j - 1, k), x(i, j + 1, k)));
        if (lo) { ma = mx2(ma, x(i, j, k - 1)); mi = mn2(mi, x(i, j, k - 1)); }
        if (hi) { ma = mx2(ma, x(i, j, k + 1)); mi = mn2(mi, x(i, j, k + 1)); }
        mx(i, j, k) = ma;
        mn(i, j, k) = mi;
      }
  }
}

// cp/cn from the bounds and the antidiffusive face fluxes F (std: donor
// fluxes f*ns; gauge: the velocities v themselves).
template <class R>
void cpcn(const Dims& d, Buf<R>& x, Buf<R>& mx, Buf<R>& mn, Buf<R>& h, Buf<R>& F1, Buf<R>& F2,
          Buf<R>& F3, Buf<R>& cp, Buf<R>& cn, R ep) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        cp(i, j, k) = (mx(i, j, k) - x(i, j, k)) * h(i, j, k) /
                      (pn(F1(i + 1, j, k)) + pp(F1(i, j, k)) + pn(F2(i, j + 1, k)) + pp(F2(i, j, k)) +
                       pn(F3(i, j, k + 1)) + pp(F3(i, j, k)) + ep);
        cn(i, j, k) = (x(i, j, k) - mn(i, j, k)) * h(i, j, k) /
                      (pp(F1(i + 1, j, k)) + pn(F1(i, j, k)) + pp(F2(i, j + 1, k)) + pn(F2(i, j, k)) +
                       pp(F3(i, j, k + 1)) + pn(F3(i, j, k)) + ep);
      }
  halo_zero_or_wrap(cp, d);
  halo_zero_or_wrap(cn, d);
}

template <class R> inline R min3(R a, R b) { return mn2(mn2(R(1), a), b); }

// Standard-form limited velocity (antidiff3d-standard-gpubc.f90:373-379).
template <class R>
inline R vlim_std(R v, R a1, R a2, R xl, R xr) {
  return pp(v) * (a1 * possign(xl) + a2 * possign(-xl)) - pn(v) * (a2 * possign(xr) + a1 * possign(-xr));
}

// ---- standard limited fluxes + update (antidiff3d-standard-gpubc.f90:372-459) ----
template <class R>
void limit_update_std(const Dims& d, bool nonos, Buf<R>& x, Buf<R>& v1, Buf<R>& v2, Buf<R>& v3,
                      Buf<R>& cp, Buf<R>& cn, Buf<R>& rhr, Buf<R>& h, Buf<R>& w1, Buf<R>& w2,
                      Buf<R>& w3, Buf<R>& f1, Buf<R>& f2, Buf<R>& f3, Buf<R>& xout) {
  const int i0 = d.bx ? 1 : 2, j0 = d.by ? 1 : 2, k0 = d.bz ? 1 : 2;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        if (i >= i0) {
          const R w = nonos ? vlim_std(v1(i, j, k), min3(cp(i, j, k), cn(i - 1, j, k)),
                                       min3(cp(i - 1, j, k), cn(i, j, k)), x(i - 1, j, k), x(i, j, k))
                            : v1(i, j, k);
          w1(i, j, k) = w;
          f1(i, j, k) = donor(x(i - 1, j, k) / rhr(i - 1, j, k), x(i, j, k) / rhr(i, j, k), w);
        }
        if (j >= j0) {
          const R w = nonos ? vlim_std(v2(i, j, k), min3(cp(i, j, k), cn(i, j - 1, k)),
                                       min3(cp(i, j - 1, k), cn(i, j, k)), x(i, j - 1, k), x(i, j, k))
                            : v2(i, j, k);
          w2(i, j, k) = w;
          f2(i, j, k) = donor(x(i, j - 1, k) / rhr(i, j - 1, k), x(i, j, k) / rhr(i, j, k), w);
        }
        if (k >= k0) {
          const R w = nonos ? vlim_std(v3(i, j, k), min3(cp(i, j, k), cn(i, j, k - 1)),
                                       min3(cp(i, j, k - 1), cn(i, j, k)), x(i, j, k - 1), x(i, j, k))
                            : v3(i, j, k);
          w3(i, j, k) = w;
          f3(i, j, k) = donor(x(i, j, k - 1) / rhr(i, j, k - 1), x(i, j, k) / rhr(i, j, k), w);
        }
      }
  face_bc(f1, d, 0); face_bc(f2, d, 1); face_bc(f3, d, 2);
  face_bc(w1, d, 0); face_bc(w2, d, 1); face_bc(w3, d, 2);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        const R hinv = R(1) / h(i, j, k);
        xout(i, j, k) = rhr(i, j, k) * (x(i, j, k) / rhr(i, j, k) -
                                        (f1(i + 1, j, k) - f1(i, j, k) + f2(i, j + 1, k) - f2(i, j, k) +
                                         f3(i, j, k + 1) - f3(i, j, k)) * hinv);
      }
}

// ---- gauge limited fluxes + update (antidiff3d-gauge-gpubc.f90:340-428) ----
template <class R>
void limit_update_gauge(const Dims& d, bool nonos, Buf<R>& x, Buf<R>& v1, Buf<R>& v2, Buf<R>& v3,
                        Buf<R>& cp, Buf<R>& cn, Buf<R>& rhr, Buf<R>& h, Buf<R>& w1, Buf<R>& w2,
                        Buf<R>& w3, Buf<R>& xout) {
  const int i0 = d.bx ? 1 : 2, j0 = d.by ? 1 : 2, k0 = d.bz ? 1 : 2;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        if (i >= i0) {
          const R v = v1(i, j, k);
          w1(i, j, k) = nonos ? pp(v) * min3(cp(i, j, k), cn(i - 1, j, k)) - pn(v) * min3(cp(i - 1, j, k), cn(i, j, k)) : v;
        }
        if (j >= j0) {
          const R v = v2(i, j, k);
          w2(i, j, k) = nonos ? pp(v) * min3(cp(i, j, k), cn(i, j - 1, k)) - pn(v) * min3(cp(i, j - 1, k), cn(i, j, k)) : v;
        }
        if (k >= k0) {
          const R v = v3(i, j, k);
          w3(i, j, k) = nonos ? pp(v) * min3(cp(i, j, k), cn(i, j, k - 1)) - pn(v) * min3(cp(i, j, k - 1), cn(i, j, k)) : v;
        }
      }
  face_bc(w1, d, 0); face_bc(w2, d, 1); face_bc(w3, d, 2);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        xout(i, j, k) = rhr(i, j, k) * (x(i, j, k) / rhr(i, j, k) -
                                        (w1(i + 1, j, k) - w1(i, j, k) + w2(i, j + 1, k) - w2(i, j, k) +
                                         w3(i, j, k + 1) - w3(i, j, k)) / h(i, j, k));
      }
}

// ---- mpdata3d_rho_gauge_gpubc (mpdata3d-rho-gauge-gpubc.f90:23-622) -------
// Density step: predictor, upwind without rhr that keeps its fluxes
// (:137-210), gauge antidiffusion (:230-446), then x_incomp, pexr1/2, rhr and
// the mass fluxes u = upwind flux + limited antidiffusive flux (:461-606).
template <class R>
int rho_gauge(const orc_grid* g, R* ox, R* oy, R* oz, R* pu, R* pv, R* pw, R* u1o, R* u2o, R* u3o,
              R* x_in, R* x_incomp, const R* h_in, R* rhoadv, R* rhr_out, const R* pexe, R* pexr1,
              R* pexr2, const R* bcx, const R* bcy, R dxi, R dyi, R dzi, R dt, R dt_ratio, int liner);
// The density step after the predictor: u1o..u3o hold the C-grid Courant
// numbers on entry and the mass fluxes on exit.
template <class R>
int rho_step(const orc_grid* g, R* u1o, R* u2o, R* u3o, R* x_in, R* x_incomp, const R* h_in, R* rhoadv,
             R* rhr_out, const R* pexe, R* pexr1, R* pexr2, const R* bcx, const R* bcy, int liner);

bool dims_ok(const orc_grid* g) {
  if (!g) return false;
  if (g->ih < 1) return false;
  if (g->np < (g->ibcx ? 1 : 2) || g->mp < (g->ibcy ? 1 : 2) || g->lp < (g->ibcz ? 1 : 2)) return false;
  auto b = [](int v) { return v == 0 || v == 1; };
  return b(g->ibcx) && b(g->ibcy) && b(g->ibcz);
}

template <class R>
int advec(const orc_grid* g, int opt, int t_adv, int iord, int nonos, R* x, const R* bcx,
          const R* bcy, const R* uadv, const R* vadv, const R* wadv, const R* rhr_in,
          const R* h_in) {
  if (!dims_ok(g)) return -1;
  if (opt != 4 && opt != 6) return -2;
  if (opt == 4 && t_adv != 1 && t_adv != 2) return -2;
  if (opt == 4 && (iord < 2 || iord > 8)) return -2;
  if (!x || !uadv || !vadv || !wadv || !rhr_in || !h_in) return -3;
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  if ((!d.bx && !bcx) || (!d.by && !bcy)) return -3;
  const R ep = R(1e-10);  // ep_nonos, common/epsilons.f90:3
  const int NX = d.np + 2, NY = d.mp + 2, NZ = d.lp + 2;
  V3<R> X = view<R>(x, d.ih, d.np + 2 * d.ih, d.mp + 2 * d.ih);

  Buf<R> xin(NX, NY, NZ), h(NX, NY, NZ), rhr(NX, NY, NZ);
  Buf<R> u1(NX + 1, NY, NZ), u2(NX, NY + 1, NZ), u3(NX, NY, NZ + 1);
  load_cell(xin, x, d);
  load_cell(h, h_in, d);
  load_cell(rhr, rhr_in, d);
  load_face(u1, uadv, d, 0);
  load_face(u2, vadv, d, 1);
  load_face(u3, wadv, d, 2);
  // putbcinxh (mpdataoperators.inc:253-287): Dirichlet x/y halos from bcx/bcy.
  if (!d.bx)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++) {
        xin(0, j, k) = bcx[(j - 1) + (long)d.mp * (k - 1)];
        xin(d.np + 1, j, k) = bcx[(j - 1) + (long)d.mp * (k - 1) + (long)d.mp * d.lp];
      }
  if (!d.by)
    for (int k = 1; k <= d.lp; k++)
      for (int i = 1; i <= d.np; i++) {
        xin(i, 0, k) = bcy[(i - 1) + (long)d.np * (k - 1)];
        xin(i, d.mp + 1, k) = bcy[(i - 1) + (long)d.np * (k - 1) + (long)d.np * d.lp];
      }

  Buf<R> xant(NX, NY, NZ);
  upwind(d, xin, u1, u2, u3, h, rhr, xant);

  if (opt == 6) {  // advec.f90:221-232: upwind only, copy back
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++)
        for (int i = 1; i <= d.np; i++) X(i, j, k) = xant(i, j, k);
    // the psi halo keeps the Dirichlet values written by putbcinxh
    if (!d.bx)
      for (int k = 1; k <= d.lp; k++)
        for (int j = 1; j <= d.mp; j++) { X(0, j, k) = xin(0, j, k); X(d.np + 1, j, k) = xin(d.np + 1, j, k); }
    if (!d.by)
      for (int k = 1; k <= d.lp; k++)
        for (int i = 1; i <= d.np; i++) { X(i, 0, k) = xin(i, 0, k); X(i, d.mp + 1, k) = xin(i, d.mp + 1, k); }
    return 0;
  }

  const bool gauge = (t_adv == 1);
  Buf<R> v1(NX + 1, NY, NZ), v2(NX, NY + 1, NZ), v3(NX, NY, NZ + 1);
  Buf<R> w1(NX + 1, NY, NZ), w2(NX, NY + 1, NZ), w3(NX, NY, NZ + 1);
  Buf<R> f1(NX + 1, NY, NZ), f2(NX, NY + 1, NZ), f3(NX, NY, NZ + 1);
  Buf<R> g1(NX + 1, NY, NZ), g2(NX, NY + 1, NZ), g3(NX, NY, NZ + 1);
  Buf<R> mx(NX, NY, NZ), mn(NX, NY, NZ), cp(NX, NY, NZ), cn(NX, NY, NZ), xnew(NX, NY, NZ);

  // x_in halo for the bounds: zero-gradient (cp_last_to_halo_xy) / periodic
  Buf<R> xb(NX, NY, NZ);
  std::copy(xin.d.begin(), xin.d.end(), xb.d.begin());
  halo_last(xb, d);

  // "a" fields of the passes after the first corrective one: the previous
  // pass's limited pseudo-velocities (published MPDATA recursion; the
  // reference itself stops at iord=2, antidiff3d-gauge-gpubc.f90:81-83).
  Buf<R> b1(NX + 1, NY, NZ), b2(NX, NY + 1, NZ), b3(NX, NY, NZ + 1);
  Buf<R>* xc = &xant;
  Buf<R>* xn = &xnew;
  Buf<R>*a1 = &u1, *a2 = &u2, *a3 = &u3;
  for (int pass = 2; pass <= iord; pass++) {
    halo_second_last(*xc, d);  // cp_scnd_last_to_halo_xy_fulld
    if (gauge)
      pseudo_gauge(d, *xc, *a1, *a2, *a3, h, v1, v2, v3);
    else
      pseudo_std(d, *xc, *a1, *a2, *a3, h, v1, v2, v3, f1, f2, f3, ep);
    if (nonos) {
      bounds_fold(d, *xc, mx, mn, pass == 2, xb);
      if (gauge)
        cpcn(d, *xc, mx, mn, h, v1, v2, v3, cp, cn, ep);
      else
        cpcn(d, *xc, mx, mn, h, f1, f2, f3, cp, cn, ep);
    }
    if (gauge)
      limit_update_gauge(d, nonos != 0, *xc, v1, v2, v3, cp, cn, rhr, h, w1, w2, w3, *xn);
    else
      limit_update_std(d, nonos != 0, *xc, v1, v2, v3, cp, cn, rhr, h, w1, w2, w3, g1, g2, g3, *xn);
    std::swap(xc, xn);
    if (pass < iord) {
      std::copy(w1.d.begin(), w1.d.end(), b1.d.begin());
      std::copy(w2.d.begin(), w2.d.end(), b2.d.begin());
      std::copy(w3.d.begin(), w3.d.end(), b3.d.begin());
      a1 = &b1; a2 = &b2; a3 = &b3;
    }
  }

  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) X(i, j, k) = (*xc)(i, j, k);
  // psi halo after the step: the zero-gradient copy of the old boundary values
  // written by cp_last_to_halo_xy (antidiff3d-*-gpubc.f90:256 / :215)
  if (!d.bx)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++) { X(0, j, k) = xin(1, j, k); X(d.np + 1, j, k) = xin(d.np, j, k); }
  if (!d.by)
    for (int k = 1; k <= d.lp; k++)
      for (int i = 1; i <= d.np; i++) { X(i, 0, k) = xin(i, 1, k); X(i, d.mp + 1, k) = xin(i, d.mp, k); }
  return 0;
}

// ---- velprd_traj0, velprdA_to_C, the driver's level roll ----
// Three-level momentum stacks ox/oy/oz (level stride lev), psi-shaped levels.
template <class R>
struct Pred {
  Dims d;
  int SX, SY;
  long lev;
  R* o[3];
  R* phys[3];
  V3<R> H;
};

template <class R>
Pred<R> pred_of(const Dims& d, R* ox, R* oy, R* oz, R* u, R* v, R* w, const R* h_in) {
  Pred<R> p;
  p.d = d;
  p.SX = d.np + 2 * d.ih;
  p.SY = d.mp + 2 * d.ih;
  p.lev = (long)p.SX * p.SY * (d.lp + 2 * d.ih);
  p.o[0] = ox; p.o[1] = oy; p.o[2] = oz;
  p.phys[0] = u; p.phys[1] = v; p.phys[2] = w;
  p.H = view<R>(const_cast<R*>(h_in), d.ih, p.SX, p.SY);
  return p;
}

// velprd_traj0 / velprd_traj0_adapt_dt (module_velprd.f90:60-83, :133-156):
// n+1/2 momenta times dt/dx into level 1
template <class R>
void pred_level(const Pred<R>& p, R dt, R dxi, R dyi, R dzi, R dt_ratio) {
  const Dims& d = p.d;
  const R gc[3] = {dt * dxi, dt * dyi, dt * dzi};  // module_velprd.f90:52-54
  for (int c = 0; c < 3; c++) {
    V3<R> O0 = view<R>(p.o[c], d.ih, p.SX, p.SY), O1 = view<R>(p.o[c] + p.lev, d.ih, p.SX, p.SY),
          O2 = view<R>(p.o[c] + 2 * p.lev, d.ih, p.SX, p.SY);
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++)
        for (int i = 1; i <= d.np; i++) {
          const R a0 = O0(i, j, k) * p.H(i, j, k);
          const R a2 = O2(i, j, k);
          const R a1 = a0 + dt_ratio * (a0 - a2);
          O1(i, j, k) = R(0.5) * (a1 + a0) * gc[c];
        }
  }
}

// velprdA_to_C (:197-361) of level 1: halo extrapolation on open walls, then averaging
template <class R>
void pred_a_to_c(const Pred<R>& p, R* u1o, R* u2o, R* u3o) {
  const Dims& d = p.d;
  const int SX = p.SX, SY = p.SY, ih = d.ih;
  V3<R> A1 = view<R>(p.o[0] + p.lev, ih, SX, SY), A2 = view<R>(p.o[1] + p.lev, ih, SX, SY),
        A3 = view<R>(p.o[2] + p.lev, ih, SX, SY);
  if (!d.bx)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++) {
        A1(0, j, k) = R(2) * A1(1, j, k) - A1(2, j, k);
        A1(d.np + 1, j, k) = R(2) * A1(d.np, j, k) - A1(d.np - 1, j, k);
      }
  if (!d.by)
    for (int k = 1; k <= d.lp; k++)
      for (int i = 1; i <= d.np; i++) {
        A2(i, 0, k) = R(2) * A2(i, 1, k) - A2(i, 2, k);
        A2(i, d.mp + 1, k) = R(2) * A2(i, d.mp, k) - A2(i, d.mp - 1, k);
      }
  if (!d.bz)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        A3(i, j, 0) = R(2) * A3(i, j, 1) - A3(i, j, 2);
        A3(i, j, d.lp + 1) = R(2) * A3(i, j, d.lp) - A3(i, j, d.lp - 1);
      }
  V3<R> U1 = view<R>(u1o, ih, SX + 1, SY), U2 = view<R>(u2o, ih, SX, SY + 1), U3 = view<R>(u3o, ih, SX, SY);
  auto wx = [&](int i) { return d.bx ? (i < 1 ? i + d.np : (i > d.np ? i - d.np : i)) : i; };
  auto wy = [&](int j) { return d.by ? (j < 1 ? j + d.mp : (j > d.mp ? j - d.mp : j)) : j; };
  auto wz = [&](int k) { return d.bz ? (k < 1 ? k + d.lp : (k > d.lp ? k - d.lp : k)) : k; };
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 1; k <= d.lp + 1; k++)
    for (int j = 1; j <= d.mp + 1; j++)
      for (int i = 1; i <= d.np + 1; i++) {
        if (j <= d.mp && k <= d.lp) {
          const int ii = (d.bx && i == d.np + 1) ? 1 : i;
          U1(i, j, k) = R(0.5) * (A1(ii, j, k) + A1(wx(ii - 1), j, k));
        }
        if (i <= d.np && k <= d.lp) {
          const int jj = (d.by && j == d.mp + 1) ? 1 : j;
          U2(i, j, k) = R(0.5) * (A2(i, jj, k) + A2(i, wy(jj - 1), k));
        }
        if (i <= d.np && j <= d.mp) {
          const int kk = (d.bz && k == d.lp + 1) ? 1 : k;
          U3(i, j, k) = R(0.5) * (A3(i, j, kk) + A3(i, j, wz(kk - 1)));
        }
      }
}

// velprd_driver.f90:254-270 — roll levels, store n momenta for the next step
template <class R>
void pred_roll(const Pred<R>& p, R dt_ratio) {
  const Dims& d = p.d;
  const int SX = p.SX, SY = p.SY, ih = d.ih;
  for (int c = 0; c < 3; c++) {
    V3<R> O0 = view<R>(p.o[c], ih, SX, SY), O2 = view<R>(p.o[c] + 2 * p.lev, ih, SX, SY);
    V3<R> P0{nullptr, 0, 0, 0}, P1{nullptr, 0, 0, 0}, P2{nullptr, 0, 0, 0};
    R* ph = p.phys[c];
    if (ph) {
      P0 = view<R>(ph, ih, SX, SY);
      P1 = view<R>(ph + p.lev, ih, SX, SY);
      P2 = view<R>(ph + 2 * p.lev, ih, SX, SY);
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++)
        for (int i = 1; i <= d.np; i++) {
          if (ph) {
            P1(i, j, k) = P0(i, j, k) + dt_ratio * (P0(i, j, k) - P2(i, j, k));
            P2(i, j, k) = P0(i, j, k);
          }
          O2(i, j, k) = O0(i, j, k) * p.H(i, j, k);
        }
  }
}

// velprd_traj0 + velprdA_to_C + the driver's level roll, as the driver's
// plain path runs them (velprd_driver.f90:236-270)
template <class R>
int velprd(const orc_grid* g, R* ox, R* oy, R* oz, R* u, R* v, R* w, const R* h_in, R dxi, R dyi,
           R dzi, R dt, R dt_ratio, R* u1o, R* u2o, R* u3o) {
  if (!dims_ok(g)) return -1;
  if (!ox || !oy || !oz || !h_in || !u1o || !u2o || !u3o) return -3;
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  const Pred<R> p = pred_of<R>(d, ox, oy, oz, u, v, w, h_in);
  pred_level<R>(p, dt, dxi, dyi, dzi, dt_ratio);
  pred_a_to_c<R>(p, u1o, u2o, u3o);
  pred_roll<R>(p, dt_ratio);
  return 0;
}

// compute_courants (common/diagutils.f90:606-654): serial maxima over the
// interior, starting from -HUGE
template <class R>
void courants(const Pred<R>& p, int level, R dxi, R dyi, R dzi, R dt, R cr[7]) {
  const Dims& d = p.d;
  for (int c = 0; c < 7; c++) cr[c] = -std::numeric_limits<R>::max();
  const int lv = level == 2 ? 1 : 0;
  V3<R> X = view<R>(p.o[0] + lv * p.lev, d.ih, p.SX, p.SY), Y = view<R>(p.o[1] + lv * p.lev, d.ih, p.SX, p.SY),
        Z = view<R>(p.o[2] + lv * p.lev, d.ih, p.SX, p.SY);
  const R gc1 = dt * dxi, gc2 = dt * dyi, gc3 = dt * dzi;
  auto mx = [](R a, R b) { return a > b ? a : b; };
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        R a, b, c;
        if (level == 2) {
          const R dinv = R(1) / p.H(i, j, k);
          a = std::fabs(X(i, j, k) * dinv);
          b = std::fabs(Y(i, j, k) * dinv);
          c = std::fabs(Z(i, j, k) * dinv);
        } else {
          a = std::fabs(gc1 * X(i, j, k));
          b = std::fabs(gc2 * Y(i, j, k));
          c = std::fabs(gc3 * Z(i, j, k));
        }
        cr[0] = mx(cr[0], a + b + c);
        cr[1] = mx(cr[1], a + b);
        cr[2] = mx(cr[2], a + c);
        cr[3] = mx(cr[3], b + c);
        cr[4] = mx(cr[4], a);
        cr[5] = mx(cr[5], b);
        cr[6] = mx(cr[6], c);
      }
}

// velprd_driver (velprd_driver.f90:16-270), scalars in R.  Returns 0, -2
// (substepping with adaptivity, the STOP at :74), -9 (the STOP at :123, or a
// non-finite Courant number that would loop forever).
template <class R>
int velprd_driver(const orc_grid* g, int* nsubsteps, int* nsubsteps_o, int lsubstepping, R* dtn, R* dtnold,
                  int ltimeadapt, int lvertsplit, int lcrdiag_nphlf, R crmaxlim, R dtmax, R* ox, R* oy, R* oz,
                  R* u, R* v, R* w, R* uadv, R* vadv, R* wadv, const R* h, R dxi, R dyi, R dzi, R dt,
                  double* diag) {
  if (!dims_ok(g)) return -1;
  if (!nsubsteps || !nsubsteps_o || !dtn || !dtnold || !ox || !oy || !oz || !uadv || !vadv || !wadv || !h)
    return -3;
  if (lsubstepping && ltimeadapt) return -2;
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  const Pred<R> p = pred_of<R>(d, ox, oy, oz, u, v, w, h);
  const R TINYR = std::numeric_limits<R>::min();
  R cr[7];
  auto split = [&]() { return (cr[1] > R(0.5) * cr[6] ? cr[1] : R(0.5) * cr[6]) + TINYR; };
  auto traj0 = [&](R dtx, R r) {
    pred_level<R>(p, dtx, dxi, dyi, dzi, r);
    pred_a_to_c<R>(p, uadv, vadv, wadv);
  };
  R dt_ratio = R(1);
  R dtntemp = *dtn;
  if (lsubstepping && *nsubsteps == 1) dt_ratio = (dt / (R(0.0f) * *nsubsteps + R(1))) / (dt / *nsubsteps_o);
  if (lsubstepping) dtntemp = dt;
  if (ltimeadapt) dtntemp = *dtn;
  if (lcrdiag_nphlf) {
    pred_level<R>(p, dtntemp, dxi, dyi, dzi, dt_ratio);  // velprd_traj0_adapt_dt
    courants<R>(p, 2, dxi, dyi, dzi, dtntemp, cr);
  } else {
    courants<R>(p, 1, dxi, dyi, dzi, dtntemp, cr);
  }
  R cr_for_dt = cr[0];
  if (lvertsplit) cr_for_dt = split();
  if (lsubstepping) {
    bool ok = true;
    if (cr_for_dt > crmaxlim && *nsubsteps == 1) {
      *nsubsteps = (int)std::ceil(cr_for_dt);
      if (cr_for_dt / *nsubsteps > crmaxlim) *nsubsteps += 1;
      ok = false;
    } else if (cr_for_dt / *nsubsteps > R(10) && *nsubsteps > 1) {
      return -9;
    }
    *dtn = dt / *nsubsteps;
    if (lvertsplit) {
      dt_ratio = *dtn / *dtnold;
      traj0(*dtn, dt_ratio);
      courants<R>(p, 2, dxi, dyi, dzi, *dtn, cr);
      cr_for_dt = cr[0];
    }
    for (int round = 0; !ok; round++) {
      if (round >= 10000 || !(cr_for_dt == cr_for_dt)) return -9;
      dt_ratio = *dtn / *dtnold;
      traj0(*dtn, dt_ratio);
      courants<R>(p, 2, dxi, dyi, dzi, *dtn, cr);
      cr_for_dt = cr[0];
      if (lvertsplit) cr_for_dt = split();
      if (cr_for_dt <= crmaxlim) {
        ok = true;
      } else {
        *nsubsteps += 1;
        *dtn = dt / *nsubsteps;
      }
    }
    *nsubsteps_o = *nsubsteps;
    *dtnold = *dtn;
    *dtn = dt / *nsubsteps;
    if (*nsubsteps > 1 || !lcrdiag_nphlf)
      traj0(*dtn, dt_ratio);
    else
      pred_a_to_c<R>(p, uadv, vadv, wadv);
  } else if (ltimeadapt) {
    R crmaxlimtemp = crmaxlim;
    *dtnold = *dtn;
    for (int round = 0;; round++) {
      if (round >= 10000 || !(cr_for_dt == cr_for_dt)) return -9;
      R t = (crmaxlimtemp / (std::fabs(cr_for_dt) + TINYR)) * *dtn;
      t = t < dtmax ? t : dtmax;
      if (t > *dtnold && ((t - *dtnold) / *dtnold) > R(0.1f)) *dtn = t;
      if (t <= *dtnold) *dtn = t;
      dt_ratio = *dtn / *dtnold;
      traj0(*dtn, dt_ratio);
      courants<R>(p, 2, dxi, dyi, dzi, *dtn, cr);
      cr_for_dt = cr[0];
      if (lvertsplit) cr_for_dt = split();
      if (cr_for_dt <= crmaxlim) break;
      crmaxlimtemp = R(0.99f) * crmaxlimtemp;
    }
  } else {
    if (!lcrdiag_nphlf)
      traj0(*dtn, dt_ratio);
    else
      pred_a_to_c<R>(p, uadv, vadv, wadv);
  }
  if (lvertsplit) {  // FullXYZDomainWithHaloLoopDC: k = 1-ih .. lp+ih, halo included
    const long n = (long)p.SX * p.SY * (d.lp + 2 * d.ih);
    for (long t = 0; t < n; t++) wadv[t] = R(0.5f) * wadv[t];
  }
  pred_roll<R>(p, dt_ratio);
  if (diag) {
    for (int c = 0; c < 7; c++) diag[c] = (double)cr[c];
    diag[7] = (double)cr_for_dt;
    diag[8] = (double)dt_ratio;
  }
  return 0;
}

template <class R>
int rho_gauge(const orc_grid* g, R* ox, R* oy, R* oz, R* pu, R* pv, R* pw, R* u1o, R* u2o, R* u3o,
              R* x_in, R* x_incomp, const R* h_in, R* rhoadv, R* rhr_out, const R* pexe, R* pexr1,
              R* pexr2, const R* bcx, const R* bcy, R dxi, R dyi, R dzi, R dt, R dt_ratio, int liner) {
  if (!dims_ok(g)) return -1;
  if (!x_in || !x_incomp || !rhoadv || !rhr_out || !pexe || !pexr1 || !pexr2) return -3;
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  if ((!d.bx && !bcx) || (!d.by && !bcy)) return -3;
  // velprd_driver (:106-111): predictor into u1..u3, level roll
  int rc = velprd<R>(g, ox, oy, oz, pu, pv, pw, h_in, dxi, dyi, dzi, dt, dt_ratio, u1o, u2o, u3o);
  if (rc) return rc;
  return rho_step<R>(g, u1o, u2o, u3o, x_in, x_incomp, h_in, rhoadv, rhr_out, pexe, pexr1, pexr2, bcx, bcy, liner);
}

template <class R>
int rho_step(const orc_grid* g, R* u1o, R* u2o, R* u3o, R* x_in, R* x_incomp, const R* h_in, R* rhoadv,
             R* rhr_out, const R* pexe, R* pexr1, R* pexr2, const R* bcx, const R* bcy, int liner) {
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  const R ep = R(1e-10);
  const int NX = d.np + 2, NY = d.mp + 2, NZ = d.lp + 2, ih = d.ih;
  const int SX = d.np + 2 * ih, SY = d.mp + 2 * ih;
  V3<R> X = view<R>(x_in, ih, SX, SY), XC = view<R>(x_incomp, ih, SX, SY), RA = view<R>(rhoadv, ih, SX, SY),
        RO = view<R>(rhr_out, ih, SX, SY), PE = view<R>(const_cast<R*>(pexe), ih, SX, SY),
        P1 = view<R>(pexr1, ih, SX, SY), P2 = view<R>(pexr2, ih, SX, SY);
  // rhoadv = x_incomp (:121-123)
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) RA(i, j, k) = XC(i, j, k);
  Buf<R> xin(NX, NY, NZ), h(NX, NY, NZ), ones(NX, NY, NZ);
  Buf<R> u1(NX + 1, NY, NZ), u2(NX, NY + 1, NZ), u3(NX, NY, NZ + 1);
  load_cell(xin, x_in, d);
  load_cell(h, h_in, d);
  std::fill(ones.d.begin(), ones.d.end(), R(1));
  load_face(u1, u1o, d, 0);
  load_face(u2, u2o, d, 1);
  load_face(u3, u3o, d, 2);
  if (!d.bx)  // putbcinxh (:124)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++) {
        xin(0, j, k) = bcx[(j - 1) + (long)d.mp * (k - 1)];
        xin(d.np + 1, j, k) = bcx[(j - 1) + (long)d.mp * (k - 1) + (long)d.mp * d.lp];
      }
  if (!d.by)
    for (int k = 1; k <= d.lp; k++)
      for (int i = 1; i <= d.np; i++) {
        xin(i, 0, k) = bcy[(i - 1) + (long)d.np * (k - 1)];
        xin(i, d.mp + 1, k) = bcy[(i - 1) + (long)d.np * (k - 1) + (long)d.np * d.lp];
      }
  // upwind that keeps its fluxes (:137-210); no rhr, division by h
  Buf<R> xant(NX, NY, NZ), fn1(NX + 1, NY, NZ), fn2(NX, NY + 1, NZ), fn3(NX, NY, NZ + 1);
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        const R x = xin(i, j, k);
        const R f1p = donor(x, xin(i + 1, j, k), u1(i + 1, j, k));
        const R f1 = donor(xin(i - 1, j, k), x, u1(i, j, k));
        const R f2p = donor(x, xin(i, j + 1, k), u2(i, j + 1, k));
        const R f2 = donor(xin(i, j - 1, k), x, u2(i, j, k));
        R f3p, f3;
        if (!d.bz && k == 1) { f3p = donor(x, xin(i, j, k + 1), u3(i, j, k + 1)); f3 = -f3p; }
        else if (!d.bz && k == d.lp) { f3 = donor(xin(i, j, k - 1), x, u3(i, j, k)); f3p = -f3; }
        else { f3p = donor(x, xin(i, j, k + 1), u3(i, j, k + 1)); f3 = donor(xin(i, j, k - 1), x, u3(i, j, k)); }
        xant(i, j, k) = x - (f1p - f1 + f2p - f2 + f3p - f3) / h(i, j, k);
        fn1(i, j, k) = f1;
        fn2(i, j, k) = f2;
        fn3(i, j, k) = f3;
        if (i == d.np) fn1(d.np + 1, j, k) = f1p;  // :192-197
        if (j == d.mp) fn2(i, d.mp + 1, k) = f2p;  // :198-203
        if (k == d.lp) fn3(i, j, d.lp + 1) = f3p;  // :205-210
      }
  Buf<R> w1(NX + 1, NY, NZ), w2(NX, NY + 1, NZ), w3(NX, NY, NZ + 1);
  Buf<R>* xfin = &xant;
  Buf<R> xnew(NX, NY, NZ);
  if (!liner) {
    Buf<R> v1(NX + 1, NY, NZ), v2(NX, NY + 1, NZ), v3(NX, NY, NZ + 1);
    Buf<R> mx(NX, NY, NZ), mn(NX, NY, NZ), cp(NX, NY, NZ), cn(NX, NY, NZ);
    Buf<R> xb(NX, NY, NZ);
    std::copy(xin.d.begin(), xin.d.end(), xb.d.begin());
    halo_last(xb, d);
    halo_second_last(xant, d);
    pseudo_gauge(d, xant, u1, u2, u3, h, v1, v2, v3);
    bounds_fold(d, xant, mx, mn, true, xb);
    cpcn(d, xant, mx, mn, h, v1, v2, v3, cp, cn, ep);
    // with rhr = 1 the gauge update rhr*(xant/rhr - div/h) is xant - div/h (:482-485)
    limit_update_gauge(d, true, xant, v1, v2, v3, cp, cn, ones, h, w1, w2, w3, xnew);
    xfin = &xnew;
  }
  // outputs (:486-493, 570-606); mass fluxes on faces 1..n+1
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        const R xv = (*xfin)(i, j, k);
        X(i, j, k) = xv;
        const R xc = xv * h(i, j, k);
        XC(i, j, k) = xc;
        P1(i, j, k) = xc * PE(i, j, k);
        P2(i, j, k) = xc;
        RO(i, j, k) = RA(i, j, k) / xc;
      }
  // boundary faces of the upwind fluxes follow the same rules as the others
  if (d.bx) wrap(fn1, d, true, false, false);
  if (d.by) wrap(fn2, d, false, true, false);
  if (d.bz) wrap(fn3, d, false, false, true);
  else
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) fn3(i, j, 1) = -fn3(i, j, 2);
  V3<R> U1 = view<R>(u1o, ih, SX + 1, SY), U2 = view<R>(u2o, ih, SX, SY + 1), U3 = view<R>(u3o, ih, SX, SY);
  for (int k = 1; k <= d.lp + 1; k++)
    for (int j = 1; j <= d.mp + 1; j++)
      for (int i = 1; i <= d.np + 1; i++) {
        if (j <= d.mp && k <= d.lp) U1(i, j, k) = fn1(i, j, k) + (liner ? R(0) : w1(i, j, k));
        if (i <= d.np && k <= d.lp) U2(i, j, k) = fn2(i, j, k) + (liner ? R(0) : w2(i, j, k));
        if (i <= d.np && j <= d.mp) U3(i, j, k) = fn3(i, j, k) + (liner ? R(0) : w3(i, j, k));
      }
  // psi halo: zero-gradient copy of the old boundary values after the
  // antidiffusion (cp_last_to_halo_xy, :356), Dirichlet values otherwise
  if (!d.bx)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++) {
        X(0, j, k) = liner ? xin(0, j, k) : xin(1, j, k);
        X(d.np + 1, j, k) = liner ? xin(d.np + 1, j, k) : xin(d.np, j, k);
      }
  if (!d.by)
    for (int k = 1; k <= d.lp; k++)
      for (int i = 1; i <= d.np; i++) {
        X(i, 0, k) = liner ? xin(i, 0, k) : xin(i, 1, k);
        X(i, d.mp + 1, k) = liner ? xin(i, d.mp + 1, k) : xin(i, d.mp, k);
      }
  return 0;
}

}  // namespace

extern "C" {

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
void orc_set_literal_sums(int on) { g_literal_sums = on ? 1 : 0; }
int orc_get_threads(void) { return g_threads; }

int orc_advec_dwarf_f64(const orc_grid* g, int opt, int t_adv, int iord, int nonos, double* x,
                        const double* x_lr, const double* x_bt, const double* uadv,
                        const double* vadv, const double* wadv, const double* rhr,
                        const double* rhoadv) {
  return advec<double>(g, opt, t_adv, iord, nonos, x, x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv);
}
int orc_advec_dwarf_f32(const orc_grid* g, int opt, int t_adv, int iord, int nonos, float* x,
                        const float* x_lr, const float* x_bt, const float* uadv, const float* vadv,
                        const float* wadv, const float* rhr, const float* rhoadv) {
  return advec<float>(g, opt, t_adv, iord, nonos, x, x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv);
}
int orc_advec_steps_f64(const orc_grid* g, int n, int opt, int t_adv, int iord, int nonos,
                        double* x, const double* x_lr, const double* x_bt, const double* uadv,
                        const double* vadv, const double* wadv, const double* rhr,
                        const double* rhoadv) {
  for (int s = 0; s < n; s++) {
    int rc = advec<double>(g, opt, t_adv, iord, nonos, x, x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv);
    if (rc) return rc;
  }
  return 0;
}
int orc_advec_steps_f32(const orc_grid* g, int n, int opt, int t_adv, int iord, int nonos,
                        float* x, const float* x_lr, const float* x_bt, const float* uadv,
                        const float* vadv, const float* wadv, const float* rhr,
                        const float* rhoadv) {
  for (int s = 0; s < n; s++) {
    int rc = advec<float>(g, opt, t_adv, iord, nonos, x, x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv);
    if (rc) return rc;
  }
  return 0;
}

int orc_upwind_f64(const orc_grid* g, const double* x, const double* bcx, const double* bcy,
                   const double* uadv, const double* vadv, const double* wadv, const double* rhr_in,
                   const double* h_in, double* xant_out) {
  if (!dims_ok(g)) return -1;
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  const int NX = d.np + 2, NY = d.mp + 2, NZ = d.lp + 2;
  Buf<double> xin(NX, NY, NZ), h(NX, NY, NZ), rhr(NX, NY, NZ), xant(NX, NY, NZ);
  Buf<double> u1(NX + 1, NY, NZ), u2(NX, NY + 1, NZ), u3(NX, NY, NZ + 1);
  load_cell(xin, x, d); load_cell(h, h_in, d); load_cell(rhr, rhr_in, d);
  load_face(u1, uadv, d, 0); load_face(u2, vadv, d, 1); load_face(u3, wadv, d, 2);
  if (!d.bx)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++) {
        xin(0, j, k) = bcx[(j - 1) + (long)d.mp * (k - 1)];
        xin(d.np + 1, j, k) = bcx[(j - 1) + (long)d.mp * (k - 1) + (long)d.mp * d.lp];
      }
  if (!d.by)
    for (int k = 1; k <= d.lp; k++)
      for (int i = 1; i <= d.np; i++) {
        xin(i, 0, k) = bcy[(i - 1) + (long)d.np * (k - 1)];
        xin(i, d.mp + 1, k) = bcy[(i - 1) + (long)d.np * (k - 1) + (long)d.np * d.lp];
      }
  upwind(d, xin, u1, u2, u3, h, rhr, xant);
  V3<double> XO = view<double>(xant_out, d.ih, d.np + 2 * d.ih, d.mp + 2 * d.ih);
  for (int k = 1; k <= d.lp; k++)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) XO(i, j, k) = xant(i, j, k);
  return 0;
}

int orc_rho_gauge_f64(const orc_grid* g, double* ox, double* oy, double* oz, double* u, double* v,
                      double* w, double* u1, double* u2, double* u3, double* x_in, double* x_incomp,
                      const double* h, double* rhoadv, double* rhr, const double* pexe, double* pexr1,
                      double* pexr2, const double* bcx, const double* bcy, double dxi, double dyi,
                      double dzi, double dt, double dt_ratio, int liner) {
  return rho_gauge<double>(g, ox, oy, oz, u, v, w, u1, u2, u3, x_in, x_incomp, h, rhoadv, rhr, pexe,
                           pexr1, pexr2, bcx, bcy, dxi, dyi, dzi, dt, dt_ratio, liner);
}

int orc_tangent_adjoint_f64(const orc_grid* g, int t_adv, int iord, int nonos, int nsteps, const double* x0,
                            const double* bcx, const double* bcy, const double* u1, const double* u2,
                            const double* u3, const double* rhr, const double* h, const double* target,
                            double* J, double* xN, double* gx0, double* gu1, double* gu2, double* gu3,
                            const double* dx0, const double* du1, const double* du2, const double* du3,
                            double* dJ_tl);

// The density step after its predictor (rho_step): u1..u3 hold the C-grid
// Courant numbers on entry and the mass fluxes on exit.
int orc_rho_step_f64(const orc_grid* g, double* u1, double* u2, double* u3, double* x_in, double* x_incomp,
                     const double* h, double* rhoadv, double* rhr, const double* pexe, double* pexr1,
                     double* pexr2, const double* bcx, const double* bcy, int liner) {
  if (!dims_ok(g)) return -1;
  if (!u1 || !u2 || !u3 || !x_in || !x_incomp || !h || !rhoadv || !rhr || !pexe || !pexr1 || !pexr2) return -3;
  if ((!g->ibcx && !bcx) || (!g->ibcy && !bcy)) return -3;
  return rho_step<double>(g, u1, u2, u3, x_in, x_incomp, h, rhoadv, rhr, pexe, pexr1, pexr2, bcx, bcy, liner);
}

// Un-checkpointed FP64 adjoint by reverse-mode AD of the oracle's own step:
// J = 0.5*sum((x_N - target)^2) over the interior after nsteps steps with a
// fixed velocity; gradients with respect to x_0 (interior) and every element
// of u1..u3 (elements the step never reads get zero).  h, rhr, bcx, bcy are
// constants.  Single-threaded (one global tape).
int orc_adjoint_f64(const orc_grid* g, int t_adv, int iord, int nonos, int nsteps, const double* x0,
                    const double* bcx, const double* bcy, const double* u1, const double* u2,
                    const double* u3, const double* rhr, const double* h, const double* target,
                    double* J, double* xN, double* gx0, double* gu1, double* gu2, double* gu3) {
  return orc_tangent_adjoint_f64(g, t_adv, iord, nonos, nsteps, x0, bcx, bcy, u1, u2, u3, rhr, h, target, J,
                                 xN, gx0, gu1, gu2, gu3, nullptr, nullptr, nullptr, nullptr, nullptr);
}

// Same, plus the tangent-linear model on the same tape: with directions
// dx0 (psi-shaped) and du1..du3 (C-grid shaped), dJ_tl receives
// sum((x_N - target) * dx_N), the directional derivative of J by forward
// propagation; the dot-product test compares it with <dx0,gx0> + <du,gu>.
int orc_tangent_adjoint_f64(const orc_grid* g, int t_adv, int iord, int nonos, int nsteps, const double* x0,
                            const double* bcx, const double* bcy, const double* u1, const double* u2,
                            const double* u3, const double* rhr, const double* h, const double* target,
                            double* J, double* xN, double* gx0, double* gu1, double* gu2, double* gu3,
                            const double* dx0, const double* du1, const double* du2, const double* du3,
                            double* dJ_tl) {
  if (!dims_ok(g)) return -1;
  if (!x0 || !u1 || !u2 || !u3 || !rhr || !h || !target || !J || !gx0 || !gu1 || !gu2 || !gu3) return -3;
  const int ih = g->ih;
  const long SX = g->np + 2 * ih, SY = g->mp + 2 * ih, SZ = g->lp + 2 * ih;
  const long nps = SX * SY * SZ, n1 = (SX + 1) * SY * SZ, n2 = SX * (SY + 1) * SZ, n3 = SX * SY * (SZ + 1);
  Tape tape;
  g_tape = &tape;
  const int saved = g_threads;
  g_threads = 1;
  auto var = [&](double v) { AD r(v); r.id = tape.push(-1, 0.0, -1, 0.0); return r; };
  std::vector<AD> X(nps), U1(n1), U2(n2), U3(n3), H(nps), RR(nps);
  std::vector<AD> BX(bcx ? (size_t)g->mp * g->lp * 2 : 0), BY(bcy ? (size_t)g->np * g->lp * 2 : 0);
  std::vector<int> xid(nps, -1);
  auto interior = [&](long e) {
    const long i = e % SX, j = (e / SX) % SY, k = e / (SX * SY);
    return i >= ih && i < ih + g->np && j >= ih && j < ih + g->mp && k >= ih && k < ih + g->lp;
  };
  for (long e = 0; e < nps; e++) {
    X[e] = interior(e) ? var(x0[e]) : AD(x0[e]);
    xid[e] = X[e].id;
    H[e] = AD(h[e]);
    RR[e] = AD(rhr[e]);
  }
  for (long e = 0; e < n1; e++) U1[e] = var(u1[e]);
  for (long e = 0; e < n2; e++) U2[e] = var(u2[e]);
  for (long e = 0; e < n3; e++) U3[e] = var(u3[e]);
  for (size_t e = 0; e < BX.size(); e++) BX[e] = AD(bcx[e]);
  for (size_t e = 0; e < BY.size(); e++) BY[e] = AD(bcy[e]);
  const int uid1 = U1[0].id, uid2 = U2[0].id, uid3 = U3[0].id;
  int rc = 0;
  for (int s = 0; s < nsteps && !rc; s++)
    rc = advec<AD>(g, 4, t_adv, iord, nonos, X.data(), bcx ? BX.data() : nullptr,
                   bcy ? BY.data() : nullptr, U1.data(), U2.data(), U3.data(), RR.data(), H.data());
  if (rc) { g_tape = nullptr; g_threads = saved; return rc; }
  if (dJ_tl && dx0 && du1 && du2 && du3) {
    // forward tangent sweep: tan[n] = da*tan[a] + db*tan[b]; inputs carry the directions
    std::vector<double> tan(tape.a.size(), 0.0);
    for (long e = 0; e < nps; e++)
      if (xid[e] >= 0) tan[xid[e]] = dx0[e];
    for (long e = 0; e < n1; e++) tan[uid1 + e] = du1[e];
    for (long e = 0; e < n2; e++) tan[uid2 + e] = du2[e];
    for (long e = 0; e < n3; e++) tan[uid3 + e] = du3[e];
    for (size_t n = 0; n < tape.a.size(); n++) {
      double t = tan[n];
      if (tape.a[n] >= 0) t += tape.da[n] * tan[tape.a[n]];
      if (tape.b[n] >= 0) t += tape.db[n] * tan[tape.b[n]];
      tan[n] = t;
    }
    double d = 0.0;
    for (long e = 0; e < nps; e++)
      if (interior(e) && X[e].id >= 0) d += (X[e].v - target[e]) * tan[X[e].id];
    *dJ_tl = d;
  }
  std::vector<double> adj(tape.a.size(), 0.0);
  double jsum = 0.0;
  for (long e = 0; e < nps; e++) {
    if (xN) xN[e] = X[e].v;
    if (!interior(e)) continue;
    const double r = X[e].v - target[e];
    jsum += r * r;
    if (X[e].id >= 0) adj[X[e].id] += r;
  }
  *J = 0.5 * jsum;
  for (long n = (long)tape.a.size() - 1; n >= 0; n--) {
    const double an = adj[n];
    if (an == 0.0) continue;
    if (tape.a[n] >= 0) adj[tape.a[n]] += tape.da[n] * an;
    if (tape.b[n] >= 0) adj[tape.b[n]] += tape.db[n] * an;
  }
  for (long e = 0; e < nps; e++) gx0[e] = xid[e] >= 0 ? adj[xid[e]] : 0.0;
  for (long e = 0; e < n1; e++) gu1[e] = adj[uid1 + e];
  for (long e = 0; e < n2; e++) gu2[e] = adj[uid2 + e];
  for (long e = 0; e < n3; e++) gu3[e] = adj[uid3 + e];
  g_tape = nullptr;
  g_threads = saved;
  return 0;
}

// Reverse-mode AD of the density step after its predictor (rho_step): the
// checker of mpdata_rho_gauge_adjoint_*.  The step's outputs, psi (x_in),
// x_incomp, pexr1, pexr2 and rhr on the interior and the mass fluxes u1..u3 on
// the faces 1..n+1, are seeded with the given cotangents (NULL: zero); the
// gradients are with respect to the interior of the input psi, every element
// of the C-grid Courant numbers u1..u3, and the interiors of the x_incomp
// input and of pexe.  h, bcx and bcy are constants.  Single-threaded (one
// global tape).
int orc_rho_adjoint_f64(const orc_grid* g, const double* u1, const double* u2, const double* u3,
                        const double* x_in, const double* x_incomp, const double* h, const double* pexe,
                        const double* bcx, const double* bcy, const double* l_x, const double* l_u1,
                        const double* l_u2, const double* l_u3, const double* l_xinc, const double* l_p1,
                        const double* l_p2, const double* l_rhr, double* g_x, double* g_u1, double* g_u2,
                        double* g_u3, double* g_xinc, double* g_pexe) {
  if (!dims_ok(g)) return -1;
  if (!u1 || !u2 || !u3 || !x_in || !x_incomp || !h || !pexe || !g_x || !g_u1 || !g_u2 || !g_u3 || !g_xinc ||
      !g_pexe)
    return -3;
  if ((!g->ibcx && !bcx) || (!g->ibcy && !bcy)) return -3;
  const int ih = g->ih;
  const long SX = g->np + 2 * ih, SY = g->mp + 2 * ih, SZ = g->lp + 2 * ih;
  const long nps = SX * SY * SZ, n1 = (SX + 1) * SY * SZ, n2 = SX * (SY + 1) * SZ, n3 = SX * SY * (SZ + 1);
  Tape tape;
  g_tape = &tape;
  const int saved = g_threads;
  g_threads = 1;
  auto var = [&](double v) { AD r(v); r.id = tape.push(-1, 0.0, -1, 0.0); return r; };
  auto interior = [&](long e) {
    const long i = e % SX, j = (e / SX) % SY, k = e / (SX * SY);
    return i >= ih && i < ih + g->np && j >= ih && j < ih + g->mp && k >= ih && k < ih + g->lp;
  };
  std::vector<AD> X(nps), XC(nps), H(nps), PE(nps), RA(nps), RO(nps), P1(nps), P2(nps), U1(n1), U2(n2), U3(n3);
  std::vector<AD> BX(bcx ? (size_t)g->mp * g->lp * 2 : 0), BY(bcy ? (size_t)g->np * g->lp * 2 : 0);
  std::vector<int> xid(nps, -1), cid(nps, -1), pid(nps, -1);
  for (long e = 0; e < nps; e++) {
    const bool in = interior(e);
    X[e] = in ? var(x_in[e]) : AD(x_in[e]);
    XC[e] = in ? var(x_incomp[e]) : AD(x_incomp[e]);
    PE[e] = in ? var(pexe[e]) : AD(pexe[e]);
    xid[e] = X[e].id;
    cid[e] = XC[e].id;
    pid[e] = PE[e].id;
    H[e] = AD(h[e]);
  }
  for (long e = 0; e < n1; e++) U1[e] = var(u1[e]);
  for (long e = 0; e < n2; e++) U2[e] = var(u2[e]);
  for (long e = 0; e < n3; e++) U3[e] = var(u3[e]);
  for (size_t e = 0; e < BX.size(); e++) BX[e] = AD(bcx[e]);
  for (size_t e = 0; e < BY.size(); e++) BY[e] = AD(bcy[e]);
  const int uid1 = U1[0].id, uid2 = U2[0].id, uid3 = U3[0].id;
  const int rc = rho_step<AD>(g, U1.data(), U2.data(), U3.data(), X.data(), XC.data(), H.data(), RA.data(),
                              RO.data(), PE.data(), P1.data(), P2.data(), bcx ? BX.data() : nullptr,
                              bcy ? BY.data() : nullptr, 0);
  if (rc) {
    g_tape = nullptr;
    g_threads = saved;
    return rc;
  }
  std::vector<double> adj(tape.a.size(), 0.0);
  auto seed = [&](const AD& a, const double* c, long e) {
    if (c && a.id >= 0) adj[a.id] += c[e];
  };
  for (long e = 0; e < nps; e++) {
    if (!interior(e)) continue;
    seed(X[e], l_x, e);
    seed(XC[e], l_xinc, e);
    seed(P1[e], l_p1, e);
    seed(P2[e], l_p2, e);
    seed(RO[e], l_rhr, e);
  }
  // the mass fluxes: faces 1..n+1 along their own axis
  for (int k = 1; k <= g->lp + 1; k++)
    for (int j = 1; j <= g->mp + 1; j++)
      for (int i = 1; i <= g->np + 1; i++) {
        const long i0 = i - 1 + ih, j0 = j - 1 + ih, k0 = k - 1 + ih;
        if (j <= g->mp && k <= g->lp) seed(U1[i0 + j0 * (SX + 1) + k0 * (SX + 1) * SY], l_u1, i0 + j0 * (SX + 1) + k0 * (SX + 1) * SY);
        if (i <= g->np && k <= g->lp) seed(U2[i0 + j0 * SX + k0 * SX * (SY + 1)], l_u2, i0 + j0 * SX + k0 * SX * (SY + 1));
        if (i <= g->np && j <= g->mp) seed(U3[i0 + j0 * SX + k0 * SX * SY], l_u3, i0 + j0 * SX + k0 * SX * SY);
      }
  for (long n = (long)tape.a.size() - 1; n >= 0; n--) {
    const double an = adj[n];
    if (an == 0.0) continue;
    if (tape.a[n] >= 0) adj[tape.a[n]] += tape.da[n] * an;
    if (tape.b[n] >= 0) adj[tape.b[n]] += tape.db[n] * an;
  }
  for (long e = 0; e < nps; e++) {
    g_x[e] = xid[e] >= 0 ? adj[xid[e]] : 0.0;
    g_xinc[e] = cid[e] >= 0 ? adj[cid[e]] : 0.0;
    g_pexe[e] = pid[e] >= 0 ? adj[pid[e]] : 0.0;
  }
  for (long e = 0; e < n1; e++) g_u1[e] = adj[uid1 + e];
  for (long e = 0; e < n2; e++) g_u2[e] = adj[uid2 + e];
  for (long e = 0; e < n3; e++) g_u3[e] = adj[uid3 + e];
  g_tape = nullptr;
  g_threads = saved;
  return 0;
}

int orc_velprd_f64(const orc_grid* g, double* ox, double* oy, double* oz, double* u, double* v,
                   double* w, const double* h, double dxi, double dyi, double dzi, double dt,
                   double dt_ratio, double* u1, double* u2, double* u3) {
  return velprd<double>(g, ox, oy, oz, u, v, w, h, dxi, dyi, dzi, dt, dt_ratio, u1, u2, u3);
}
int orc_velprd_f32(const orc_grid* g, float* ox, float* oy, float* oz, float* u, float* v,
                   float* w, const float* h, float dxi, float dyi, float dzi, float dt,
                   float dt_ratio, float* u1, float* u2, float* u3) {
  return velprd<float>(g, ox, oy, oz, u, v, w, h, dxi, dyi, dzi, dt, dt_ratio, u1, u2, u3);
}

int orc_compute_courants_f64(const orc_grid* g, int ntimelevel, double* ox, double* oy, double* oz, const double* h,
                             double dxi, double dyi, double dzi, double dt, double* cr) {
  if (!dims_ok(g)) return -1;
  if (ntimelevel != 1 && ntimelevel != 2) return -2;
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  courants<double>(pred_of<double>(d, ox, oy, oz, nullptr, nullptr, nullptr, h), ntimelevel, dxi, dyi, dzi, dt, cr);
  return 0;
}
int orc_compute_courants_f32(const orc_grid* g, int ntimelevel, float* ox, float* oy, float* oz, const float* h,
                             float dxi, float dyi, float dzi, float dt, float* cr) {
  if (!dims_ok(g)) return -1;
  if (ntimelevel != 1 && ntimelevel != 2) return -2;
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  courants<float>(pred_of<float>(d, ox, oy, oz, nullptr, nullptr, nullptr, h), ntimelevel, dxi, dyi, dzi, dt, cr);
  return 0;
}
int orc_velprd_driver_f64(const orc_grid* g, int* nsubsteps, int* nsubsteps_o, int lsubstepping, double* dtn,
                          double* dtnold, int ltimeadapt, int lvertsplit, int lcrdiag_nphlf, double crmaxlim,
                          double dtmax, double* ox, double* oy, double* oz, double* u, double* v, double* w,
                          double* uadv, double* vadv, double* wadv, const double* h, double dxi, double dyi,
                          double dzi, double dt, double* diag) {
  return velprd_driver<double>(g, nsubsteps, nsubsteps_o, lsubstepping, dtn, dtnold, ltimeadapt, lvertsplit,
                               lcrdiag_nphlf, crmaxlim, dtmax, ox, oy, oz, u, v, w, uadv, vadv, wadv, h, dxi,
                               dyi, dzi, dt, diag);
}
int orc_velprd_driver_f32(const orc_grid* g, int* nsubsteps, int* nsubsteps_o, int lsubstepping, float* dtn,
                          float* dtnold, int ltimeadapt, int lvertsplit, int lcrdiag_nphlf, float crmaxlim,
                          float dtmax, float* ox, float* oy, float* oz, float* u, float* v, float* w,
                          float* uadv, float* vadv, float* wadv, const float* h, float dxi, float dyi, float dzi,
                          float dt, double* diag) {
  return velprd_driver<float>(g, nsubsteps, nsubsteps_o, lsubstepping, dtn, dtnold, ltimeadapt, lvertsplit,
                              lcrdiag_nphlf, crmaxlim, dtmax, ox, oy, oz, u, v, w, uadv, vadv, wadv, h, dxi, dyi,
                              dzi, dt, diag);
}

// velprdA_to_C_ver2 (module_velprd.f90:366-520): the C-grid averaging of given
// A-grid Courant numbers, with the one-sided halo extrapolation on open walls.
int orc_a_to_c_f64(const orc_grid* g, double* uadv, double* vadv, double* wadv, double* u1o,
                   double* u2o, double* u3o) {
  if (!dims_ok(g)) return -1;
  const Dims d{g->np, g->mp, g->lp, g->ih, g->ibcx, g->ibcy, g->ibcz};
  const int ih = d.ih, SX = d.np + 2 * ih, SY = d.mp + 2 * ih;
  V3<double> A1 = view<double>(uadv, ih, SX, SY), A2 = view<double>(vadv, ih, SX, SY),
             A3 = view<double>(wadv, ih, SX, SY);
  if (!d.bx)
    for (int k = 1; k <= d.lp; k++)
      for (int j = 1; j <= d.mp; j++) {
        A1(0, j, k) = 2.0 * A1(1, j, k) - A1(2, j, k);
        A1(d.np + 1, j, k) = 2.0 * A1(d.np, j, k) - A1(d.np - 1, j, k);
      }
  if (!d.by)
    for (int k = 1; k <= d.lp; k++)
      for (int i = 1; i <= d.np; i++) {
        A2(i, 0, k) = 2.0 * A2(i, 1, k) - A2(i, 2, k);
        A2(i, d.mp + 1, k) = 2.0 * A2(i, d.mp, k) - A2(i, d.mp - 1, k);
      }
  if (!d.bz)
    for (int j = 1; j <= d.mp; j++)
      for (int i = 1; i <= d.np; i++) {
        A3(i, j, 0) = 2.0 * A3(i, j, 1) - A3(i, j, 2);
        A3(i, j, d.lp + 1) = 2.0 * A3(i, j, d.lp) - A3(i, j, d.lp - 1);
      }
  V3<double> U1 = view<double>(u1o, ih, SX + 1, SY), U2 = view<double>(u2o, ih, SX, SY + 1),
             U3 = view<double>(u3o, ih, SX, SY);
  auto wx = [&](int i) { return d.bx ? (i < 1 ? i + d.np : (i > d.np ? i - d.np : i)) : i; };
  auto wy = [&](int j) { return d.by ? (j < 1 ? j + d.mp : (j > d.mp ? j - d.mp : j)) : j; };
  auto wz = [&](int k) { return d.bz ? (k < 1 ? k + d.lp : (k > d.lp ? k - d.lp : k)) : k; };
  for (int k = 1; k <= d.lp + 1; k++)
    for (int j = 1; j <= d.mp + 1; j++)
      for (int i = 1; i <= d.np + 1; i++) {
        if (j <= d.mp && k <= d.lp) {
          const int ii = (d.bx && i == d.np + 1) ? 1 : i;
          U1(i, j, k) = 0.5 * (A1(ii, j, k) + A1(wx(ii - 1), j, k));
        }
        if (i <= d.np && k <= d.lp) {
          const int jj = (d.by && j == d.mp + 1) ? 1 : j;
          U2(i, j, k) = 0.5 * (A2(i, jj, k) + A2(i, wy(jj - 1), k));
        }
        if (i <= d.np && j <= d.mp) {
          const int kk = (d.bz && k == d.lp + 1) ? 1 : k;
          U3(i, j, k) = 0.5 * (A3(i, j, kk) + A3(i, j, wz(kk - 1)));
        }
      }
  return 0;
}

}  // extern "C"
