// Shared device-side definitions of the MPDATA step: grid geometry, array
// views over the reference's Fortran layout, boundary index maps and the
// MPDATA point operators (advection/src_algorithms/mpdataoperators.inc:50-96).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mpdata {

// Grid geometry and boundary flags (1 = periodic axis).
struct Geo {
  int np, mp, lp, ih;
  int bx, by, bz;
};

// View of a 3-D Fortran-ordered array; p points at the logical element
// (1,1,1), so halo elements sit at negative offsets inside the caller's
// allocation.  Indices are the reference's 1-based (i,j,k).
template <class R>
struct Arr {
  R* p;
  long sy, sz;
  __device__ __forceinline__ R ld(int i, int j, int k) const {
    return p[(long)(i - 1) + (long)(j - 1) * sy + (long)(k - 1) * sz];
  }
  __device__ __forceinline__ R& at(int i, int j, int k) const {
    return p[(long)(i - 1) + (long)(j - 1) * sy + (long)(k - 1) * sz];
  }
};

// Caller arrays with halo width ih: extents (n0, n1, *) along x and y.
template <class R>
inline Arr<R> caller_view(R* base, int ih, int n0, int n1) {
  const long sy = n0, sz = (long)n0 * n1;
  return Arr<R>{base + ih + ih * sy + ih * sz, sy, sz};
}
// Workspace scratch: interior cells (or faces 1..n along the own axis), no halo.
template <class R>
inline Arr<R> scratch_view(R* base, const Geo& g) {
  return Arr<R>{base, (long)g.np, (long)g.np * g.mp};
}

// ---- index maps for reads one cell outside [1, n] ----
__device__ __forceinline__ int wrapi(int i, int n) { return i < 1 ? i + n : (i > n ? i - n : i); }
// reflection about the first/last interior cell: x(0)=x(2), x(n+1)=x(n-1)
// (cp_scnd_last_to_halo_xy_fulld, mpdataoperators.inc:479-513)
__device__ __forceinline__ int refl(int i, int n) { return i < 1 ? 2 - i : (i > n ? 2 * n - i : i); }
// zero gradient: x(0)=x(1), x(n+1)=x(n) (cp_last_to_halo_xy, mpdataoperators.inc:551-584)
__device__ __forceinline__ int clampi(int i, int n) { return i < 1 ? 1 : (i > n ? n : i); }

// ---- point operators (device forms of mpdataoperators.inc:50-96) ----
template <class R> __device__ __forceinline__ R pp(R y) { return y > R(0) ? y : R(0); }
template <class R> __device__ __forceinline__ R pn(R y) { return y < R(0) ? -y : R(0); }
template <class R> __device__ __forceinline__ R mx2(R a, R b) { return a > b ? a : b; }
template <class R> __device__ __forceinline__ R mn2(R a, R b) { return a < b ? a : b; }
template <class R> __device__ __forceinline__ R donor(R y1, R y2, R a) { return pp(a) * y1 - pn(a) * y2; }
template <class R> __device__ __forceinline__ R vdyf(R x1, R x2, R a, R rinv) {
  return (fabs(a) - a * a * rinv) * (x2 - x1) * R(0.5);
}
template <class R> __device__ __forceinline__ R rat4(R z0, R z1, R z2, R z3) {
  return ((z3 + z2) - (z1 + z0)) * R(0.25);
}
template <class R> __device__ __forceinline__ R vdyfa(R x1, R x2, R a, R rinv, R ep) {
  return (fabs(a) - a * a * rinv) * (fabs(x2) - fabs(x1)) / (fabs(x2) + fabs(x1) + ep);
}
template <class R> __device__ __forceinline__ R vcorra(R a, R b, R y1, R y2, R rinv) {
  return -(R(0.125) * a * b * y1 * rinv / y2);
}
template <class R> __device__ __forceinline__ R possign(R x) { return signbit(x) ? R(0) : R(1); }
template <class R> __device__ __forceinline__ R min3(R a, R b) { return mn2(mn2(R(1), a), b); }

// ep_nonos (common/epsilons.f90:3)
template <class R> struct Eps;
template <> struct Eps<double> { static constexpr double v = 1e-10; };
template <> struct Eps<float> { static constexpr float v = 1e-10f; };

}  // namespace mpdata
