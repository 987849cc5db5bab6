// Velocity predictor: velprd_traj0 (module_velprd.f90:15-89), velprdA_to_C
// (:166-364), the level roll of velprd_driver (velprd_driver.f90:254-270),
// and the Courant-number maxima the driver steers substepping and adaptive
// time steps with (common/diagutils.f90:588-672).  Strict IEEE, same
// expression order as the reference.
#include <cmath>

#include "mpdata_common.cuh"
#include "mpdata_stages.cuh"

namespace mpdata {

// n+1/2 momenta times dt/dx into level 1 (module_velprd.f90:60-83):
// 0.5*(a1+a0)*gc in the reference's order.  The halving runs on the integer
// pipe (scale_down); the product by gc is skipped when gc is exactly 1 and is
// another scale_down when gc is 2^-s (FP64).  R1: the time-step ratio r is
// exactly 1, so r*(a0-a2) is a0-a2.  A warp whose densities are all exactly
// 1 takes a0 = ox(level 0) without the product.
template <class R>
struct GcK {
  R k[3];
  int s[3];  // -1: k == 1; s >= 1: k == 2^-s (FP64); 0: multiply
};
template <class R>
GcK<R> gc_factors(R gc1, R gc2, R gc3) {
  GcK<R> f;
  const R gc[3] = {gc1, gc2, gc3};
  for (int c = 0; c < 3; c++) {
    f.k[c] = gc[c];
    int e = 0;
    const double m = std::frexp((double)gc[c], &e);  // gc = m*2^e, m in [0.5, 1)
    f.s[c] = gc[c] == R(1) ? -1 : (sizeof(R) == 8 && m == 0.5 && 1 - e >= 1 && 1 - e <= 60) ? 1 - e : 0;
  }
  return f;
}
__device__ __forceinline__ double mul_gc(double x, double k, int s) {
  return s < 0 ? x : (s ? scale_down(x, s, k) : x * k);
}
__device__ __forceinline__ float mul_gc(float x, float k, int s) { return s < 0 ? x : x * k; }

template <class R, bool U, bool R1>
__device__ __forceinline__ void pred_level_cell(long lev, long off, R* ox, R* oy, R* oz, R hc, const GcK<R>& gc,
                                                R r) {
  R* o[3] = {ox, oy, oz};
  // the six loads first: a store could alias them as far as the compiler knows
  R l0[3], l2[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    l0[c] = o[c][off];
    l2[c] = o[c][off + 2 * lev];
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const R a0 = U ? l0[c] : l0[c] * hc;
    const R a1 = a0 + (R1 ? a0 - l2[c] : r * (a0 - l2[c]));
    o[c][off + lev] = mul_gc(scale_down<1>(a1 + a0), gc.k[c], gc.s[c]);
  }
}

// True on every lane when each live lane's density is exactly 1 (FP64; FP32
// kernels keep the products).  Called by all 32 lanes before any returns.
template <class R>
__device__ __forceinline__ bool warp_unit_h(bool live, const Arr<R>& h, int i, int j, int k) {
  if constexpr (sizeof(R) == 8) {
    return __all_sync(0xffffffffu, !live || is_one(h.ld(i, j, k)));
  } else {
    return false;
  }
}

template <class R, bool R1>
__global__ void __launch_bounds__(128) k_pred_level(Geo g, long lev, R* ox, R* oy, R* oz, Arr<R> h,
                                                    GcK<R> gc, R r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  const bool live = i <= g.np && j <= g.mp;
  const bool unit = warp_unit_h<R>(live, h, i, j, k);
  if (!live) return;
  // ox/oy/oz point at the logical (1,1,1) of level 0; levels are psi-shaped
  const long off = (long)(i - 1) + (long)(j - 1) * h.sy + (long)(k - 1) * h.sz;
  if (unit)
    pred_level_cell<R, true, R1>(lev, off, ox, oy, oz, R(1), gc, r);
  else
    pred_level_cell<R, false, R1>(lev, off, ox, oy, oz, h.ld(i, j, k), gc, r);
}

// C-grid averaging with the open-wall extrapolation 2a(1)-a(2)
// (module_velprd.f90:197-361), then the level roll (velprd_driver.f90:254-270).
// The level roll of velprd_driver.f90:254-270 for cell (i,j,k): physical
// velocities extrapolated into level 1 and copied into level 2, and the
// level-0 momenta times h stored in level 2 for the next step.
template <class R, bool U = false>
__device__ __forceinline__ void roll_cell(long lev, R* ox, R* oy, R* oz, R* pu, R* pv, R* pw, const Arr<R>& h,
                                          R r, int i, int j, int k) {
  const long off = (long)(i - 1) + (long)(j - 1) * h.sy + (long)(k - 1) * h.sz;
  const R hc = U ? R(1) : h.ld(i, j, k);
  R* o[3] = {ox, oy, oz};
  R* p[3] = {pu, pv, pw};
  R q0[3], p0[3] = {R(0), R(0), R(0)}, p2[3] = {R(0), R(0), R(0)};
#pragma unroll
  for (int c = 0; c < 3; c++) {  // loads first
    q0[c] = o[c][off];
    if (p[c]) {
      p0[c] = p[c][off];
      p2[c] = p[c][off + 2 * lev];
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    if (p[c]) {
      p[c][off + lev] = p0[c] + r * (p0[c] - p2[c]);
      p[c][off + 2 * lev] = p0[c];
    }
    o[c][off + 2 * lev] = U ? q0[c] : q0[c] * hc;
  }
}

template <class R, bool ROLL>
__global__ void __launch_bounds__(128) k_pred_cgrid(Geo g, long lev, R* ox, R* oy, R* oz, R* pu, R* pv,
                                                    R* pw, Arr<R> h, Arr<R> u1, Arr<R> u2, Arr<R> u3,
                                                    R r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  const bool rl = ROLL && i <= g.np && j <= g.mp && k <= g.lp;
  const bool unit = ROLL && warp_unit_h<R>(rl, h, i, j, k);
  if (i > g.np + 1 || j > g.mp + 1) return;
  // level-1 views (ox etc. point at the logical (1,1,1) of level 0)
  const Arr<R> A1{ox + lev, h.sy, h.sz}, A2{oy + lev, h.sy, h.sz}, A3{oz + lev, h.sy, h.sz};
  // every face's loads, then its stores (a store would fence later loads)
  const bool e1 = j <= g.mp && k <= g.lp, e2 = i <= g.np && k <= g.lp, e3 = i <= g.np && j <= g.mp;
  R a1 = R(0), b1 = R(0), a2 = R(0), b2 = R(0), a3 = R(0), b3 = R(0);
  if (e1) {
    if (g.bx) {
      const int ii = i > g.np ? 1 : i;
      a1 = A1.ld(ii, j, k);
      b1 = A1.ld(wrapi(ii - 1, g.np), j, k);
    } else {
      a1 = i <= g.np ? A1.ld(i, j, k) : R(2) * A1.ld(g.np, j, k) - A1.ld(g.np - 1, j, k);
      b1 = i > 1 ? A1.ld(i - 1, j, k) : R(2) * A1.ld(1, j, k) - A1.ld(2, j, k);
    }
  }
  if (e2) {
    if (g.by) {
      const int jj = j > g.mp ? 1 : j;
      a2 = A2.ld(i, jj, k);
      b2 = A2.ld(i, wrapi(jj - 1, g.mp), k);
    } else {
      a2 = j <= g.mp ? A2.ld(i, j, k) : R(2) * A2.ld(i, g.mp, k) - A2.ld(i, g.mp - 1, k);
      b2 = j > 1 ? A2.ld(i, j - 1, k) : R(2) * A2.ld(i, 1, k) - A2.ld(i, 2, k);
    }
  }
  if (e3) {
    if (g.bz) {
      const int kk = k > g.lp ? 1 : k;
      a3 = A3.ld(i, j, kk);
      b3 = A3.ld(i, j, wrapi(kk - 1, g.lp));
    } else {
      a3 = k <= g.lp ? A3.ld(i, j, k) : R(2) * A3.ld(i, j, g.lp) - A3.ld(i, j, g.lp - 1);
      b3 = k > 1 ? A3.ld(i, j, k - 1) : R(2) * A3.ld(i, j, 1) - A3.ld(i, j, 2);
    }
  }
  if (e1) {
    if (!g.bx) {
      if (i == 1) A1.at(0, j, k) = b1;
      if (i == g.np + 1) A1.at(g.np + 1, j, k) = a1;
    }
    u1.at(i, j, k) = scale_down<1>(a1 + b1);
  }
  if (e2) {
    if (!g.by) {
      if (j == 1) A2.at(i, 0, k) = b2;
      if (j == g.mp + 1) A2.at(i, g.mp + 1, k) = a2;
    }
    u2.at(i, j, k) = scale_down<1>(a2 + b2);
  }
  if (e3) {
    if (!g.bz) {
      if (k == 1) A3.at(i, j, 0) = b3;
      if (k == g.lp + 1) A3.at(i, j, g.lp + 1) = a3;
    }
    u3.at(i, j, k) = scale_down<1>(a3 + b3);
  }
  if (rl) {
    if (unit)
      roll_cell<R, true>(lev, ox, oy, oz, pu, pv, pw, h, r, i, j, k);
    else
      roll_cell<R>(lev, ox, oy, oz, pu, pv, pw, h, r, i, j, k);
  }
}

// SMs of the current device (queried once).
int num_sms() {
  static int n = 0;
  if (n < 1) {
    int dev = 0, v = 0;
    n = (cudaGetDevice(&dev) == cudaSuccess &&
         cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            ? v
            : 152;
  }
  return n;
}

// The C-grid averaging of level 1 (velprdA_to_C, module_velprd.f90:197-361)
// as a march up the z columns: each thread owns the (i, j) column of a chunk
// of planes and keeps the level-1 value of the plane below in a register, so
// every plane is read once for the z faces.  The thread of the last cell in x
// (y) also forms the face np+1 (mp+1), and the top chunk the faces lp+1.
// Faces, wall extrapolations 2a(1)-a(2) and their halo writes are those of
// k_pred_cgrid, expression for expression.
template <class R>
__global__ void __launch_bounds__(256, 6) k_pred_cgrid_z(Geo g, long lev, R* ox, R* oy, R* oz, Arr<R> h, Arr<R> u1,
                                                      Arr<R> u2, Arr<R> u3, int kchunk) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int kb = blockIdx.z * kchunk + 1;
  if (i > g.np || j > g.mp || kb > g.lp) return;
  const int ke = min(g.lp, kb + kchunk - 1);
  const Arr<R> A1{ox + lev, h.sy, h.sz}, A2{oy + lev, h.sy, h.sz}, A3{oz + lev, h.sy, h.sz};
  const bool xe = i == g.np, ye = j == g.mp;
  // level 1 below the chunk: the lower value of face kb
  R b3;
  if (kb > 1)
    b3 = A3.ld(i, j, kb - 1);
  else
    b3 = g.bz ? A3.ld(i, j, g.lp) : R(2) * A3.ld(i, j, 1) - A3.ld(i, j, 2);
  if (!g.bz && kb == 1) A3.at(i, j, 0) = b3;
  for (int k = kb; k <= ke; k++) {
    const R a1 = A1.ld(i, j, k);
    const R b1 = i > 1 ? A1.ld(i - 1, j, k) : (g.bx ? A1.ld(g.np, j, k) : R(2) * A1.ld(1, j, k) - A1.ld(2, j, k));
    const R a2 = A2.ld(i, j, k);
    const R b2 = j > 1 ? A2.ld(i, j - 1, k) : (g.by ? A2.ld(i, g.mp, k) : R(2) * A2.ld(i, 1, k) - A2.ld(i, 2, k));
    const R a3 = A3.ld(i, j, k);
    R a1e = R(0), a2e = R(0);
    if (xe) a1e = g.bx ? A1.ld(1, j, k) : R(2) * A1.ld(g.np, j, k) - A1.ld(g.np - 1, j, k);
    if (ye) a2e = g.by ? A2.ld(i, 1, k) : R(2) * A2.ld(i, g.mp, k) - A2.ld(i, g.mp - 1, k);
    if (!g.bx && i == 1) A1.at(0, j, k) = b1;
    if (!g.by && j == 1) A2.at(i, 0, k) = b2;
    u1.at(i, j, k) = scale_down<1>(a1 + b1);
    u2.at(i, j, k) = scale_down<1>(a2 + b2);
    u3.at(i, j, k) = scale_down<1>(a3 + b3);
    if (xe) {
      if (!g.bx) A1.at(g.np + 1, j, k) = a1e;
      u1.at(g.np + 1, j, k) = scale_down<1>(a1e + a1);
    }
    if (ye) {
      if (!g.by) A2.at(i, g.mp + 1, k) = a2e;
      u2.at(i, g.mp + 1, k) = scale_down<1>(a2e + a2);
    }
    b3 = a3;
  }
  if (ke == g.lp) {  // the top faces lp+1
    const R a3e = g.bz ? A3.ld(i, j, 1) : R(2) * A3.ld(i, j, g.lp) - A3.ld(i, j, g.lp - 1);
    if (!g.bz) A3.at(i, j, g.lp + 1) = a3e;
    u3.at(i, j, g.lp + 1) = scale_down<1>(a3e + b3);
  }
}

// velprd_traj0 and the driver's level roll in one pass over the cells (the
// whole predictor's first launch): the roll reads only the cell's own
// level-0 momenta and density, which the n+1/2 momenta read too, and writes
// level 2 after the cell's level 2 has been read, so the C-grid averaging
// that follows reads level 1 alone.
template <class R, bool R1>
__global__ void __launch_bounds__(128) k_pred_level_roll(Geo g, long lev, R* ox, R* oy, R* oz, R* pu, R* pv,
                                                         R* pw, Arr<R> h, GcK<R> gc, R r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  const bool live = i <= g.np && j <= g.mp;
  const bool unit = warp_unit_h<R>(live, h, i, j, k);
  if (!live) return;
  const long off = (long)(i - 1) + (long)(j - 1) * h.sy + (long)(k - 1) * h.sz;
  if (unit) {
    pred_level_cell<R, true, R1>(lev, off, ox, oy, oz, R(1), gc, r);
    roll_cell<R, true>(lev, ox, oy, oz, pu, pv, pw, h, r, i, j, k);
  } else {
    pred_level_cell<R, false, R1>(lev, off, ox, oy, oz, h.ld(i, j, k), gc, r);
    roll_cell<R>(lev, ox, oy, oz, pu, pv, pw, h, r, i, j, k);
  }
}

template <class R>
__global__ void __launch_bounds__(128) k_pred_roll(Geo g, long lev, R* ox, R* oy, R* oz, R* pu, R* pv, R* pw,
                                                   Arr<R> h, R r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > g.np || j > g.mp) return;
  roll_cell<R>(lev, ox, oy, oz, pu, pv, pw, h, r, i, j, k);
}

// ---- adjoint of the predictor ----------------------------------------------
// The predictor is linear in the momenta of levels 0 and 2 (h and the time
// steps held fixed): per component, a0 = l0*h, a1 = a0 + r*(a0 - l2),
// A = (a1 + a0)*hg (level 1, module_velprd.f90:60-83), u(f) = 0.5*(A(f) + A(f-1))
// on the C grid with the periodic wrap or the open-wall extrapolation
// 2A(1) - A(2) (:197-361), and the roll writes l0*h into level 2
// (velprd_driver.f90:254-270).  Its transpose, gathered per cell (no atomics):
// dJ/dA(c) collects the faces that read A(c), then dJ/dl0 += (2 + r)*hg*h*dJ/dA
// + h*dJ/d(level 2 written), and dJ/d(level 2 read) = -r*hg*dJ/dA.

// dJ/dA at cell c of an axis of n cells from the face gradients gf(1..n+1).
template <class R, class F>
__device__ __forceinline__ R face_gather(const F& gf, int c, int n, bool per) {
  R s = R(0.5) * (gf(c) + gf(c + 1));  // face c reads A(c) as its upper cell, face c+1 as its lower
  if (per) {
    if (c == n) s = s + R(0.5) * gf(1);      // face 1's lower cell wraps to n
    if (c == 1) s = s + R(0.5) * gf(n + 1);  // face n+1 is face 1: its upper cell is 1
  } else {
    if (c == 1) s = s + gf(1);               // face 1's lower value 2A(1) - A(2)
    if (c == 2) s = s - R(0.5) * gf(1);
    if (c == n) s = s + gf(n + 1);           // face n+1's upper value 2A(n) - A(n-1)
    if (c == n - 1) s = s - R(0.5) * gf(n + 1);
  }
  return s;
}

// gx/gy/gz: gradient level stacks laid out as ox/oy/oz (logical (1,1,1) of
// level 0); gu1..gu3: dJ/du on the C grid.  In: level 1 = dJ/d(level 1),
// level 2 = dJ/d(level 2 as the roll wrote it); out: level 0 accumulates
// dJ/d(level 0), level 2 = dJ/d(level 2 as the predictor read it).
template <class R>
__global__ void __launch_bounds__(128) k_pred_adjoint(Geo g, long lev, R* gx, R* gy, R* gz, Arr<R> h, Arr<R> gu1,
                                                      Arr<R> gu2, Arr<R> gu3, R hg1, R hg2, R hg3, R r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > g.np || j > g.mp) return;
  const long off = (long)(i - 1) + (long)(j - 1) * h.sy + (long)(k - 1) * h.sz;
  const R hc = h.ld(i, j, k);
  const R ga[3] = {face_gather<R>([&](int f) { return gu1.ld(f, j, k); }, i, g.np, g.bx != 0),
                   face_gather<R>([&](int f) { return gu2.ld(i, f, k); }, j, g.mp, g.by != 0),
                   face_gather<R>([&](int f) { return gu3.ld(i, j, f); }, k, g.lp, g.bz != 0)};
  R* o[3] = {gx, gy, gz};
  const R hg[3] = {hg1, hg2, hg3};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const R a = ga[c] + o[c][off + lev];  // plus dJ/d(level 1) itself
    const R g2 = o[c][off + 2 * lev];
    o[c][off] = o[c][off] + (R(2) + r) * hg[c] * hc * a + hc * g2;
    o[c][off + 2 * lev] = -r * hg[c] * a;
  }
}

template <class R>
int run_pred_adjoint(const PredPlan<R>& P, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 grd((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  k_pred_adjoint<R><<<grd, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.h, P.u1, P.u2, P.u3, R(0.5) * P.gc1,
                                        R(0.5) * P.gc2, R(0.5) * P.gc3, P.dt_ratio);
  add_launches(1);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
template int run_pred_adjoint<double>(const PredPlan<double>&, cudaStream_t);
template int run_pred_adjoint<float>(const PredPlan<float>&, cudaStream_t);

// compute_courants (common/diagutils.f90:588-672): the maxima over the
// interior of |a_x|+|a_y|+|a_z|, the three pair sums and the three
// components, where a = gc*ox(level 0) (LEV2 false) or ox(level 1)/h (LEV2
// true, as dinv=1/h then a product).  A maximum does not depend on the order
// it is taken in, so per-thread maxima over order keys, a warp shuffle, a
// shared-memory fold and one 64-bit atomicMax per block give exactly the
// serial result.  keys[c] holds the unsigned order key of maximum c.
__device__ __forceinline__ unsigned long long ukey(double x) {
  return (unsigned long long)okey(x) ^ 0x8000000000000000ULL;
}

template <class R, bool LEV2>
__global__ void __launch_bounds__(256) k_courants(Geo g, const R* ox, const R* oy, const R* oz, Arr<R> h, R gc1,
                                                  R gc2, R gc3, unsigned long long* keys) {
  unsigned long long m[7];
#pragma unroll
  for (int c = 0; c < 7; c++) m[c] = 0ULL;  // below the key of every number
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i <= g.np && j <= g.mp) {
    for (int k = blockIdx.z + 1; k <= g.lp; k += gridDim.z) {
      const long off = (long)(i - 1) + (long)(j - 1) * h.sy + (long)(k - 1) * h.sz;
      R a, b, c;
      if (LEV2) {
        const R dinv = R(1) / h.p[off];
        a = fabs(ox[off] * dinv);
        b = fabs(oy[off] * dinv);
        c = fabs(oz[off] * dinv);
      } else {
        a = fabs(gc1 * ox[off]);
        b = fabs(gc2 * oy[off]);
        c = fabs(gc3 * oz[off]);
      }
      const R v[7] = {a + b + c, a + b, a + c, b + c, a, b, c};
#pragma unroll
      for (int q = 0; q < 7; q++) {
        const unsigned long long kq = ukey((double)v[q]);
        m[q] = kq > m[q] ? kq : m[q];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 7; q++)
    for (int d = 16; d > 0; d >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, m[q], d);
      m[q] = o > m[q] ? o : m[q];
    }
  __shared__ unsigned long long sm[8][7];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, warp = tid >> 5, nw = (blockDim.x * blockDim.y) >> 5;
  if ((tid & 31) == 0)
#pragma unroll
    for (int q = 0; q < 7; q++) sm[warp][q] = m[q];
  __syncthreads();
  if (tid < 7) {
    unsigned long long r = sm[0][tid];
    for (int w = 1; w < nw; w++) r = sm[w][tid] > r ? sm[w][tid] : r;
    atomicMax(keys + tid, r);
  }
}

// wadv = 0.5*wadv over its first lp+2*ih planes, halo included
// (FullXYZDomainWithHaloLoopDC, velprd_driver.f90:250-252)
template <class R>
__global__ void k_halve(R* p, long n) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    p[t] = R(0.5) * p[t];
}

template <class R>
int run_pred_parts(const PredPlan<R>& P, bool level, bool cgrid, bool roll, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 g1((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  const dim3 g2((g.np + 1 + 31) / 32, (g.mp + 1 + 3) / 4, g.lp + 1);
  int n = 0;
  if (level) {
    if (P.prof) P.prof->begin(ST_PRED_LEVEL, s);
    const GcK<R> gc = gc_factors(P.gc1, P.gc2, P.gc3);
    if (P.dt_ratio == R(1))
      k_pred_level<R, true><<<g1, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.h, gc, P.dt_ratio);
    else
      k_pred_level<R, false><<<g1, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.h, gc, P.dt_ratio);
    if (P.prof) P.prof->end(ST_PRED_LEVEL, s);
    n++;
  }
  if (cgrid) {
    if (P.prof) P.prof->begin(ST_PRED_CGRID, s);
    if (roll)
      k_pred_cgrid<R, true><<<g2, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.u, P.v, P.w, P.h, P.u1, P.u2, P.u3,
                                               P.dt_ratio);
    else
      k_pred_cgrid<R, false><<<g2, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.u, P.v, P.w, P.h, P.u1, P.u2, P.u3,
                                                P.dt_ratio);
    if (P.prof) P.prof->end(ST_PRED_CGRID, s);
    n++;
  } else if (roll) {
    k_pred_roll<R><<<g1, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.u, P.v, P.w, P.h, P.dt_ratio);
    n++;
  }
  add_launches(n);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

// The whole predictor: n+1/2 momenta and level roll in one launch, then the
// C-grid averaging of level 1.
template <class R>
int run_predictor(const PredPlan<R>& P, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 g1((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  const dim3 g2((g.np + 1 + 31) / 32, (g.mp + 1 + 3) / 4, g.lp + 1);
  const GcK<R> gc = gc_factors(P.gc1, P.gc2, P.gc3);
  if (P.prof) P.prof->begin(ST_PRED_LEVEL, s);
  if (P.dt_ratio == R(1))
    k_pred_level_roll<R, true><<<g1, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.u, P.v, P.w, P.h, gc,
                                                 P.dt_ratio);
  else
    k_pred_level_roll<R, false><<<g1, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.u, P.v, P.w, P.h, gc,
                                                  P.dt_ratio);
  if (P.prof) P.prof->end(ST_PRED_LEVEL, s);
  if (P.prof) P.prof->begin(ST_PRED_CGRID, s);
  if constexpr (sizeof(R) == 4) {
    // FP32: the z-march (0.188 against 0.226 ms per step at 512x512x128), about
    // four waves of the 6 resident 256-thread blocks per SM (40 registers)
    const int gx = (g.np + 31) / 32, gy = (g.mp + 7) / 8;
    int nch = (4 * 6 * num_sms() + gx * gy - 1) / (gx * gy);
    nch = nch < 1 ? 1 : (nch > g.lp ? g.lp : nch);
    const int kchunk = (g.lp + nch - 1) / nch;
    const dim3 grid(gx, gy, (g.lp + kchunk - 1) / kchunk);
    k_pred_cgrid_z<R><<<grid, dim3(32, 8, 1), 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.h, P.u1, P.u2, P.u3, kchunk);
  } else {
    // FP64: the per-cell kernel (0.272 against the z-march's 0.301 ms)
    k_pred_cgrid<R, false><<<g2, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.u, P.v, P.w, P.h, P.u1, P.u2, P.u3,
                                              P.dt_ratio);
  }
  if (P.prof) P.prof->end(ST_PRED_CGRID, s);
  add_launches(2);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template <class R>
int run_courants(const PredPlan<R>& P, int level, R dxi, R dyi, R dzi, R dt, unsigned long long* keys,
                 cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 8, 1);
  const int gx = (g.np + 31) / 32, gy = (g.mp + 7) / 8;
  int gz = 1216 / (gx * gy);
  gz = gz < 1 ? 1 : (gz > g.lp ? g.lp : gz);
  const dim3 grid(gx, gy, gz);
  if (level == 2)
    k_courants<R, true><<<grid, blk, 0, s>>>(g, P.ox + P.lev, P.oy + P.lev, P.oz + P.lev, P.h, R(0), R(0), R(0),
                                             keys);
  else  // diagutils.f90:624-626
    k_courants<R, false><<<grid, blk, 0, s>>>(g, P.ox, P.oy, P.oz, P.h, dt * dxi, dt * dyi, dt * dzi, keys);
  add_launches(1);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template <class R>
int run_halve(R* p, long n, cudaStream_t s) {
  k_halve<R><<<1216, 256, 0, s>>>(p, n);
  add_launches(1);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template int run_predictor<double>(const PredPlan<double>&, cudaStream_t);
template int run_predictor<float>(const PredPlan<float>&, cudaStream_t);
template int run_pred_parts<double>(const PredPlan<double>&, bool, bool, bool, cudaStream_t);
template int run_pred_parts<float>(const PredPlan<float>&, bool, bool, bool, cudaStream_t);
template int run_courants<double>(const PredPlan<double>&, int, double, double, double, double,
                                  unsigned long long*, cudaStream_t);
template int run_courants<float>(const PredPlan<float>&, int, float, float, float, float, unsigned long long*,
                                 cudaStream_t);
template int run_halve<double>(double*, long, cudaStream_t);
template int run_halve<float>(float*, long, cudaStream_t);

}  // namespace mpdata
