// Velocity predictor: velprd_traj0 (module_velprd.f90:15-89), velprdA_to_C
// (:166-364) and the level roll of velprd_driver (velprd_driver.f90:254-270).
// Strict IEEE, same expression order as the reference.
#include "mpdata_common.cuh"
#include "mpdata_stages.cuh"

namespace mpdata {

// n+1/2 momenta times dt/dx into level 1 (module_velprd.f90:60-83)
template <class R>
__global__ void __launch_bounds__(128) k_pred_level(Geo g, long lev, R* ox, R* oy, R* oz, Arr<R> h,
                                                    R gc1, R gc2, R gc3, R r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > g.np || j > g.mp) return;
  const R hc = h.ld(i, j, k);
  R* o[3] = {ox, oy, oz};
  const R gc[3] = {gc1, gc2, gc3};
  // ox/oy/oz point at the logical (1,1,1) of level 0; levels are psi-shaped
  const long off = (long)(i - 1) + (long)(j - 1) * h.sy + (long)(k - 1) * h.sz;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    R* p0 = o[c] + off;
    const R a0 = p0[0] * hc;
    const R a2 = p0[2 * lev];
    const R a1 = a0 + r * (a0 - a2);
    p0[lev] = R(0.5) * (a1 + a0) * gc[c];
  }
}

// C-grid averaging with the open-wall extrapolation 2a(1)-a(2)
// (module_velprd.f90:197-361), then the level roll (velprd_driver.f90:254-270).
template <class R>
__global__ void __launch_bounds__(128) k_pred_cgrid(Geo g, long lev, R* ox, R* oy, R* oz, R* pu, R* pv,
                                                    R* pw, Arr<R> h, Arr<R> u1, Arr<R> u2, Arr<R> u3,
                                                    R r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > g.np + 1 || j > g.mp + 1) return;
  // level-1 views (ox etc. point at the logical (1,1,1) of level 0)
  const Arr<R> A1{ox + lev, h.sy, h.sz}, A2{oy + lev, h.sy, h.sz}, A3{oz + lev, h.sy, h.sz};
  if (j <= g.mp && k <= g.lp) {
    R a, b;
    if (g.bx) {
      const int ii = i > g.np ? 1 : i;
      a = A1.ld(ii, j, k);
      b = A1.ld(wrapi(ii - 1, g.np), j, k);
    } else {
      a = i <= g.np ? A1.ld(i, j, k) : R(2) * A1.ld(g.np, j, k) - A1.ld(g.np - 1, j, k);
      b = i > 1 ? A1.ld(i - 1, j, k) : R(2) * A1.ld(1, j, k) - A1.ld(2, j, k);
      if (i == 1) A1.at(0, j, k) = b;
      if (i == g.np + 1) A1.at(g.np + 1, j, k) = a;
    }
    u1.at(i, j, k) = R(0.5) * (a + b);
  }
  if (i <= g.np && k <= g.lp) {
    R a, b;
    if (g.by) {
      const int jj = j > g.mp ? 1 : j;
      a = A2.ld(i, jj, k);
      b = A2.ld(i, wrapi(jj - 1, g.mp), k);
    } else {
      a = j <= g.mp ? A2.ld(i, j, k) : R(2) * A2.ld(i, g.mp, k) - A2.ld(i, g.mp - 1, k);
      b = j > 1 ? A2.ld(i, j - 1, k) : R(2) * A2.ld(i, 1, k) - A2.ld(i, 2, k);
      if (j == 1) A2.at(i, 0, k) = b;
      if (j == g.mp + 1) A2.at(i, g.mp + 1, k) = a;
    }
    u2.at(i, j, k) = R(0.5) * (a + b);
  }
  if (i <= g.np && j <= g.mp) {
    R a, b;
    if (g.bz) {
      const int kk = k > g.lp ? 1 : k;
      a = A3.ld(i, j, kk);
      b = A3.ld(i, j, wrapi(kk - 1, g.lp));
    } else {
      a = k <= g.lp ? A3.ld(i, j, k) : R(2) * A3.ld(i, j, g.lp) - A3.ld(i, j, g.lp - 1);
      b = k > 1 ? A3.ld(i, j, k - 1) : R(2) * A3.ld(i, j, 1) - A3.ld(i, j, 2);
      if (k == 1) A3.at(i, j, 0) = b;
      if (k == g.lp + 1) A3.at(i, j, g.lp + 1) = a;
    }
    u3.at(i, j, k) = R(0.5) * (a + b);
  }
  if (i <= g.np && j <= g.mp && k <= g.lp) {
    const long off = (long)(i - 1) + (long)(j - 1) * h.sy + (long)(k - 1) * h.sz;
    const R hc = h.ld(i, j, k);
    R* o[3] = {ox, oy, oz};
    R* p[3] = {pu, pv, pw};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (p[c]) {
        R* q = p[c] + off;
        const R p0 = q[0], p2 = q[2 * lev];
        q[lev] = p0 + r * (p0 - p2);
        q[2 * lev] = p0;
      }
      R* q = o[c] + off;
      q[2 * lev] = q[0] * hc;
    }
  }
}

template <class R>
int run_predictor(const PredPlan<R>& P, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 g1((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  const dim3 g2((g.np + 1 + 31) / 32, (g.mp + 1 + 3) / 4, g.lp + 1);
  if (P.prof) P.prof->begin(ST_PRED_LEVEL, s);
  k_pred_level<R><<<g1, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.h, P.gc1, P.gc2, P.gc3, P.dt_ratio);
  if (P.prof) P.prof->end(ST_PRED_LEVEL, s);
  if (P.prof) P.prof->begin(ST_PRED_CGRID, s);
  k_pred_cgrid<R><<<g2, blk, 0, s>>>(g, P.lev, P.ox, P.oy, P.oz, P.u, P.v, P.w, P.h, P.u1, P.u2, P.u3,
                                     P.dt_ratio);
  if (P.prof) P.prof->end(ST_PRED_CGRID, s);
  add_launches(2);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template int run_predictor<double>(const PredPlan<double>&, cudaStream_t);
template int run_predictor<float>(const PredPlan<float>&, cudaStream_t);

}  // namespace mpdata
