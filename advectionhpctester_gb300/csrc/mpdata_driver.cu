// Courant control of the velocity predictor: velprd_driver
// (advection/src_algorithms/velprd_driver.f90:16-270) and compute_courants
// (common/diagutils.f90:588-672).
//
// The driver is host control flow around four device pieces: the n+1/2
// momenta (velprd_traj0_adapt_dt), the C-grid averaging (velprdA_to_C), the
// seven Courant maxima (one reduction kernel, read back with one stream
// synchronisation, as the reference's globmax synchronises) and the final
// level roll.  Its scalar arithmetic runs in the field precision R, as the
// reference's REAL(euwp) scalars do; the reference's default-kind literals
// (0.1, 0.99, 0.*n+1) keep their single-precision values.  Its STOPs become
// error codes, and every loop that the reference could spin forever (a
// non-finite Courant number) stops after a fixed number of rounds.
#include <cmath>
#include <cstring>
#include <limits>

#include "mpdata.h"
#include "mpdata_common.cuh"
#include "mpdata_stages.cuh"

namespace mpdata {
int grid_ok(const mpdata_grid* g);  // mpdata_capi.cu
}

using namespace mpdata;

namespace {

constexpr int kMaxRounds = 10000;

// unsigned order key of a double (the device side's okey with the sign bit flipped)
unsigned long long host_ukey(double x) {
  long long b;
  std::memcpy(&b, &x, 8);
  const long long k = b ^ ((b >> 63) & 0x7fffffffffffffffLL);
  return (unsigned long long)k ^ 0x8000000000000000ULL;
}
double host_from_ukey(unsigned long long u) {
  const long long k = (long long)(u ^ 0x8000000000000000ULL);
  const long long b = k ^ ((k >> 63) & 0x7fffffffffffffffLL);
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}

template <class R>
struct Drv {
  PredPlan<R> P;
  unsigned long long* keys = nullptr;  // device, 7 order keys
  cudaStream_t s = nullptr;
  R cr[7];
  ~Drv() {
    if (keys) cudaFreeAsync(keys, s);
  }
};

template <class R>
PredPlan<R> plan_of(const mpdata_grid& g, R* ox, R* oy, R* oz, R* u, R* v, R* w, const R* h, R* uadv, R* vadv,
                    R* wadv) {
  const int ih = g.ih;
  const int sx = g.np + 2 * ih, sy = g.mp + 2 * ih, sz = g.lp + 2 * ih;
  const long off = ih + (long)ih * sx + (long)ih * sx * sy;
  PredPlan<R> P;
  P.g = Geo{g.np, g.mp, g.lp, g.ih, g.ibcx, g.ibcy, g.ibcz};
  P.lev = (long)sx * sy * sz;
  P.ox = ox + off;
  P.oy = oy + off;
  P.oz = oz + off;
  P.u = u ? u + off : nullptr;
  P.v = v ? v + off : nullptr;
  P.w = w ? w + off : nullptr;
  P.h = caller_view<R>(const_cast<R*>(h), ih, sx, sy);
  if (uadv) P.u1 = caller_view<R>(uadv, ih, sx + 1, sy);
  if (vadv) P.u2 = caller_view<R>(vadv, ih, sx, sy + 1);
  if (wadv) P.u3 = caller_view<R>(wadv, ih, sx, sy);
  P.gc1 = P.gc2 = P.gc3 = R(0);
  P.dt_ratio = R(1);
  P.prof = nullptr;
  return P;
}

// compute_courants into d.cr (cr3d, crxy, crxz, cryz, crx, cry, crz)
template <class R>
int courants(Drv<R>& d, int level, R dxi, R dyi, R dzi, R dt) {
  unsigned long long init[7], out[7];
  const unsigned long long k0 = host_ukey((double)(-std::numeric_limits<R>::max()));  // -HUGE (:611-617)
  for (int c = 0; c < 7; c++) init[c] = k0;
  if (cudaMemcpyAsync(d.keys, init, sizeof init, cudaMemcpyHostToDevice, d.s) != cudaSuccess) return MPDATA_E_CUDA;
  if (run_courants<R>(d.P, level, dxi, dyi, dzi, dt, d.keys, d.s)) return MPDATA_E_CUDA;
  if (cudaMemcpyAsync(out, d.keys, sizeof out, cudaMemcpyDeviceToHost, d.s) != cudaSuccess) return MPDATA_E_CUDA;
  if (cudaStreamSynchronize(d.s) != cudaSuccess) return MPDATA_E_CUDA;
  for (int c = 0; c < 7; c++) d.cr[c] = (R)host_from_ukey(out[c]);
  return MPDATA_OK;
}

template <class R>
int traj0(Drv<R>& d, bool with_cgrid, R dt, R dt_ratio, R dxi, R dyi, R dzi) {
  d.P.gc1 = dt * dxi;  // module_velprd.f90:52-54
  d.P.gc2 = dt * dyi;
  d.P.gc3 = dt * dzi;
  d.P.dt_ratio = dt_ratio;
  return run_pred_parts<R>(d.P, true, with_cgrid, false, d.s) ? MPDATA_E_CUDA : MPDATA_OK;
}

template <class R>
R cr_split(const Drv<R>& d) {  // velprd_driver.f90:103
  const R a = d.cr[1], b = R(0.5) * d.cr[6];
  return (a > b ? a : b) + std::numeric_limits<R>::min();
}

template <class R>
int compute_courants_impl(R* cr, const R* ox, const R* oy, const R* oz, const R* h, int ntimelevel, R dxi, R dyi,
                          R dzi, R dt, int np, int mp, int lp, int ih, void* stream) {
  if (!cr || !ox || !oy || !oz || !h) return MPDATA_E_NULL;
  if (ntimelevel != 1 && ntimelevel != 2) return MPDATA_E_OPTS;  // STOP 'Wrong ox level' (:653)
  // the boundary flags do not enter compute_courants; periodic ones pass the check for any size
  const mpdata_grid g{np, mp, lp, ih, 1, 1, 1};
  int rc = grid_ok(&g);
  if (rc) return rc;
  Drv<R> d;
  d.s = static_cast<cudaStream_t>(stream);
  d.P = plan_of<R>(g, const_cast<R*>(ox), const_cast<R*>(oy), const_cast<R*>(oz), nullptr, nullptr, nullptr, h,
                   nullptr, nullptr, nullptr);
  if (cudaMallocAsync(&d.keys, 7 * sizeof(unsigned long long), d.s) != cudaSuccess) {
    d.keys = nullptr;
    return MPDATA_E_CUDA;
  }
  if ((rc = courants<R>(d, ntimelevel, dxi, dyi, dzi, dt))) return rc;
  for (int c = 0; c < 7; c++) cr[c] = d.cr[c];
  return MPDATA_OK;
}

template <class R>
int velprd_driver_impl(int* nsubsteps, int* nsubsteps_o, int lsubstepping, R* dtn, R* dtnold, int ltimeadapt,
                       int lvertsplit, int lcrdiag_nphlf, R crmaxlim, R dtmax, R* ox, R* oy, R* oz, R* u, R* v,
                       R* w, R* uadv, R* vadv, R* wadv, const R* h, int ipoles, int ibcx, int ibcy, int ibcz,
                       int np, int mp, int lp, int ih, R dxi, R dyi, R dzi, R dt, double* diag, void* stream) {
  if (!nsubsteps || !nsubsteps_o || !dtn || !dtnold || !ox || !oy || !oz || !uadv || !vadv || !wadv || !h)
    return MPDATA_E_NULL;
  if (ipoles != 0) return MPDATA_E_UNSUPPORTED;
  const mpdata_grid g{np, mp, lp, ih, ibcx, ibcy, ibcz};
  int rc = grid_ok(&g);
  if (rc) return rc;
  if (lsubstepping && ltimeadapt) return MPDATA_E_OPTS;  // :74 STOP
  if (lsubstepping && (*nsubsteps < 1 || *nsubsteps_o < 1)) return MPDATA_E_OPTS;
  Drv<R> d;
  d.s = static_cast<cudaStream_t>(stream);
  d.P = plan_of<R>(g, ox, oy, oz, u, v, w, h, uadv, vadv, wadv);
  if (cudaMallocAsync(&d.keys, 7 * sizeof(unsigned long long), d.s) != cudaSuccess) {
    d.keys = nullptr;
    return MPDATA_E_CUDA;
  }
  const R TINYR = std::numeric_limits<R>::min();
  // 1. (:80-83)
  R dt_ratio = R(1);
  R dtntemp = *dtn;
  if (lsubstepping && *nsubsteps == 1) dt_ratio = (dt / (R(0.0f) * *nsubsteps + R(1))) / (dt / *nsubsteps_o);
  // 2. (:87-101)
  if (lsubstepping) dtntemp = dt;
  if (ltimeadapt) dtntemp = *dtn;
  if (lcrdiag_nphlf) {
    if ((rc = traj0<R>(d, false, dtntemp, dt_ratio, dxi, dyi, dzi))) return rc;
    if ((rc = courants<R>(d, 2, dxi, dyi, dzi, dtntemp))) return rc;
  } else {
    if ((rc = courants<R>(d, 1, dxi, dyi, dzi, dtntemp))) return rc;
  }
  R cr_for_dt = d.cr[0];
  if (lvertsplit) cr_for_dt = cr_split(d);  // 3. (:103)
  if (lsubstepping) {
    // 5. (:108-130)
    bool ok = true;
    if (cr_for_dt > crmaxlim && *nsubsteps == 1) {
      *nsubsteps = (int)std::ceil(cr_for_dt);
      if (cr_for_dt / *nsubsteps > crmaxlim) *nsubsteps += 1;
      ok = false;
    } else if (cr_for_dt / *nsubsteps > R(10) && *nsubsteps > 1) {
      return MPDATA_E_COURANT;  // STOP 'Courant > 1 for nsubsteps >1' (:123)
    }
    *dtn = dt / *nsubsteps;
    // 6. (:135-166)
    if (lvertsplit) {
      dt_ratio = *dtn / *dtnold;
      if ((rc = traj0<R>(d, true, *dtn, dt_ratio, dxi, dyi, dzi))) return rc;
      if ((rc = courants<R>(d, 2, dxi, dyi, dzi, *dtn))) return rc;
      cr_for_dt = d.cr[0];
    }
    for (int round = 0; !ok; round++) {
      if (round >= kMaxRounds || !(cr_for_dt == cr_for_dt)) return MPDATA_E_COURANT;
      dt_ratio = *dtn / *dtnold;
      if ((rc = traj0<R>(d, true, *dtn, dt_ratio, dxi, dyi, dzi))) return rc;
      if ((rc = courants<R>(d, 2, dxi, dyi, dzi, *dtn))) return rc;
      cr_for_dt = d.cr[0];
      if (lvertsplit) cr_for_dt = cr_split(d);
      if (cr_for_dt <= crmaxlim) {
        ok = true;
      } else {
        *nsubsteps += 1;
        *dtn = dt / *nsubsteps;
      }
    }
    *nsubsteps_o = *nsubsteps;  // (:171-173)
    *dtnold = *dtn;
    *dtn = dt / *nsubsteps;
    // 7a / 7b (:175-184)
    if (*nsubsteps > 1 || !lcrdiag_nphlf) {
      if ((rc = traj0<R>(d, true, *dtn, dt_ratio, dxi, dyi, dzi))) return rc;
    } else if (run_pred_parts<R>(d.P, false, true, false, d.s)) {
      return MPDATA_E_CUDA;
    }
  } else if (ltimeadapt) {
    // (:189-228)
    R crmaxlimtemp = crmaxlim;
    *dtnold = *dtn;
    for (int round = 0;; round++) {
      if (round >= kMaxRounds || !(cr_for_dt == cr_for_dt)) return MPDATA_E_COURANT;
      R t = (crmaxlimtemp / (std::fabs(cr_for_dt) + TINYR)) * *dtn;
      t = t < dtmax ? t : dtmax;
      if (t > *dtnold && ((t - *dtnold) / *dtnold) > R(0.1f)) *dtn = t;
      if (t <= *dtnold) *dtn = t;
      dt_ratio = *dtn / *dtnold;
      if ((rc = traj0<R>(d, true, *dtn, dt_ratio, dxi, dyi, dzi))) return rc;
      if ((rc = courants<R>(d, 2, dxi, dyi, dzi, *dtn))) return rc;
      cr_for_dt = d.cr[0];
      if (lvertsplit) cr_for_dt = cr_split(d);
      if (cr_for_dt <= crmaxlim) break;
      crmaxlimtemp = R(0.99f) * crmaxlimtemp;
    }
  } else {
    // 8a / 8b (:236-248)
    if (!lcrdiag_nphlf) {
      if ((rc = traj0<R>(d, true, *dtn, dt_ratio, dxi, dyi, dzi))) return rc;
    } else if (run_pred_parts<R>(d.P, false, true, false, d.s)) {
      return MPDATA_E_CUDA;
    }
  }
  if (lvertsplit) {  // (:250-252)
    const long n = (long)(np + 2 * ih) * (mp + 2 * ih) * (lp + 2 * ih);
    if (run_halve<R>(wadv, n, d.s)) return MPDATA_E_CUDA;
  }
  d.P.dt_ratio = dt_ratio;  // (:254-270)
  if (run_pred_parts<R>(d.P, false, false, true, d.s)) return MPDATA_E_CUDA;
  if (diag) {
    for (int c = 0; c < 7; c++) diag[c] = (double)d.cr[c];
    diag[7] = (double)cr_for_dt;
    diag[8] = (double)dt_ratio;
  }
  return MPDATA_OK;
}

}  // namespace

extern "C" {

int mpdata_compute_courants_f64(double* cr, const double* ox, const double* oy, const double* oz, const double* h,
                                int ntimelevel, double dxi, double dyi, double dzi, double dt, int np, int mp,
                                int lp, int ih, void* stream) {
  return compute_courants_impl<double>(cr, ox, oy, oz, h, ntimelevel, dxi, dyi, dzi, dt, np, mp, lp, ih, stream);
}
int mpdata_compute_courants_f32(float* cr, const float* ox, const float* oy, const float* oz, const float* h,
                                int ntimelevel, float dxi, float dyi, float dzi, float dt, int np, int mp, int lp,
                                int ih, void* stream) {
  return compute_courants_impl<float>(cr, ox, oy, oz, h, ntimelevel, dxi, dyi, dzi, dt, np, mp, lp, ih, stream);
}

int mpdata_velprd_driver_f64(int* nsubsteps, int* nsubsteps_o, int lsubstepping, double* dtn, double* dtnold,
                             int ltimeadapt, int lvertsplit, int lcrdiag_nphlf, double crmaxlim, double dtmax,
                             double* ox, double* oy, double* oz, double* u, double* v, double* w, double* uadv,
                             double* vadv, double* wadv, const double* h, int ipoles, int ibcx, int ibcy, int ibcz,
                             int np, int mp, int lp, int ih, double dxi, double dyi, double dzi, double dt,
                             double* diag, void* stream) {
  return velprd_driver_impl<double>(nsubsteps, nsubsteps_o, lsubstepping, dtn, dtnold, ltimeadapt, lvertsplit,
                                    lcrdiag_nphlf, crmaxlim, dtmax, ox, oy, oz, u, v, w, uadv, vadv, wadv, h,
                                    ipoles, ibcx, ibcy, ibcz, np, mp, lp, ih, dxi, dyi, dzi, dt, diag, stream);
}
int mpdata_velprd_driver_f32(int* nsubsteps, int* nsubsteps_o, int lsubstepping, float* dtn, float* dtnold,
                             int ltimeadapt, int lvertsplit, int lcrdiag_nphlf, float crmaxlim, float dtmax,
                             float* ox, float* oy, float* oz, float* u, float* v, float* w, float* uadv,
                             float* vadv, float* wadv, const float* h, int ipoles, int ibcx, int ibcy, int ibcz,
                             int np, int mp, int lp, int ih, float dxi, float dyi, float dzi, float dt,
                             double* diag, void* stream) {
  return velprd_driver_impl<float>(nsubsteps, nsubsteps_o, lsubstepping, dtn, dtnold, ltimeadapt, lvertsplit,
                                   lcrdiag_nphlf, crmaxlim, dtmax, ox, oy, oz, u, v, w, uadv, vadv, wadv, h,
                                   ipoles, ibcx, ibcy, ibcz, np, mp, lp, ih, dxi, dyi, dzi, dt, diag, stream);
}

}  // extern "C"
