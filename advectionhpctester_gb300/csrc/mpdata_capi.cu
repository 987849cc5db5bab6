// C ABI of the MPDATA step (include/mpdata.h): argument validation, device
// workspace management and dispatch to the stage kernels.  Errors are
// returned as negative codes; nothing here exits (the reference STOPs on bad
// options, advec.f90:174,203,210).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/mpdata.h"
#include "mpdata_common.cuh"
#include "mpdata_fused.cuh"
#include "mpdata_stages.cuh"

using namespace mpdata;

namespace mpdata {
template <class R>
int run_reduce(Geo g, int mode, const R* a, const R* h, const R* rhr, const void* b, int b_is_f64,
               double* part, double* out, cudaStream_t s);
int reduce_blocks();
template <class R>
int run_bound_violations(Geo g, const Arr<R>& psi, const Arr<R>& mx, const Arr<R>& mn, double tol,
                         unsigned long long* count, cudaStream_t s);
}

namespace {

constexpr uint32_t WS_MAGIC = 0x4d504454u;  // "MPDT"
constexpr int NFIELD = 15;  // per problem: xant v1..3 f1..3 w1..3 cp cn mx mn q
constexpr int NVEL = 4;     // per velocity: hinv hmx hmy hmz
constexpr int NGVEL = 12;   // per batch velocity group with several fields: gvf[12] (gauge)
constexpr int NGVS = 9;     // ... and gvs[9] (standard form)
constexpr int NSCRATCH = NFIELD + NVEL;

// Pool-backed event timer: one (start, stop) pair per recorded launch,
// harvested and recycled when the host asks for the totals.
struct EventProf : Prof {
  struct Rec { int stage; cudaEvent_t a, b; };
  std::vector<cudaEvent_t> pool;
  std::vector<Rec> pending;
  cudaEvent_t open_start[NSTAGE] = {};
  double total_ms[NSTAGE] = {};
  long long launches[NSTAGE] = {};
  bool failed = false;
  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) { failed = true; return nullptr; }
    return e;
  }
  void begin(int st, cudaStream_t s) override {
    cudaEvent_t e = get();
    if (e) cudaEventRecord(e, s);
    open_start[st] = e;
  }
  void end(int st, cudaStream_t s) override {
    cudaEvent_t e = get();
    if (e) cudaEventRecord(e, s);
    if (open_start[st] && e) pending.push_back({st, open_start[st], e});
    open_start[st] = nullptr;
  }
  int harvest() {
    for (const Rec& r : pending) {
      if (cudaEventSynchronize(r.b) != cudaSuccess) return MPDATA_E_CUDA;
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) return MPDATA_E_CUDA;
      total_ms[r.stage] += ms;
      launches[r.stage] += 1;
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    pending.clear();
    return failed ? MPDATA_E_CUDA : MPDATA_OK;
  }
  ~EventProf() override {
    for (const Rec& r : pending) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

struct Workspace {
  uint32_t magic;
  mpdata_grid g;
  mpdata_opts o;
  size_t ncell;
  size_t nhi;  // faces n+1 of the density step's upwind fluxes
  size_t elem;
  void* mem;
  int* d_err;
  cudaStream_t last;
  EventProf* prof;
  void* adj;  // adjoint scratch (10 fields), allocated on first use
  // fused single-precision path (periodic gauge grids): its arena shares
  // `mem` with the stage path's scratch, which it never needs at the same time
  bool fused;
  int fz_px, fz_kchunk;
  int fz_mx, fz_mn;    // arena fields holding the last fused step's extrema (-1: none)
  bool fz_extrema;     // the last step ran fused: the extrema live in the arena
  alignas(64) CUtensorMap fz_map;
};

int check_grid(const mpdata_grid* g) {
  if (!g) return MPDATA_E_NULL;
  auto b = [](int v) { return v == 0 || v == 1; };
  if (!b(g->ibcx) || !b(g->ibcy) || !b(g->ibcz)) return MPDATA_E_DIMS;
  if (g->ih < 1 || g->ih > 8) return MPDATA_E_DIMS;
  // open walls reflect about cell 2 / n-1, z walls mirror face 2 / lp
  if (g->np < (g->ibcx ? 1 : 2) || g->mp < (g->ibcy ? 1 : 2) || g->lp < (g->ibcz ? 1 : 2))
    return MPDATA_E_DIMS;
  // launch geometry: grid.y = ceil((mp+1)/4), grid.z = lp+1
  if (g->mp > 4 * 65535 - 8 || g->lp > 65534 || g->np > (1 << 30)) return MPDATA_E_DIMS;
  // 32-bit strides: the largest plane (a C-grid array, halo included) stays below 2^31 elements
  if ((long long)(g->np + 2 * g->ih + 1) * (g->mp + 2 * g->ih + 1) >= (1LL << 31)) return MPDATA_E_DIMS;
  return MPDATA_OK;
}

int check_opts(const mpdata_opts* o) {
  if (!o) return MPDATA_E_NULL;
  if (o->iord < 1 || o->iord > 8) return MPDATA_E_OPTS;
  if (o->nonos != 0 && o->nonos != 1) return MPDATA_E_OPTS;
  if (o->gauge != 0 && o->gauge != 1) return MPDATA_E_OPTS;
  if (o->precision != 32 && o->precision != 64) return MPDATA_E_OPTS;
  if (o->predictor != 0) return MPDATA_E_UNSUPPORTED;
  return MPDATA_OK;
}

Workspace* as_ws(void* p) {
  Workspace* w = static_cast<Workspace*>(p);
  if (!w || w->magic != WS_MAGIC) return nullptr;
  return w;
}

Geo geo_of(const mpdata_grid& g) { return Geo{g.np, g.mp, g.lp, g.ih, g.ibcx, g.ibcy, g.ibcz}; }

// Descriptor of one problem: caller arrays (Fortran layout views) and
// scratch fields carved from `base` (interior-shaped, ncell elements each).
template <class R>
Prob<R> make_prob(const mpdata_grid& g, int gauge, R* psi, const R* u1, const R* u2, const R* u3,
                  const R* h, const R* rhr, const R* bcx, const R* bcy, R* base, size_t ncell,
                  R* vel_base, int own_vel) {
  const int ih = g.ih;
  const int sx = g.np + 2 * ih, sy = g.mp + 2 * ih;
  Prob<R> P;
  memset(&P, 0, sizeof P);
  P.g = geo_of(g);
  P.stdf = gauge ? 0 : 1;
  P.own_vel = own_vel;
  P.psi = caller_view<R>(psi, ih, sx, sy);
  P.u1 = caller_view<R>(const_cast<R*>(u1), ih, sx + 1, sy);
  P.u2 = caller_view<R>(const_cast<R*>(u2), ih, sx, sy + 1);
  P.u3 = caller_view<R>(const_cast<R*>(u3), ih, sx, sy);
  P.h = caller_view<R>(const_cast<R*>(h), ih, sx, sy);
  P.rhr = caller_view<R>(const_cast<R*>(rhr), ih, sx, sy);
  P.bcx = bcx;
  P.bcy = bcy;
  Arr<R>* vel[NVEL] = {&P.hinv, &P.hmx, &P.hmy, &P.hmz};
  for (int s = 0; s < NVEL; s++) *vel[s] = scratch_view<R>(vel_base + (size_t)s * ncell, P.g);
  Arr<R>* slots[NFIELD] = {&P.xant, &P.v1, &P.v2, &P.v3, &P.f1, &P.f2, &P.f3, &P.w1,
                           &P.w2,   &P.w3, &P.cp, &P.cn, &P.mx, &P.mn, &P.q};
  for (int s = 0; s < NFIELD; s++) *slots[s] = scratch_view<R>(base + (size_t)s * ncell, P.g);
  return P;
}

// One step of the workspace's problem P: the fused single-precision kernels
// when the workspace qualifies, else the stage kernels (same bits).
template <class R>
int ws_step(Workspace* w, const Prob<R>& P, Prof* prof, cudaStream_t s) {
  if constexpr (sizeof(R) == 4) {
    if (w->fused) {
      FusedPlan F;
      F.g = P.g;
      F.psi = P.psi;
      F.u1 = P.u1;
      F.u2 = P.u2;
      F.u3 = P.u3;
      F.h = P.h;
      F.rhr = P.rhr;
      F.arena = static_cast<float*>(w->mem);
      F.px = w->fz_px;
      F.fs = (long)w->fz_px * w->g.mp * w->g.lp;
      F.kchunk = w->fz_kchunk;
      F.err = w->d_err;
      F.tmap = &w->fz_map;
      w->fz_extrema = true;
      return run_step_fused(F, w->o.iord, prof, s, &w->fz_mx, &w->fz_mn) == 0 ? MPDATA_OK : MPDATA_E_CUDA;
    }
  }
  w->fz_extrema = false;
  return run_step<R>(P, w->o.iord, w->o.nonos, prof, s) == 0 ? MPDATA_OK : MPDATA_E_CUDA;
}

template <class R>
int step_impl(void* ws, R* psi, const R* u1, const R* u2, const R* u3, const R* h, const R* rhr,
              const R* bcx, const R* bcy, void* stream) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (w->elem != sizeof(R)) return MPDATA_E_WS;
  if (!psi || !u1 || !u2 || !u3 || !h || !rhr) return MPDATA_E_NULL;
  if ((!w->g.ibcx && !bcx) || (!w->g.ibcy && !bcy)) return MPDATA_E_NULL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  w->last = s;
  R* base = static_cast<R*>(w->mem);
  Prob<R> P = make_prob<R>(w->g, w->o.gauge, psi, u1, u2, u3, h, rhr, bcx, bcy, base, w->ncell,
                           base + (size_t)NFIELD * w->ncell, 1);
  return ws_step<R>(w, P, w->prof, s);
}

template <class R>
int velprd_impl(void* ws, R* ox, R* oy, R* oz, R* u, R* v, R* wv, const R* h, R dxi, R dyi, R dzi,
                R dt, R dt_ratio, R* u1, R* u2, R* u3, void* stream) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (w->elem != sizeof(R)) return MPDATA_E_WS;
  if (!ox || !oy || !oz || !h || !u1 || !u2 || !u3) return MPDATA_E_NULL;
  const mpdata_grid& g = w->g;
  const int ih = g.ih;
  const int sx = g.np + 2 * ih, sy = g.mp + 2 * ih, sz = g.lp + 2 * ih;
  const long off = ih + (long)ih * sx + (long)ih * sx * sy;
  PredPlan<R> P;
  P.g = geo_of(g);
  P.lev = (long)sx * sy * sz;
  P.ox = ox + off;
  P.oy = oy + off;
  P.oz = oz + off;
  P.u = u ? u + off : nullptr;
  P.v = v ? v + off : nullptr;
  P.w = wv ? wv + off : nullptr;
  P.h = caller_view<R>(const_cast<R*>(h), ih, sx, sy);
  P.u1 = caller_view<R>(u1, ih, sx + 1, sy);
  P.u2 = caller_view<R>(u2, ih, sx, sy + 1);
  P.u3 = caller_view<R>(u3, ih, sx, sy);
  // gc1=dt*dxi (module_velprd.f90:52-54)
  P.gc1 = dt * dxi;
  P.gc2 = dt * dyi;
  P.gc3 = dt * dzi;
  P.dt_ratio = dt_ratio;
  P.prof = w->prof;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  w->last = s;
  return run_predictor<R>(P, s) == 0 ? MPDATA_OK : MPDATA_E_CUDA;
}

// The predictor's transpose (run_pred_adjoint): the plan's level stacks and
// C-grid arrays are the gradient arrays.
template <class R>
int velprd_adjoint_impl(void* ws, const R* h, R dxi, R dyi, R dzi, R dt, R dt_ratio, const R* gu1, const R* gu2,
                        const R* gu3, R* gox, R* goy, R* goz, void* stream) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (w->elem != sizeof(R)) return MPDATA_E_WS;
  if (!h || !gu1 || !gu2 || !gu3 || !gox || !goy || !goz) return MPDATA_E_NULL;
  const mpdata_grid& g = w->g;
  const int ih = g.ih;
  const int sx = g.np + 2 * ih, sy = g.mp + 2 * ih, sz = g.lp + 2 * ih;
  const long off = ih + (long)ih * sx + (long)ih * sx * sy;
  PredPlan<R> P;
  P.g = geo_of(g);
  P.lev = (long)sx * sy * sz;
  P.ox = gox + off;
  P.oy = goy + off;
  P.oz = goz + off;
  P.u = P.v = P.w = nullptr;
  P.h = caller_view<R>(const_cast<R*>(h), ih, sx, sy);
  P.u1 = caller_view<R>(const_cast<R*>(gu1), ih, sx + 1, sy);
  P.u2 = caller_view<R>(const_cast<R*>(gu2), ih, sx, sy + 1);
  P.u3 = caller_view<R>(const_cast<R*>(gu3), ih, sx, sy);
  P.gc1 = dt * dxi;
  P.gc2 = dt * dyi;
  P.gc3 = dt * dzi;
  P.dt_ratio = dt_ratio;
  P.prof = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  w->last = s;
  return run_pred_adjoint<R>(P, s) == 0 ? MPDATA_OK : MPDATA_E_CUDA;
}

// mpdata3d_rho_gauge_gpubc: predictor, density step, outputs.
template <class R>
int rho_impl(void* ws, R* ox, R* oy, R* oz, R* u, R* v, R* wv, R* u1, R* u2, R* u3, R* x_in, R* x_incomp,
             const R* h, R* rhoadv, R* rhr, const R* pexe, R* pexr1, R* pexr2, const R* bcx, const R* bcy,
             R dxi, R dyi, R dzi, R dt, R dt_ratio, int liner, void* stream) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (w->elem != sizeof(R)) return MPDATA_E_WS;
  if (!w->o.gauge) return MPDATA_E_OPTS;  // the reference's density step is the gauge form
  if (!x_in || !x_incomp || !h || !rhoadv || !rhr || !pexe || !pexr1 || !pexr2) return MPDATA_E_NULL;
  if ((!w->g.ibcx && !bcx) || (!w->g.ibcy && !bcy)) return MPDATA_E_NULL;
  int rc = velprd_impl<R>(ws, ox, oy, oz, u, v, wv, h, dxi, dyi, dzi, dt, dt_ratio, u1, u2, u3, stream);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  R* base = static_cast<R*>(w->mem);
  Prob<R> P = make_prob<R>(w->g, 1, x_in, u1, u2, u3, h, h, bcx, bcy, base, w->ncell,
                           base + (size_t)NFIELD * w->ncell, 1);
  const mpdata_grid& g = w->g;
  const int ih = g.ih, sx = g.np + 2 * ih, sy = g.mp + 2 * ih;
  P.rho = 1;
  P.x_incomp = caller_view<R>(x_incomp, ih, sx, sy);
  P.rhoadv = caller_view<R>(rhoadv, ih, sx, sy);
  P.rhr_out = caller_view<R>(rhr, ih, sx, sy);
  P.pexe = caller_view<R>(const_cast<R*>(pexe), ih, sx, sy);
  P.pexr1 = caller_view<R>(pexr1, ih, sx, sy);
  P.pexr2 = caller_view<R>(pexr2, ih, sx, sy);
  R* hi = base + (size_t)NSCRATCH * w->ncell;
  P.f1hi = hi;
  P.f2hi = hi + (size_t)g.mp * g.lp;
  P.f3hi = hi + (size_t)g.mp * g.lp + (size_t)g.np * g.lp;
  w->fz_extrema = false;
  return run_step<R>(P, liner ? 1 : w->o.iord, w->o.nonos, w->prof, s) == 0 ? MPDATA_OK : MPDATA_E_CUDA;
}

// The reference keeps its scratch in module globals allocated once per grid;
// advec_dwarf therefore caches one workspace per (grid, options).
std::mutex g_cache_mu;
std::vector<Workspace*> g_cache;

bool same(const Workspace* w, const mpdata_grid& g, const mpdata_opts& o) {
  return !memcmp(&w->g, &g, sizeof g) && !memcmp(&w->o, &o, sizeof o);
}

// advec.f90:148-244.  The SELECT on legacyoptmode (and on t_adv for 2 and 4)
// runs first and stops on a bad value; CASE(5) leaves the upwind pointer
// unassociated, so the reference's later call through it has no defined
// result (MPDATA_E_UNSUPPORTED here).  Then lvertsplit=.TRUE. and
// legacyoptmode 2 do nothing (their calls are commented out, :213-220), 6 runs
// the upwind step and copies xant back (:221-231), and 4 runs upwind followed
// by the antidiffusive corrections (:232-241).
template <class R>
int advec_dwarf_impl(int legacyoptmode, int t_adv, int lvertsplit, int np, int mp, int lp, int ih,
                     int ipoles, int ibcx, int ibcy, int ibcz, R* x, const R* x_lr, const R* x_bt,
                     const R* uadv, const R* vadv, const R* wadv, const R* rhr, const R* rhoadv,
                     int iord, int nonos, void* stream) {
  if (legacyoptmode != 2 && legacyoptmode != 4 && legacyoptmode != 5 && legacyoptmode != 6)
    return MPDATA_E_OPTS;
  if ((legacyoptmode == 2 || legacyoptmode == 4) && t_adv != 1 && t_adv != 2) return MPDATA_E_OPTS;
  if (lvertsplit || legacyoptmode == 2) return MPDATA_OK;
  if (legacyoptmode == 5) return MPDATA_E_UNSUPPORTED;
  if (ipoles != 0) return MPDATA_E_UNSUPPORTED;
  mpdata_grid g{np, mp, lp, ih, ibcx, ibcy, ibcz};
  mpdata_opts o{legacyoptmode == 6 ? 1 : iord, legacyoptmode == 6 ? 0 : nonos,
                legacyoptmode == 4 && t_adv == 1 ? 1 : 0, (int)(8 * sizeof(R)), 0};
  if (legacyoptmode == 4 && iord < 2) return MPDATA_E_OPTS;
  int rc = check_grid(&g);
  if (rc) return rc;
  rc = check_opts(&o);
  if (rc) return rc;
  Workspace* w = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    for (Workspace* c : g_cache)
      if (same(c, g, o)) w = c;
    if (!w) {
      void* p = nullptr;
      rc = mpdata_ws_create(&g, &o, &p);
      if (rc) return rc;
      w = static_cast<Workspace*>(p);
      g_cache.push_back(w);
    }
  }
  return step_impl<R>(w, x, uadv, vadv, wadv, rhoadv, rhr, x_lr, x_bt, stream);
}

}  // namespace

namespace mpdata {
int grid_ok(const mpdata_grid* g) { return check_grid(g); }
int opts_ok(const mpdata_opts* o) { return check_opts(o); }
}  // namespace mpdata

namespace {
// psi (caller layout) against the running extrema the workspace's last step kept
template <class R>
int count_violations(Workspace* w, const void* psi, double tol, unsigned long long* d, cudaStream_t s) {
  R* base = static_cast<R*>(w->mem);
  R* x = const_cast<R*>(static_cast<const R*>(psi));
  const Prob<R> P = make_prob<R>(w->g, w->o.gauge, x, x, x, x, x, x, nullptr, nullptr, base, w->ncell,
                                 base + (size_t)NFIELD * w->ncell, 1);
  if (w->fz_extrema && w->fz_mx >= 0) {  // the last step ran fused: its extrema are arena fields
    const long fs = (long)w->fz_px * w->g.mp * w->g.lp;
    const Arr<R> mx{base + (size_t)w->fz_mx * fs, w->fz_px, w->fz_px * w->g.mp};
    const Arr<R> mn{base + (size_t)w->fz_mn * fs, w->fz_px, w->fz_px * w->g.mp};
    return run_bound_violations<R>(P.g, P.psi, mx, mn, tol, d, s) ? MPDATA_E_CUDA : MPDATA_OK;
  }
  return run_bound_violations<R>(P.g, P.psi, P.mx, P.mn, tol, d, s) ? MPDATA_E_CUDA : MPDATA_OK;
}
}  // namespace



extern "C" {

int mpdata_ws_create(const mpdata_grid* grid, const mpdata_opts* opts, void** ws) {
  if (!ws) return MPDATA_E_NULL;
  *ws = nullptr;
  int rc = check_grid(grid);
  if (rc) return rc;
  rc = check_opts(opts);
  if (rc) return rc;
  Workspace* w = new (std::nothrow) Workspace();
  if (!w) return MPDATA_E_CUDA;
  w->magic = WS_MAGIC;
  w->g = *grid;
  w->o = *opts;
  w->ncell = (size_t)grid->np * grid->mp * grid->lp;
  w->elem = opts->precision == 64 ? sizeof(double) : sizeof(float);
  w->last = nullptr;
  w->prof = nullptr;
  w->adj = nullptr;
  w->nhi = (size_t)grid->mp * grid->lp + (size_t)grid->np * grid->lp + (size_t)grid->np * grid->mp;
  w->fused = fused_eligible(geo_of(*grid), opts->precision, opts->gauge, opts->nonos, opts->iord, 0);
  w->fz_mx = w->fz_mn = -1;
  w->fz_extrema = false;
  size_t elems = w->ncell * NSCRATCH + w->nhi;
  if (w->fused) {
    w->fz_kchunk = fused_kchunk(geo_of(*grid));
    const size_t fz = fused_arena_elems(geo_of(*grid), &w->fz_px);
    if (fz > elems) elems = fz;
  }
  if (cudaMalloc(&w->mem, elems * w->elem) != cudaSuccess) {
    cudaGetLastError();
    delete w;
    return MPDATA_E_CUDA;
  }
  if (cudaMalloc(&w->d_err, sizeof(int)) != cudaSuccess || cudaMemset(w->d_err, 0, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(w->mem);
    delete w;
    return MPDATA_E_CUDA;
  }
  if (w->fused && fused_make_tmap(&w->fz_map, static_cast<float*>(w->mem), w->fz_px, geo_of(*grid))) {
    cudaFree(w->mem);
    cudaFree(w->d_err);
    delete w;
    return MPDATA_E_CUDA;
  }
  *ws = w;
  return MPDATA_OK;
}

int mpdata_ws_destroy(void* ws) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    for (size_t i = 0; i < g_cache.size(); i++)
      if (g_cache[i] == w) {
        g_cache.erase(g_cache.begin() + i);
        break;
      }
  }
  w->magic = 0;
  delete w->prof;
  if (w->adj) cudaFree(w->adj);
  cudaError_t e1 = cudaFree(w->mem);
  cudaError_t e2 = cudaFree(w->d_err);
  delete w;
  return (e1 == cudaSuccess && e2 == cudaSuccess) ? MPDATA_OK : MPDATA_E_CUDA;
}

int mpdata_step_f64(void* ws, double* psi, const double* u1, const double* u2, const double* u3,
                    const double* h, const double* rhr, const double* bcx, const double* bcy,
                    void* stream) {
  return step_impl<double>(ws, psi, u1, u2, u3, h, rhr, bcx, bcy, stream);
}
int mpdata_step_f32(void* ws, float* psi, const float* u1, const float* u2, const float* u3,
                    const float* h, const float* rhr, const float* bcx, const float* bcy,
                    void* stream) {
  return step_impl<float>(ws, psi, u1, u2, u3, h, rhr, bcx, bcy, stream);
}

int mpdata_advec_dwarf_f64(int legacyoptmode, int t_adv, int lupdatemulti, int lvertsplit, int np,
                           int mp, int lp, int ih, int ipoles, int ibcx, int ibcy, int ibcz,
                           double* x, const double* x_lr, const double* x_bt, const double* uadv,
                           const double* vadv, const double* wadv, const double* rhr,
                           const double* rhoadv, int iord, int nonos, void* stream) {
  (void)lupdatemulti;
  return advec_dwarf_impl<double>(legacyoptmode, t_adv, lvertsplit, np, mp, lp, ih, ipoles, ibcx, ibcy, ibcz, x,
                                  x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv, iord, nonos, stream);
}
int mpdata_advec_dwarf_f32(int legacyoptmode, int t_adv, int lupdatemulti, int lvertsplit, int np,
                           int mp, int lp, int ih, int ipoles, int ibcx, int ibcy, int ibcz,
                           float* x, const float* x_lr, const float* x_bt, const float* uadv,
                           const float* vadv, const float* wadv, const float* rhr,
                           const float* rhoadv, int iord, int nonos, void* stream) {
  (void)lupdatemulti;
  return advec_dwarf_impl<float>(legacyoptmode, t_adv, lvertsplit, np, mp, lp, ih, ipoles, ibcx, ibcy, ibcz, x,
                                 x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv, iord, nonos, stream);
}

int mpdata_release_cached(void) {
  std::vector<Workspace*> all;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    all.swap(g_cache);
  }
  int rc = MPDATA_OK;
  for (Workspace* w : all)
    if (mpdata_ws_destroy(w) != MPDATA_OK) rc = MPDATA_E_CUDA;
  return rc;
}

int mpdata_velprd_f64(void* ws, double* ox, double* oy, double* oz, double* u, double* v,
                      double* w, const double* h, double dxi, double dyi, double dzi, double dt,
                      double dt_ratio, double* u1, double* u2, double* u3, void* stream) {
  return velprd_impl<double>(ws, ox, oy, oz, u, v, w, h, dxi, dyi, dzi, dt, dt_ratio, u1, u2, u3, stream);
}
int mpdata_velprd_f32(void* ws, float* ox, float* oy, float* oz, float* u, float* v, float* w,
                      const float* h, float dxi, float dyi, float dzi, float dt, float dt_ratio,
                      float* u1, float* u2, float* u3, void* stream) {
  return velprd_impl<float>(ws, ox, oy, oz, u, v, w, h, dxi, dyi, dzi, dt, dt_ratio, u1, u2, u3, stream);
}

int mpdata_velprd_adjoint_f64(void* ws, const double* h, double dxi, double dyi, double dzi, double dt,
                              double dt_ratio, const double* g_u1, const double* g_u2, const double* g_u3,
                              double* g_ox, double* g_oy, double* g_oz, void* stream) {
  return velprd_adjoint_impl<double>(ws, h, dxi, dyi, dzi, dt, dt_ratio, g_u1, g_u2, g_u3, g_ox, g_oy, g_oz, stream);
}
int mpdata_velprd_adjoint_f32(void* ws, const float* h, float dxi, float dyi, float dzi, float dt, float dt_ratio,
                              const float* g_u1, const float* g_u2, const float* g_u3, float* g_ox, float* g_oy,
                              float* g_oz, void* stream) {
  return velprd_adjoint_impl<float>(ws, h, dxi, dyi, dzi, dt, dt_ratio, g_u1, g_u2, g_u3, g_ox, g_oy, g_oz, stream);
}

int mpdata_rho_gauge_f64(void* ws, double* ox, double* oy, double* oz, double* u, double* v, double* w,
                         double* u1, double* u2, double* u3, double* x_in, double* x_incomp,
                         const double* h, double* rhoadv, double* rhr, const double* pexe, double* pexr1,
                         double* pexr2, const double* bcx, const double* bcy, double dxi, double dyi,
                         double dzi, double dt, double dt_ratio, int liner, void* stream) {
  return rho_impl<double>(ws, ox, oy, oz, u, v, w, u1, u2, u3, x_in, x_incomp, h, rhoadv, rhr, pexe, pexr1,
                          pexr2, bcx, bcy, dxi, dyi, dzi, dt, dt_ratio, liner, stream);
}
int mpdata_rho_gauge_f32(void* ws, float* ox, float* oy, float* oz, float* u, float* v, float* w,
                         float* u1, float* u2, float* u3, float* x_in, float* x_incomp, const float* h,
                         float* rhoadv, float* rhr, const float* pexe, float* pexr1, float* pexr2,
                         const float* bcx, const float* bcy, float dxi, float dyi, float dzi, float dt,
                         float dt_ratio, int liner, void* stream) {
  return rho_impl<float>(ws, ox, oy, oz, u, v, w, u1, u2, u3, x_in, x_incomp, h, rhoadv, rhr, pexe, pexr1,
                         pexr2, bcx, bcy, dxi, dyi, dzi, dt, dt_ratio, liner, stream);
}

int mpdata_ws_error(void* ws, int* error_word) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (!error_word) return MPDATA_E_NULL;
  if (cudaStreamSynchronize(w->last) != cudaSuccess) return MPDATA_E_CUDA;
  if (cudaMemcpy(error_word, w->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return MPDATA_E_CUDA;
  return MPDATA_OK;
}

long long mpdata_launch_count(void) { return (long long)launch_count(); }

int mpdata_ws_bound_violations(void* ws, const void* psi, double tol, long long* count, void* stream) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (!psi || !count) return MPDATA_E_NULL;
  if (!w->o.nonos || w->o.iord < 3) return MPDATA_E_UNSUPPORTED;  // the extrema are kept from iord 3 on
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long* d = nullptr;
  if (cudaMallocAsync(&d, sizeof *d, s) != cudaSuccess) return MPDATA_E_CUDA;
  int rc = cudaMemsetAsync(d, 0, sizeof *d, s) == cudaSuccess ? MPDATA_OK : MPDATA_E_CUDA;
  if (!rc) rc = w->elem == sizeof(double) ? count_violations<double>(w, psi, tol, d, s)
                                          : count_violations<float>(w, psi, tol, d, s);
  unsigned long long h = 0;
  if (!rc && cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = MPDATA_E_CUDA;
  cudaFreeAsync(d, s);
  if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = MPDATA_E_CUDA;
  if (!rc) *count = (long long)h;
  return rc;
}

int mpdata_ws_profile(void* ws, int enable) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (enable && !w->prof) {
    w->prof = new (std::nothrow) EventProf();
    if (!w->prof) return MPDATA_E_CUDA;
  } else if (!enable && w->prof) {
    cudaStreamSynchronize(w->last);
    delete w->prof;
    w->prof = nullptr;
  }
  return MPDATA_OK;
}

int mpdata_ws_stage_times(void* ws, int nstages, double* total_ms, long long* launches) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (!total_ms || !launches) return MPDATA_E_NULL;
  if (nstages < 0) return MPDATA_E_OPTS;
  const int n = nstages < NSTAGE ? nstages : NSTAGE;
  for (int i = 0; i < n; i++) { total_ms[i] = 0.0; launches[i] = 0; }
  if (!w->prof) return NSTAGE;
  int rc = w->prof->harvest();
  if (rc) return rc;
  for (int i = 0; i < n; i++) {
    total_ms[i] = w->prof->total_ms[i];
    launches[i] = w->prof->launches[i];
  }
  return NSTAGE;
}

const char* mpdata_stage_name(int stage) {
  static const char* names[NSTAGE] = {"upwind", "pseudo_velocity", "limiter_bounds", "limited_flux",
                                      "corrective_update", "copy", "predictor_level",
                                      "predictor_cgrid", "density_outputs", "pair_sums",
                                      "fused_upwind_pseudo", "fused_pseudo", "fused_limit_update"};
  return (stage >= 0 && stage < NSTAGE) ? names[stage] : "";
}

const char* mpdata_strerror(int code) {
  switch (code) {
    case MPDATA_OK: return "ok";
    case MPDATA_E_DIMS: return "bad grid dimensions or boundary flags";
    case MPDATA_E_OPTS: return "bad options (legacyoptmode/t_adv/iord/nonos/precision)";
    case MPDATA_E_NULL: return "a required pointer is NULL";
    case MPDATA_E_WS: return "workspace missing or built for another grid/precision";
    case MPDATA_E_CUDA: return "CUDA runtime error";
    case MPDATA_E_DEVICE: return "device error word set (non-finite value)";
    case MPDATA_E_UNSUPPORTED: return "reference option outside this library's scope";
    case MPDATA_E_TOO_LARGE:
      return "problem exceeds a fixed size limit (the 32768-cell scratch of mpdata_step_noalloc_f64, "
             "2^31 batch tiles, or a 4 GiB netCDF classic slab)";
    case MPDATA_E_COURANT: return "Courant control failed: above the fatal limit while substepping, or not finite";
    case MPDATA_E_IO: return "field file missing, unreadable, not netCDF classic, or without the variable";
    default: return "unknown error";
  }
}

const char* mpdata_version(void) { return "mpdata-gb300 0.1 (sm_103a)"; }

}  // extern "C"

// ===========================================================================
// Batches: many problems advanced together (include/mpdata.h, mpdata_batch_*)
// ===========================================================================
namespace {

constexpr uint32_t BATCH_MAGIC = 0x4d504242u;  // "MPBB"

struct Batch {
  uint32_t magic;
  int nprob, ih, iord, nonos, precision;
  size_t elem;
  std::vector<mpdata_problem> pr;
  std::vector<int> owner;       // first problem of each problem's velocity group
  std::vector<size_t> foff;     // element offset of each problem's field scratch
  std::vector<size_t> voff;     // element offset of each problem's velocity scratch
  std::vector<int> gv;          // problem's velocity group precomputes its first-pass terms:
                                // bit 0 the gauge form's, bit 1 the standard form's
  std::vector<size_t> ncell;
  std::vector<int> given;       // arrays set for the problem
  std::vector<unsigned char> table;  // host image of the Prob table
  size_t pbytes;                // sizeof(Prob<R>)
  void* mem;
  void* d_table;
  unsigned char* h_stage;       // pinned staging buffer of the table upload
  cudaEvent_t upload_done;
  unsigned long long* d_tiles;   // packed tile list of the current block shape
  size_t tiles_cap;             // capacity of d_tiles (entries)
  int ntiles;
  int bx, by;
  bool dirty;
  bool use_graph;
  cudaGraphExec_t gexec;
  cudaStream_t cap;             // private stream used only for graph capture
  EventProf* prof;
  cudaStream_t last;
  // problems on the fused single-precision kernels (FP32 periodic gauge
  // problems, as single steps take them): one launch per fused kernel for
  // all of them; the others run on the tile kernels above
  std::vector<int> fzi;            // index in the fused table, or -1
  int nfz;
  std::vector<FusedArgs> fz_args;  // host image of the fused table
  void* d_fz;
  void* d_maps;                    // one tensor map per fused problem
  unsigned long long* d_items_up;  // work items of the upwind+pseudo kernel
  unsigned long long* d_items;     // ... of the other fused kernels
  int n_items_up, n_items;
  int* d_err;
};

Batch* as_batch(void* p) {
  Batch* b = static_cast<Batch*>(p);
  if (!b || b->magic != BATCH_MAGIC) return nullptr;
  return b;
}

mpdata_grid grid_of(const Batch* b, int p) {
  const mpdata_problem& q = b->pr[p];
  return mpdata_grid{q.np, q.mp, q.lp, b->ih, q.ibcx, q.ibcy, q.ibcz};
}

// Tile list for a block shape: one 64-bit word per tile of bx*by cells in
// one plane, packing the problem (bits 0-15), the tile's x and y indices
// (16-31, 32-47) and its plane k-1 (48-63).  Problems follow one another,
// and within a problem x varies fastest, then y, then k.
int set_shape(Batch* b, int bx, int by, cudaStream_t s) {
  long long total = 0;
  for (int p = 0; p < b->nprob; p++) {
    if (b->fzi[p] >= 0) continue;  // on the fused kernels
    const mpdata_problem& q = b->pr[p];
    const long long ntx = (q.np + bx - 1) / bx, nty = (q.mp + by - 1) / by;
    if (ntx > 65536 || nty > 65536) return MPDATA_E_DIMS;
    total += ntx * nty * q.lp;
  }
  if (total > 0x7fffffffLL) return MPDATA_E_TOO_LARGE;
  std::vector<unsigned long long> list;
  list.reserve((size_t)total);
  for (int p = 0; p < b->nprob; p++) {
    if (b->fzi[p] >= 0) continue;
    const mpdata_problem& q = b->pr[p];
    const int ntx = (q.np + bx - 1) / bx, nty = (q.mp + by - 1) / by;
    for (int k = 0; k < q.lp; k++)
      for (int ty = 0; ty < nty; ty++)
        for (int tx = 0; tx < ntx; tx++)
          list.push_back((unsigned long long)p | ((unsigned long long)tx << 16) |
                         ((unsigned long long)ty << 32) | ((unsigned long long)k << 48));
  }
  if (!list.empty() && list.size() > b->tiles_cap) {
    if (b->d_tiles && cudaFree(b->d_tiles) != cudaSuccess) return MPDATA_E_CUDA;
    b->d_tiles = nullptr;
    b->tiles_cap = 0;
    if (cudaMalloc(&b->d_tiles, list.size() * sizeof(unsigned long long)) != cudaSuccess) return MPDATA_E_CUDA;
    b->tiles_cap = list.size();
  }
  if (!list.empty() && cudaMemcpyAsync(b->d_tiles, list.data(), list.size() * sizeof(unsigned long long),
                                       cudaMemcpyHostToDevice, s) != cudaSuccess)
    return MPDATA_E_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MPDATA_E_CUDA;  // list is a local buffer
  b->bx = bx;
  b->by = by;
  b->ntiles = (int)total;
  if (b->gexec) {
    cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
  }
  return MPDATA_OK;
}

int upload_table(Batch* b, cudaStream_t s) {
  if (!b->dirty) return MPDATA_OK;
  for (int p = 0; p < b->nprob; p++)
    if (!b->given[p]) return MPDATA_E_NULL;
  // the previous upload must have finished reading the staging buffer
  if (cudaEventSynchronize(b->upload_done) != cudaSuccess) return MPDATA_E_CUDA;
  memcpy(b->h_stage, b->table.data(), b->table.size());
  if (cudaMemcpyAsync(b->d_table, b->h_stage, b->table.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return MPDATA_E_CUDA;
  if (b->nfz) {
    const size_t fb = b->fz_args.size() * sizeof(FusedArgs);
    memcpy(b->h_stage + b->table.size(), b->fz_args.data(), fb);
    if (cudaMemcpyAsync(b->d_fz, b->h_stage + b->table.size(), fb, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return MPDATA_E_CUDA;
  }
  if (cudaEventRecord(b->upload_done, s) != cudaSuccess) return MPDATA_E_CUDA;
  b->dirty = false;
  return MPDATA_OK;
}

template <class R>
BatchLaunch<R> launch_of(const Batch* b, int halo) {
  BatchLaunch<R> L;
  L.probs = static_cast<const Prob<R>*>(b->d_table);
  L.tiles = b->d_tiles;
  L.ntiles = b->ntiles;
  L.bx = b->bx;
  L.by = b->by;
  L.iord = b->iord;
  L.nonos = b->nonos;
  L.halo = halo;
  L.pairs = 0;
  if (sizeof(R) == 8)
    for (const mpdata_problem& q : b->pr) L.pairs |= q.gauge ? 1 : 0;
  return L;
}

// halo = 0 (the autotuner's steps write scratch only): the fused kernels,
// whose last pass writes psi, do not run
int batch_run(Batch* b, int halo, Prof* prof, cudaStream_t s) {
  if (b->ntiles > 0) {
    const int rc = b->precision == 64 ? run_batch<double>(launch_of<double>(b, halo), prof, s)
                                      : run_batch<float>(launch_of<float>(b, halo), prof, s);
    if (rc) return MPDATA_E_CUDA;
  }
  if (halo && b->nfz &&
      run_batch_fused(static_cast<const FusedArgs*>(b->d_fz), static_cast<const CUtensorMap*>(b->d_maps),
                      b->d_items_up, b->n_items_up, b->d_items, b->n_items, b->iord, prof, s))
    return MPDATA_E_CUDA;
  return MPDATA_OK;
}

template <class R>
void write_prob(Batch* b, int p, void* psi, const void* u1, const void* u2, const void* u3, const void* h,
                const void* rhr, const void* bcx, const void* bcy) {
  R* base = static_cast<R*>(b->mem);
  const mpdata_grid g = grid_of(b, p);
  Prob<R> P = make_prob<R>(g, b->pr[p].gauge, (R*)psi, (const R*)u1, (const R*)u2, (const R*)u3,
                           (const R*)h, (const R*)rhr, (const R*)bcx, (const R*)bcy, base + b->foff[p],
                           b->ncell[p], base + b->voff[p], b->owner[p] == p ? 1 : 0);
  P.pairs = (b->pr[p].gauge && sizeof(R) == 8) ? 1 : 0;  // kb_pairs fills cp/cn/q before kb_pseudo
  P.gv = b->gv[p];
  R* gbase = base + b->voff[p] + (size_t)NVEL * b->ncell[p];
  if (P.gv & 1) {
    for (int s = 0; s < NGVEL; s++) P.gvf[s] = scratch_view<R>(gbase + (size_t)s * b->ncell[p], P.g);
    gbase += (size_t)NGVEL * b->ncell[p];
  }
  if (P.gv & 2)
    for (int s = 0; s < NGVS; s++) P.gvs[s] = scratch_view<R>(gbase + (size_t)s * b->ncell[p], P.g);
  memcpy(b->table.data() + (size_t)p * sizeof(Prob<R>), &P, sizeof P);
  if constexpr (sizeof(R) == 4) {
    const int f = b->fzi[p];
    if (f >= 0) {
      FusedPlan F;
      F.g = P.g;
      F.psi = P.psi;
      F.u1 = P.u1;
      F.u2 = P.u2;
      F.u3 = P.u3;
      F.h = P.h;
      F.rhr = P.rhr;
      F.arena = base + b->foff[p];
      fused_arena_elems(P.g, &F.px);
      F.fs = (long)F.px * P.g.mp * P.g.lp;
      F.kchunk = fused_kchunk(P.g);
      F.err = b->d_err;
      F.tmap = nullptr;
      b->fz_args[f] = fused_args(F);
    }
  }
}

// tuned block shapes per (precision, iord, nonos, cells), shared by batches
std::mutex g_tune_mu;
struct TuneKey { int prec, iord, nonos; long long cells; int nprob; };
std::vector<std::pair<TuneKey, std::pair<int, int>>> g_tuned;

TuneKey key_of(const Batch* b) {
  long long cells = 0;
  for (size_t p = 0; p < b->ncell.size(); p++) cells += (long long)b->ncell[p];
  return TuneKey{b->precision, b->iord, b->nonos, cells, b->nprob};
}

}  // namespace

extern "C" {

int mpdata_batch_create(int nprob, const mpdata_problem* probs, int ih, int iord, int nonos, int precision,
                        void** batch) {
  if (!batch) return MPDATA_E_NULL;
  *batch = nullptr;
  if (!probs) return MPDATA_E_NULL;
  if (nprob < 1 || nprob > 65536) return MPDATA_E_DIMS;
  mpdata_opts o{iord, nonos, 1, precision, 0};
  int rc = check_opts(&o);
  if (rc) return rc;
  Batch* b = new (std::nothrow) Batch();
  if (!b) return MPDATA_E_CUDA;
  b->nprob = nprob;
  b->ih = ih;
  b->iord = iord;
  b->nonos = nonos;
  b->precision = precision;
  b->elem = precision == 64 ? sizeof(double) : sizeof(float);
  b->pbytes = precision == 64 ? sizeof(Prob<double>) : sizeof(Prob<float>);
  b->pr.assign(probs, probs + nprob);
  b->owner.resize(nprob);
  b->foff.resize(nprob);
  b->voff.resize(nprob);
  b->ncell.resize(nprob);
  b->given.assign(nprob, 0);
  b->fzi.assign(nprob, -1);
  b->nfz = 0;
  b->d_fz = b->d_maps = nullptr;
  b->d_items_up = b->d_items = nullptr;
  b->n_items_up = b->n_items = 0;
  b->d_err = nullptr;
  size_t off = 0;
  for (int p = 0; p < nprob; p++) {
    const mpdata_problem& q = probs[p];
    if (q.gauge != 0 && q.gauge != 1) { delete b; return MPDATA_E_OPTS; }
    mpdata_grid g{q.np, q.mp, q.lp, ih, q.ibcx, q.ibcy, q.ibcz};
    rc = check_grid(&g);
    if (rc) { delete b; return rc; }
    b->ncell[p] = (size_t)q.np * q.mp * q.lp;
    if (fused_eligible(geo_of(g), precision, q.gauge, nonos, iord, 0)) b->fzi[p] = b->nfz++;
    // a velocity group is shared within the fused problems or within the others
    int own = p;
    for (int r = 0; r < p; r++)
      if (probs[r].velocity_group == q.velocity_group && b->owner[r] == r &&
          (b->fzi[r] >= 0) == (b->fzi[p] >= 0)) { own = r; break; }
    if (own != p) {  // sharing a velocity needs the same grid and boundaries
      const mpdata_problem& o2 = probs[own];
      if (o2.np != q.np || o2.mp != q.mp || o2.lp != q.lp || o2.ibcx != q.ibcx || o2.ibcy != q.ibcy ||
          o2.ibcz != q.ibcz) { delete b; return MPDATA_E_DIMS; }
    }
    b->owner[p] = own;
    b->foff[p] = off;
    size_t nf = (size_t)NFIELD * b->ncell[p];
    if (b->fzi[p] >= 0) nf = std::max(nf, fused_arena_elems(geo_of(g), nullptr));
    off += (nf + 63) / 64 * 64;  // 256-byte aligned regions (TMA wants 16)
  }
  // a group of two or more fields shares the velocity-only terms of its
  // first-pass pseudo-velocities, for each form among its fields (velgroup_body)
  b->gv.assign(nprob, 0);
  {
    std::vector<int> members(nprob, 0), forms(nprob, 0);
    for (int p = 0; p < nprob; p++) {
      members[b->owner[p]]++;
      forms[b->owner[p]] |= probs[p].gauge ? 1 : 2;
    }
    for (int p = 0; p < nprob; p++) {
      const int o = b->owner[p];
      b->gv[p] = (iord >= 2 && members[o] >= 2) ? forms[o] : 0;
    }
  }
  for (int p = 0; p < nprob; p++)
    if (b->owner[p] == p) {
      b->voff[p] = off;
      off += (size_t)(NVEL + ((b->gv[p] & 1) ? NGVEL : 0) + ((b->gv[p] & 2) ? NGVS : 0)) * b->ncell[p];
    }
  for (int p = 0; p < nprob; p++) b->voff[p] = b->voff[b->owner[p]];
  b->table.assign((size_t)nprob * b->pbytes, 0);
  b->fz_args.assign(b->nfz, FusedArgs{});
  b->mem = b->d_table = nullptr;
  b->h_stage = nullptr;
  b->d_tiles = nullptr;
  b->tiles_cap = 0;
  b->ntiles = 0;
  b->upload_done = nullptr;
  b->gexec = nullptr;
  b->cap = nullptr;
  b->prof = nullptr;
  b->last = nullptr;
  b->use_graph = false;
  b->dirty = true;
  bool ok = cudaMalloc(&b->mem, off * b->elem) == cudaSuccess &&
            cudaMalloc(&b->d_table, b->table.size()) == cudaSuccess &&
            cudaMallocHost(&b->h_stage, b->table.size() + b->nfz * sizeof(FusedArgs)) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->upload_done, cudaEventDisableTiming) == cudaSuccess &&
            cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) == cudaSuccess;
  b->magic = BATCH_MAGIC;
  if (ok && b->nfz) {
    // fused problems: argument table, tensor maps of their arenas, work items
    std::vector<CUtensorMap> maps(b->nfz);
    std::vector<unsigned long long> up, rest;
    for (int p = 0; p < nprob && ok; p++) {
      const int f = b->fzi[p];
      if (f < 0) continue;
      const Geo g = geo_of(grid_of(b, p));
      int px = 0;
      fused_arena_elems(g, &px);
      ok = fused_make_tmap(&maps[f], static_cast<float*>(b->mem) + b->foff[p], px, g) == 0;
      fused_items(g, fused_kchunk(g), f, up, rest);
    }
    ok = ok && up.size() < 0x7fffffffu && rest.size() < 0x7fffffffu && fused_init() == 0 &&
         cudaMalloc(&b->d_fz, b->nfz * sizeof(FusedArgs)) == cudaSuccess &&
         cudaMalloc(&b->d_maps, b->nfz * sizeof(CUtensorMap)) == cudaSuccess &&
         cudaMalloc(&b->d_items_up, up.size() * sizeof(unsigned long long)) == cudaSuccess &&
         cudaMalloc(&b->d_items, rest.size() * sizeof(unsigned long long)) == cudaSuccess &&
         cudaMalloc(&b->d_err, sizeof(int)) == cudaSuccess && cudaMemset(b->d_err, 0, sizeof(int)) == cudaSuccess &&
         cudaMemcpy(b->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice) ==
             cudaSuccess &&
         cudaMemcpy(b->d_items_up, up.data(), up.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice) ==
             cudaSuccess &&
         cudaMemcpy(b->d_items, rest.data(), rest.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice) ==
             cudaSuccess;
    b->n_items_up = (int)up.size();
    b->n_items = (int)rest.size();
  }
  if (ok) {
    // default shape, or the tuned one for this batch signature
    int bx = 32, by = 4;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      const TuneKey k = key_of(b);
      for (auto& e : g_tuned)
        if (!memcmp(&e.first, &k, sizeof k)) { bx = e.second.first; by = e.second.second; }
    }
    rc = set_shape(b, bx, by, b->cap);
    ok = rc == MPDATA_OK;
  }
  if (!ok) {
    cudaGetLastError();
    mpdata_batch_destroy(b);
    return rc != MPDATA_OK ? rc : MPDATA_E_CUDA;
  }
  *batch = b;
  return MPDATA_OK;
}

int mpdata_batch_destroy(void* batch) {
  Batch* b = as_batch(batch);
  if (!b) return MPDATA_E_WS;
  b->magic = 0;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  delete b->prof;
  if (b->upload_done) { cudaEventSynchronize(b->upload_done); cudaEventDestroy(b->upload_done); }
  if (b->cap) cudaStreamDestroy(b->cap);
  cudaFreeHost(b->h_stage);
  cudaFree(b->d_tiles);
  cudaFree(b->d_table);
  cudaFree(b->d_fz);
  cudaFree(b->d_maps);
  cudaFree(b->d_items_up);
  cudaFree(b->d_items);
  cudaFree(b->d_err);
  cudaError_t e = cudaFree(b->mem);
  delete b;
  return e == cudaSuccess ? MPDATA_OK : MPDATA_E_CUDA;
}

int mpdata_batch_set(void* batch, int prob, void* psi, const void* u1, const void* u2, const void* u3,
                     const void* h, const void* rhr, const void* bcx, const void* bcy) {
  Batch* b = as_batch(batch);
  if (!b) return MPDATA_E_WS;
  if (prob < 0 || prob >= b->nprob) return MPDATA_E_DIMS;
  if (!psi || !u1 || !u2 || !u3 || !h || !rhr) return MPDATA_E_NULL;
  if ((!b->pr[prob].ibcx && !bcx) || (!b->pr[prob].ibcy && !bcy)) return MPDATA_E_NULL;
  if (b->precision == 64) write_prob<double>(b, prob, psi, u1, u2, u3, h, rhr, bcx, bcy);
  else write_prob<float>(b, prob, psi, u1, u2, u3, h, rhr, bcx, bcy);
  b->given[prob] = 1;
  b->dirty = true;
  return MPDATA_OK;
}

int mpdata_batch_step(void* batch, void* stream) {
  Batch* b = as_batch(batch);
  if (!b) return MPDATA_E_WS;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  b->last = s;
  int rc = upload_table(b, s);
  if (rc) return rc;
  if (!b->use_graph) return batch_run(b, 1, b->prof, s);
  if (!b->gexec) {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return MPDATA_E_CUDA;
    rc = batch_run(b, 1, nullptr, b->cap);
    if (cudaStreamEndCapture(b->cap, &graph) != cudaSuccess || rc) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return MPDATA_E_CUDA;
    }
    cudaError_t e = cudaGraphInstantiate(&b->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { b->gexec = nullptr; return MPDATA_E_CUDA; }
  }
  return cudaGraphLaunch(b->gexec, s) == cudaSuccess ? MPDATA_OK : MPDATA_E_CUDA;
}

int mpdata_batch_graph(void* batch, int enable) {
  Batch* b = as_batch(batch);
  if (!b) return MPDATA_E_WS;
  b->use_graph = enable != 0;
  if (!b->use_graph && b->gexec) {
    cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
  }
  return MPDATA_OK;
}

int mpdata_batch_tune(void* batch, void* stream, int* bx_out, int* by_out) {
  Batch* b = as_batch(batch);
  if (!b) return MPDATA_E_WS;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = upload_table(b, s);
  if (rc) return rc;
  if (b->ntiles == 0) {  // every problem runs on the fused kernels: no tile shape to choose
    if (bx_out) *bx_out = b->bx;
    if (by_out) *by_out = b->by;
    return MPDATA_OK;
  }
  static const int shapes[][2] = {{32, 4}, {32, 8}, {64, 2}, {64, 4}, {128, 1}, {128, 2}, {16, 8}};
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return MPDATA_E_CUDA;
  float best = 1e30f;
  int bbx = b->bx, bby = b->by;
  for (const auto& sh : shapes) {
    const int r0 = set_shape(b, sh[0], sh[1], s);
    if (r0 == MPDATA_E_DIMS || r0 == MPDATA_E_TOO_LARGE) continue;  // shape unusable for these grids
    if (r0) { rc = r0; break; }
    // halo=0: the tuning steps write scratch only, never the caller's psi
    if ((rc = batch_run(b, 0, nullptr, s))) break;
    cudaEventRecord(e0, s);
    for (int r = 0; r < 2 && !rc; r++) rc = batch_run(b, 0, nullptr, s);
    cudaEventRecord(e1, s);
    if (rc || cudaEventSynchronize(e1) != cudaSuccess) { rc = MPDATA_E_CUDA; break; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) { best = ms; bbx = sh[0]; bby = sh[1]; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const int r1 = set_shape(b, bbx, bby, s);
  if (rc) return rc;
  if (r1) return r1;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const TuneKey k = key_of(b);
    bool found = false;
    for (auto& e : g_tuned)
      if (!memcmp(&e.first, &k, sizeof k)) { e.second = {bbx, bby}; found = true; }
    if (!found) g_tuned.push_back({k, {bbx, bby}});
  }
  if (bx_out) *bx_out = bbx;
  if (by_out) *by_out = bby;
  return MPDATA_OK;
}

int mpdata_batch_set_shape(void* batch, int bx, int by, void* stream) {
  Batch* b = as_batch(batch);
  if (!b) return MPDATA_E_WS;
  if (bx < 1 || by < 1 || bx > 256 || by > 256) return MPDATA_E_OPTS;
  const int nt = bx * by;
  if (nt < 32 || nt > 256 || nt % 32) return MPDATA_E_OPTS;
  return set_shape(b, bx, by, static_cast<cudaStream_t>(stream));
}

int mpdata_batch_profile(void* batch, int enable) {
  Batch* b = as_batch(batch);
  if (!b) return MPDATA_E_WS;
  if (enable && !b->prof) {
    b->prof = new (std::nothrow) EventProf();
    if (!b->prof) return MPDATA_E_CUDA;
  } else if (!enable && b->prof) {
    cudaStreamSynchronize(b->last);
    delete b->prof;
    b->prof = nullptr;
  }
  return MPDATA_OK;
}

int mpdata_batch_stage_times(void* batch, int nstages, double* total_ms, long long* launches) {
  Batch* b = as_batch(batch);
  if (!b) return MPDATA_E_WS;
  if (!total_ms || !launches) return MPDATA_E_NULL;
  if (nstages < 0) return MPDATA_E_OPTS;
  const int n = nstages < NSTAGE ? nstages : NSTAGE;
  for (int i = 0; i < n; i++) { total_ms[i] = 0.0; launches[i] = 0; }
  if (!b->prof) return NSTAGE;
  int rc = b->prof->harvest();
  if (rc) return rc;
  for (int i = 0; i < n; i++) { total_ms[i] = b->prof->total_ms[i]; launches[i] = b->prof->launches[i]; }
  return NSTAGE;
}

}  // extern "C"

// ===========================================================================
// FP64 compensated reductions (mass, error norms)
// ===========================================================================
namespace {

template <class R>
int reduce_impl(const mpdata_grid* grid, int mode, const R* a, const R* h, const R* rhr, const void* b,
                int b_is_f64, double* host_out, void* stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t nb = (size_t)reduce_blocks() * 6 + 4;
  double* buf = nullptr;
  if (cudaMallocAsync(&buf, nb * sizeof(double), s) != cudaSuccess) return MPDATA_E_CUDA;
  rc = run_reduce<R>(geo_of(*grid), mode, a, h, rhr, b, b_is_f64, buf + 4, buf, s) ? MPDATA_E_CUDA : MPDATA_OK;
  double out[4] = {0, 0, 0, 0};
  if (!rc && cudaMemcpyAsync(out, buf, sizeof out, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = MPDATA_E_CUDA;
  cudaFreeAsync(buf, s);
  if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = MPDATA_E_CUDA;
  if (!rc) memcpy(host_out, out, sizeof out);
  return rc;
}

}  // namespace

extern "C" {

int mpdata_mass_f64(const mpdata_grid* grid, const double* psi, const double* h, const double* rhr,
                    double* mass, void* stream) {
  if (!psi || !h || !mass) return MPDATA_E_NULL;
  double out[4];
  int rc = reduce_impl<double>(grid, 0, psi, h, rhr, nullptr, 1, out, stream);
  if (!rc) *mass = out[0];
  return rc;
}
int mpdata_mass_f32(const mpdata_grid* grid, const float* psi, const float* h, const float* rhr,
                    double* mass, void* stream) {
  if (!psi || !h || !mass) return MPDATA_E_NULL;
  double out[4];
  int rc = reduce_impl<float>(grid, 0, psi, h, rhr, nullptr, 1, out, stream);
  if (!rc) *mass = out[0];
  return rc;
}

int mpdata_error_norms(const mpdata_grid* grid, const void* a, int a_is_f64, const void* b, int b_is_f64,
                       double* out, void* stream) {
  if (!a || !b || !out) return MPDATA_E_NULL;
  double r[4];
  int rc = a_is_f64 ? reduce_impl<double>(grid, 1, (const double*)a, nullptr, nullptr, b, b_is_f64, r, stream)
                    : reduce_impl<float>(grid, 1, (const float*)a, nullptr, nullptr, b, b_is_f64, r, stream);
  if (rc) return rc;
  out[0] = r[2];             // max |a-b|
  out[1] = sqrt(r[0]);       // ||a-b||_2
  out[2] = r[3];             // max |b|
  out[3] = sqrt(r[1]);       // ||b||_2
  return MPDATA_OK;
}

}  // extern "C"

// ===========================================================================
// Adjoint (include/mpdata.h, mpdata_step_adjoint_*, mpdata_adjoint_run_*)
// ===========================================================================
namespace {

template <class R>
int adj_plan(Workspace* w, Prob<R>* P, AdjPlan<R>* A, const R* psi_in, const R* u1, const R* u2, const R* u3,
             const R* h, const R* rhr, const R* bcx, const R* bcy, R* lambda, R* gu1, R* gu2, R* gu3) {
  if (w->elem != sizeof(R)) return MPDATA_E_WS;
  const int iord = w->o.iord;
  if (iord < 2 || iord - 1 > kAdjMaxPass) return MPDATA_E_UNSUPPORTED;
  if (!psi_in || !u1 || !u2 || !u3 || !h || !rhr || !lambda || !gu1 || !gu2 || !gu3) return MPDATA_E_NULL;
  if ((!w->g.ibcx && !bcx) || (!w->g.ibcy && !bcy)) return MPDATA_E_NULL;
  const size_t nrec = adj_record_fields(iord), nacc = adj_acc_fields(iord), n = w->ncell;
  if (!w->adj && cudaMalloc(&w->adj, (nrec + nacc) * n * w->elem) != cudaSuccess) {
    cudaGetLastError();
    w->adj = nullptr;
    return MPDATA_E_CUDA;
  }
  R* base = static_cast<R*>(w->mem);
  *P = make_prob<R>(w->g, w->o.gauge, const_cast<R*>(psi_in), u1, u2, u3, h, rhr, bcx, bcy, base, w->ncell,
                    base + (size_t)NFIELD * w->ncell, 1);
  const mpdata_grid& g = w->g;
  const int ih = g.ih, sx = g.np + 2 * ih, sy = g.mp + 2 * ih;
  R* a = static_cast<R*>(w->adj);
  size_t f = 0;
  auto next = [&]() { return scratch_view<R>(a + (f++) * n, P->g); };
  A->npass = iord - 1;
  for (int t = 0; t < A->npass; t++) {
    A->x[t] = next();
    for (int c = 0; c < 3; c++) A->v[t][c] = next();
    for (int c = 0; c < 3; c++) A->w[t][c] = next();
    A->cp[t] = next();
    A->cn[t] = next();
    A->mx[t] = next();
    A->mn[t] = next();
    for (int c = 0; c < 3; c++) A->fns[t][c] = next();
    A->q[t] = next();
  }
  A->acc = a + f * n;  // the accumulators, contiguous
  for (int t = 0; t < A->npass; t++) {
    A->lx[t] = next();
    for (int c = 0; c < 3; c++) A->lw[t][c] = next();
    A->lmx[t] = next();
    A->lmn[t] = next();
  }
  A->pass_acc = a + f * n;
  for (int c = 0; c < 3; c++) A->lv[c] = next();
  A->lcp = next();
  A->lcn = next();
  for (int c = 0; c < 3; c++) A->lg[c] = next();
  for (int c = 0; c < 3; c++) A->lf[c] = next();
  A->lq = next();
  A->pass_acc_elems = 12 * n;
  A->lxin = next();
  A->acc_elems = (size_t)(a + f * n - A->acc);
  A->lam = caller_view<R>(lambda, ih, sx, sy);
  A->gu1 = caller_view<R>(gu1, ih, sx + 1, sy);
  A->gu2 = caller_view<R>(gu2, ih, sx, sy + 1);
  A->gu3 = caller_view<R>(gu3, ih, sx, sy);
  A->rho = false;
  A->lm1 = A->lm2 = A->lm3 = Arr<R>{nullptr, 0, 0};
  return MPDATA_OK;
}

// Points the record arrays of B at an arena of adj_record_fields fields of n
// elements, in adj_plan's order (the accumulators stay shared).
template <class R>
void repoint_records(AdjPlan<R>* B, R* a, size_t n, const Geo& g) {
  size_t f = 0;
  auto next = [&]() { return scratch_view<R>(a + (f++) * n, g); };
  for (int t = 0; t < B->npass; t++) {
    B->x[t] = next();
    for (int c = 0; c < 3; c++) B->v[t][c] = next();
    for (int c = 0; c < 3; c++) B->w[t][c] = next();
    B->cp[t] = next();
    B->cn[t] = next();
    B->mx[t] = next();
    B->mn[t] = next();
    for (int c = 0; c < 3; c++) B->fns[t][c] = next();
    B->q[t] = next();
  }
}

template <class R>
int step_adjoint_impl(void* ws, const R* psi_in, const R* u1, const R* u2, const R* u3, const R* h, const R* rhr,
                      const R* bcx, const R* bcy, R* lambda, R* gu1, R* gu2, R* gu3, void* stream) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  Prob<R> P;
  AdjPlan<R> A;
  int rc = adj_plan<R>(w, &P, &A, psi_in, u1, u2, u3, h, rhr, bcx, bcy, lambda, gu1, gu2, gu3);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  w->last = s;
  return run_step_adjoint<R>(P, A, w->o.nonos, s) ? MPDATA_E_CUDA : MPDATA_OK;
}

// J = 0.5*|psi_N - target|^2 and its gradients over nsteps steps, with
// checkpoints every `interval` steps (default ceil(sqrt(nsteps))): the
// forward run keeps ceil(nsteps/interval) states; the reverse sweep rebuilds
// each segment's states from its checkpoint and runs the step adjoints
// backwards.  When one record arena per step of a segment fits in half of
// the free device memory, the rebuild runs the record kernels themselves
// (each step's records and its output state in one pass) and the reverse
// kernels read those records, so each step runs forward twice instead of
// three times.  Peak extra memory: (checkpoints + interval) psi-sized arrays,
// plus (interval - 1) record arenas when they are kept.
template <class R>
int adjoint_run_impl(void* ws, int nsteps, int interval, R* psi, const R* u1, const R* u2, const R* u3,
                     const R* h, const R* rhr, const R* bcx, const R* bcy, const R* target, double* J,
                     R* g_psi0, R* gu1, R* gu2, R* gu3, long long* peak_bytes, void* stream) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (nsteps < 1 || interval < 0) return MPDATA_E_OPTS;
  if (!psi || !target || !J || !g_psi0) return MPDATA_E_NULL;
  Prob<R> P;
  AdjPlan<R> A;
  int rc = adj_plan<R>(w, &P, &A, psi, u1, u2, u3, h, rhr, bcx, bcy, g_psi0, gu1, gu2, gu3);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  w->last = s;
  int K = interval;
  if (K == 0) {
    K = 1;
    while ((long long)K * K < nsteps) K++;
  }
  if (K > nsteps) K = nsteps;
  const int nck = (nsteps + K - 1) / K;
  const mpdata_grid& g = w->g;
  const int ih = g.ih, sx = g.np + 2 * ih, sy = g.mp + 2 * ih;
  const size_t plen = (size_t)sx * sy * (g.lp + 2 * ih);
  const size_t pbytes = plen * sizeof(R);
  R* ck = nullptr;   // nck checkpoints
  R* seg = nullptr;  // K states of one segment
  double* red = nullptr;
  const size_t nred = (size_t)reduce_blocks() * 6 + 4;
  if (cudaMallocAsync(&ck, pbytes * nck, s) != cudaSuccess || cudaMallocAsync(&seg, pbytes * K, s) != cudaSuccess ||
      cudaMallocAsync(&red, nred * sizeof(double), s) != cudaSuccess) {
    cudaGetLastError();
    if (ck) cudaFreeAsync(ck, s);
    if (seg) cudaFreeAsync(seg, s);
    return MPDATA_E_CUDA;
  }
  // one record arena per step of a segment (the workspace's own is the first)
  const size_t nrec = adj_record_fields(w->o.iord);
  const size_t rec_bytes = nrec * w->ncell * w->elem;
  R* recs = nullptr;
  {
    size_t free_b = 0, total_b = 0;
    if (K > 1 && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && (size_t)(K - 1) * rec_bytes < free_b / 2 &&
        cudaMallocAsync(&recs, (size_t)(K - 1) * rec_bytes, s) != cudaSuccess) {
      cudaGetLastError();
      recs = nullptr;
    }
  }
  std::vector<AdjPlan<R>> plans;
  if (recs) {
    plans.assign((size_t)K, A);
    for (int k = 1; k < K; k++) repoint_records<R>(&plans[k], recs + (size_t)(k - 1) * nrec * w->ncell, w->ncell, P.g);
  }
  if (peak_bytes)
    *peak_bytes = (long long)(pbytes * (nck + K)) + (long long)(recs ? (size_t)(K - 1) * rec_bytes : 0) +
                  (long long)(w->ncell * w->elem * (NSCRATCH + nrec + adj_acc_fields(w->o.iord)));
  R* base = static_cast<R*>(w->mem);
  auto fwd = [&](R* state) -> int {
    Prob<R> F = make_prob<R>(g, w->o.gauge, state, u1, u2, u3, h, rhr, bcx, bcy, base, w->ncell,
                             base + (size_t)NFIELD * w->ncell, 1);
    return ws_step<R>(w, F, nullptr, s);
  };
  // forward sweep with checkpoints
  for (int n = 0; n < nsteps && !rc; n++) {
    if (n % K == 0 &&
        cudaMemcpyAsync(ck + (size_t)(n / K) * plen, psi, pbytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      rc = MPDATA_E_CUDA;
    if (!rc && fwd(psi)) rc = MPDATA_E_CUDA;
  }
  // J and the seed lambda = psi_N - target (into g_psi0)
  double out[4] = {0, 0, 0, 0};
  if (!rc && run_reduce<R>(P.g, 1, psi, nullptr, nullptr, target, sizeof(R) == 8, red + 4, red, s))
    rc = MPDATA_E_CUDA;
  if (!rc && cudaMemcpyAsync(out, red, sizeof out, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = MPDATA_E_CUDA;
  if (!rc && cudaMemsetAsync(g_psi0, 0, pbytes, s) != cudaSuccess) rc = MPDATA_E_CUDA;
  if (!rc && run_seed<R>(P, caller_view<R>(psi, ih, sx, sy), caller_view<R>(const_cast<R*>(target), ih, sx, sy),
                         A.lam, s))
    rc = MPDATA_E_CUDA;
  // reverse sweep, segment by segment
  for (int c = nck - 1; c >= 0 && !rc; c--) {
    const int n0 = c * K, n1 = (n0 + K < nsteps) ? n0 + K : nsteps;
    if (cudaMemcpyAsync(seg, ck + (size_t)c * plen, pbytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      rc = MPDATA_E_CUDA;
      break;
    }
    if (recs) {
      // records of every step of the segment, each step's output into the next state
      for (int n = n0; n < n1 && !rc; n++) {
        R* src = seg + (size_t)(n - n0) * plen;
        Prob<R> B = P;
        B.psi = caller_view<R>(src, ih, sx, sy);
        const bool more = n + 1 < n1;  // the segment's last output is the next checkpoint
        const Arr<R> next = caller_view<R>(more ? src + plen : src, ih, sx, sy);
        if (more && cudaMemcpyAsync(src + plen, src, pbytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
          rc = MPDATA_E_CUDA;
        if (!rc && run_step_record<R>(B, plans[n - n0], w->o.nonos, more ? &next : nullptr, s))
          rc = MPDATA_E_CUDA;
      }
      for (int n = n1 - 1; n >= n0 && !rc; n--) {
        Prob<R> B = P;
        B.psi = caller_view<R>(seg + (size_t)(n - n0) * plen, ih, sx, sy);
        if (run_step_reverse<R>(B, plans[n - n0], w->o.nonos, s)) rc = MPDATA_E_CUDA;
      }
      continue;
    }
    for (int n = n0 + 1; n < n1 && !rc; n++) {
      R* dst = seg + (size_t)(n - n0) * plen;
      if (cudaMemcpyAsync(dst, dst - plen, pbytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess || fwd(dst) != 0)
        rc = MPDATA_E_CUDA;
    }
    for (int n = n1 - 1; n >= n0 && !rc; n--) {
      Prob<R> B = P;
      B.psi = caller_view<R>(seg + (size_t)(n - n0) * plen, ih, sx, sy);
      if (run_step_adjoint<R>(B, A, w->o.nonos, s)) rc = MPDATA_E_CUDA;
    }
  }
  cudaFreeAsync(ck, s);
  cudaFreeAsync(seg, s);
  cudaFreeAsync(red, s);
  if (recs) cudaFreeAsync(recs, s);
  if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = MPDATA_E_CUDA;
  if (!rc) *J = 0.5 * out[0];
  return rc;
}

template <class R>
__global__ void __launch_bounds__(256) k_fill(R* p, size_t n, R v) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    p[t] = v;
}

// Adjoint of the density step after its predictor: the forward is recorded
// with the density step's arithmetic (upwind without rhr, division by h),
// the outputs' reverse turns the x_incomp, pexr and rhr cotangents into one
// of psi, and the step's reverse adds the mass fluxes' cotangents to the
// upwind and last limited fluxes.  The reverse kernels read a field of ones
// as rhr (the density step has none).
template <class R>
int rho_adjoint_impl(void* ws, const R* u1, const R* u2, const R* u3, const R* x_in, const R* x_incomp, const R* h,
                     const R* pexe, const R* bcx, const R* bcy, R* lambda, const R* l_u1, const R* l_u2,
                     const R* l_u3, const R* l_xincomp, const R* l_pexr1, const R* l_pexr2, const R* l_rhr, R* g_u1,
                     R* g_u2, R* g_u3, R* g_xincomp, R* g_pexe, void* stream) {
  Workspace* w = as_ws(ws);
  if (!w) return MPDATA_E_WS;
  if (w->elem != sizeof(R)) return MPDATA_E_WS;
  if (!w->o.gauge) return MPDATA_E_OPTS;  // the reference's density step is the gauge form
  if (!x_incomp || !pexe || !g_xincomp || !g_pexe) return MPDATA_E_NULL;
  if ((l_u1 || l_u2 || l_u3) && !(l_u1 && l_u2 && l_u3)) return MPDATA_E_NULL;
  const mpdata_grid& g = w->g;
  const int ih = g.ih, sx = g.np + 2 * ih, sy = g.mp + 2 * ih;
  const size_t plen = (size_t)sx * sy * (g.lp + 2 * ih);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  R* buf = nullptr;  // rhr's ones (psi-shaped), then the step's output field (interior)
  if (cudaMallocAsync(&buf, (plen + w->ncell) * sizeof(R), s) != cudaSuccess) {
    cudaGetLastError();
    return MPDATA_E_CUDA;
  }
  k_fill<R><<<1216, 256, 0, s>>>(buf, plen, R(1));
  add_launches(1);
  Prob<R> P;
  AdjPlan<R> A;
  int rc = adj_plan<R>(w, &P, &A, x_in, u1, u2, u3, h, buf, bcx, bcy, lambda, g_u1, g_u2, g_u3);
  if (!rc) {
    w->last = s;
    P.rho = 1;
    P.x_incomp = caller_view<R>(const_cast<R*>(x_incomp), ih, sx, sy);
    P.pexe = caller_view<R>(const_cast<R*>(pexe), ih, sx, sy);
    P.rhoadv = A.lq;  // the recorded upwind copies x_incomp there; the reverse clears it
    R* hi = static_cast<R*>(w->mem) + (size_t)NSCRATCH * w->ncell;
    P.f1hi = hi;
    P.f2hi = hi + (size_t)g.mp * g.lp;
    P.f3hi = hi + (size_t)g.mp * g.lp + (size_t)g.np * g.lp;
    A.rho = true;
    if (l_u1) {
      A.lm1 = caller_view<R>(const_cast<R*>(l_u1), ih, sx + 1, sy);
      A.lm2 = caller_view<R>(const_cast<R*>(l_u2), ih, sx, sy + 1);
      A.lm3 = caller_view<R>(const_cast<R*>(l_u3), ih, sx, sy);
    }
    const Arr<R> out = scratch_view<R>(buf + plen, P.g);
    auto cv = [&](const R* p) { return p ? caller_view<R>(const_cast<R*>(p), ih, sx, sy) : Arr<R>{nullptr, 0, 0}; };
    if (run_step_record<R>(P, A, w->o.nonos, &out, s) ||
        run_rho_out_adjoint<R>(P, out, cv(l_xincomp), cv(l_pexr1), cv(l_pexr2), cv(l_rhr), A.lam,
                               caller_view<R>(g_xincomp, ih, sx, sy), caller_view<R>(g_pexe, ih, sx, sy), s) ||
        run_step_reverse<R>(P, A, w->o.nonos, s))
      rc = MPDATA_E_CUDA;
  }
  cudaFreeAsync(buf, s);
  return rc;
}

}  // namespace

extern "C" {

int mpdata_rho_gauge_adjoint_f64(void* ws, const double* u1, const double* u2, const double* u3,
                                 const double* x_in, const double* x_incomp, const double* h,
                                 const double* pexe, const double* bcx, const double* bcy, double* lambda,
                                 const double* l_u1, const double* l_u2, const double* l_u3,
                                 const double* l_xincomp, const double* l_pexr1, const double* l_pexr2,
                                 const double* l_rhr, double* g_u1, double* g_u2, double* g_u3,
                                 double* g_xincomp, double* g_pexe, void* stream) {
  return rho_adjoint_impl<double>(ws, u1, u2, u3, x_in, x_incomp, h, pexe, bcx, bcy, lambda, l_u1, l_u2, l_u3,
                                  l_xincomp, l_pexr1, l_pexr2, l_rhr, g_u1, g_u2, g_u3, g_xincomp, g_pexe, stream);
}
int mpdata_rho_gauge_adjoint_f32(void* ws, const float* u1, const float* u2, const float* u3, const float* x_in,
                                 const float* x_incomp, const float* h, const float* pexe, const float* bcx,
                                 const float* bcy, float* lambda, const float* l_u1, const float* l_u2,
                                 const float* l_u3, const float* l_xincomp, const float* l_pexr1,
                                 const float* l_pexr2, const float* l_rhr, float* g_u1, float* g_u2, float* g_u3,
                                 float* g_xincomp, float* g_pexe, void* stream) {
  return rho_adjoint_impl<float>(ws, u1, u2, u3, x_in, x_incomp, h, pexe, bcx, bcy, lambda, l_u1, l_u2, l_u3,
                                 l_xincomp, l_pexr1, l_pexr2, l_rhr, g_u1, g_u2, g_u3, g_xincomp, g_pexe, stream);
}

int mpdata_step_adjoint_f64(void* ws, const double* psi_in, const double* u1, const double* u2,
                            const double* u3, const double* h, const double* rhr, const double* bcx,
                            const double* bcy, double* lambda, double* g_u1, double* g_u2, double* g_u3,
                            void* stream) {
  return step_adjoint_impl<double>(ws, psi_in, u1, u2, u3, h, rhr, bcx, bcy, lambda, g_u1, g_u2, g_u3, stream);
}
int mpdata_step_adjoint_f32(void* ws, const float* psi_in, const float* u1, const float* u2, const float* u3,
                            const float* h, const float* rhr, const float* bcx, const float* bcy,
                            float* lambda, float* g_u1, float* g_u2, float* g_u3, void* stream) {
  return step_adjoint_impl<float>(ws, psi_in, u1, u2, u3, h, rhr, bcx, bcy, lambda, g_u1, g_u2, g_u3, stream);
}

int mpdata_adjoint_run_f64(void* ws, int nsteps, int interval, double* psi, const double* u1,
                           const double* u2, const double* u3, const double* h, const double* rhr,
                           const double* bcx, const double* bcy, const double* target, double* J,
                           double* g_psi0, double* g_u1, double* g_u2, double* g_u3,
                           long long* peak_bytes, void* stream) {
  return adjoint_run_impl<double>(ws, nsteps, interval, psi, u1, u2, u3, h, rhr, bcx, bcy, target, J, g_psi0,
                                  g_u1, g_u2, g_u3, peak_bytes, stream);
}
int mpdata_adjoint_run_f32(void* ws, int nsteps, int interval, float* psi, const float* u1, const float* u2,
                           const float* u3, const float* h, const float* rhr, const float* bcx,
                           const float* bcy, const float* target, double* J, float* g_psi0, float* g_u1,
                           float* g_u2, float* g_u3, long long* peak_bytes, void* stream) {
  return adjoint_run_impl<float>(ws, nsteps, interval, psi, u1, u2, u3, h, rhr, bcx, bcy, target, J, g_psi0,
                                 g_u1, g_u2, g_u3, peak_bytes, stream);
}

}  // extern "C"
