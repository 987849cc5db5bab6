// C ABI of the MPDATA step (include/mpdata.h): argument validation, device
// workspace management and dispatch to the stage kernels.  Errors are
// returned as negative codes; nothing here exits (the reference STOPs on bad
// options, advec.f90:174,203,210).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/mpdata.h"
#include "mpdata_common.cuh"
#include "mpdata_stages.cuh"

using namespace mpdata;

namespace {

constexpr uint32_t WS_MAGIC = 0x4d504454u;  // "MPDT"
constexpr int NSCRATCH = 16;                // xant hinv v1..3 f1..3 w1..3 cp cn mx mn q

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
  size_t elem;
  void* mem;
  int* d_err;
  cudaStream_t last;
  EventProf* prof;
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

template <class R>
StepPlan<R> make_plan(Workspace* w, R* psi, const R* u1, const R* u2, const R* u3, const R* h,
                      const R* rhr, const R* bcx, const R* bcy) {
  const mpdata_grid& g = w->g;
  const int ih = g.ih;
  const int sx = g.np + 2 * ih, sy = g.mp + 2 * ih;
  StepPlan<R> P;
  P.g = geo_of(g);
  P.iord = w->o.iord;
  P.nonos = w->o.nonos;
  P.gauge = w->o.gauge;
  P.psi = caller_view<R>(psi, ih, sx, sy);
  P.u1 = caller_view<R>(const_cast<R*>(u1), ih, sx + 1, sy);
  P.u2 = caller_view<R>(const_cast<R*>(u2), ih, sx, sy + 1);
  P.u3 = caller_view<R>(const_cast<R*>(u3), ih, sx, sy);
  P.h = caller_view<R>(const_cast<R*>(h), ih, sx, sy);
  P.rhr = caller_view<R>(const_cast<R*>(rhr), ih, sx, sy);
  P.bcx = bcx;
  P.bcy = bcy;
  R* base = static_cast<R*>(w->mem);
  Arr<R>* slots[NSCRATCH] = {&P.xant, &P.hinv, &P.v1, &P.v2, &P.v3, &P.f1, &P.f2, &P.f3,
                             &P.w1,   &P.w2,   &P.w3, &P.cp, &P.cn, &P.mx, &P.mn, &P.q};
  for (int s = 0; s < NSCRATCH; s++) *slots[s] = scratch_view<R>(base + (size_t)s * w->ncell, P.g);
  P.prof = w->prof;
  return P;
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
  StepPlan<R> P = make_plan<R>(w, psi, u1, u2, u3, h, rhr, bcx, bcy);
  return run_step<R>(P, s) == 0 ? MPDATA_OK : MPDATA_E_CUDA;
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

// The reference keeps its scratch in module globals allocated once per grid;
// advec_dwarf therefore caches one workspace per (grid, options).
std::mutex g_cache_mu;
std::vector<Workspace*> g_cache;

bool same(const Workspace* w, const mpdata_grid& g, const mpdata_opts& o) {
  return !memcmp(&w->g, &g, sizeof g) && !memcmp(&w->o, &o, sizeof o);
}

template <class R>
int advec_dwarf_impl(int legacyoptmode, int t_adv, int np, int mp, int lp, int ih, int ipoles,
                     int ibcx, int ibcy, int ibcz, R* x, const R* x_lr, const R* x_bt,
                     const R* uadv, const R* vadv, const R* wadv, const R* rhr, const R* rhoadv,
                     int iord, int nonos, void* stream) {
  // advec.f90:148-211
  if (legacyoptmode == 2) return MPDATA_OK;  // CASE(2): the reference's call is commented out
  if (legacyoptmode != 4 && legacyoptmode != 6) return MPDATA_E_OPTS;
  if (legacyoptmode == 4 && t_adv != 1 && t_adv != 2) return MPDATA_E_OPTS;
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
  if (cudaMalloc(&w->mem, w->ncell * w->elem * NSCRATCH) != cudaSuccess) {
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
  (void)lvertsplit;
  return advec_dwarf_impl<double>(legacyoptmode, t_adv, np, mp, lp, ih, ipoles, ibcx, ibcy, ibcz, x,
                                  x_lr, x_bt, uadv, vadv, wadv, rhr, rhoadv, iord, nonos, stream);
}
int mpdata_advec_dwarf_f32(int legacyoptmode, int t_adv, int lupdatemulti, int lvertsplit, int np,
                           int mp, int lp, int ih, int ipoles, int ibcx, int ibcy, int ibcz,
                           float* x, const float* x_lr, const float* x_bt, const float* uadv,
                           const float* vadv, const float* wadv, const float* rhr,
                           const float* rhoadv, int iord, int nonos, void* stream) {
  (void)lupdatemulti;
  (void)lvertsplit;
  return advec_dwarf_impl<float>(legacyoptmode, t_adv, np, mp, lp, ih, ipoles, ibcx, ibcy, ibcz, x,
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
                                      "predictor_cgrid"};
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
    default: return "unknown error";
  }
}

const char* mpdata_version(void) { return "mpdata-gb300 0.1 (sm_103a)"; }

}  // extern "C"
