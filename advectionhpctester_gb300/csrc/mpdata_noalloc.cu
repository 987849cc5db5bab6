// MPDATA step for callers that must not allocate device memory.
//
// Some host programs cannot let a library call cudaMalloc once their time
// loop runs: a model that reserves its whole device-memory budget up front
// through its own pool (so a stray allocation would fail or fragment it), or a
// code whose memory use is audited at start-up and must stay fixed.  For them
// this file offers mpdata_step_noalloc_f64: the same FP64 step as
// mpdata_step_f64, but its scratch fields live in one file-scope device array
// of fixed size instead of a workspace from mpdata_ws_create.
//
// Limits and rules (also stated in include/mpdata.h):
//  - grids of at most MPDATA_NOALLOC_MAX_CELLS interior cells (np*mp*lp);
//    larger grids are rejected with MPDATA_E_TOO_LARGE;
//  - every GPU that loads the library holds the array (19 * 32768 doubles,
//    about 5 MB) until the process exits;
//  - the first call on a device looks up the array's device address (with
//    that device current) and keeps it for the life of the process; make
//    that first call before any stream capture, and make no call on a device
//    after cudaDeviceReset there (the array may then sit elsewhere);
//  - all calls share the one array, so calls that overlap on the GPU (on
//    different streams, or from different host threads) race; order them;
//  - every scratch value a step reads is written earlier in the same step,
//    so nothing has to be cleared between calls.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/mpdata.h"
#include "mpdata_body.cuh"
#include "mpdata_stages.cuh"

using namespace mpdata;

namespace mpdata {
int grid_ok(const mpdata_grid* g);  // the workspace path's checks (mpdata_capi.cu)
int opts_ok(const mpdata_opts* o);
}

namespace {

constexpr int NOALLOC_FIELDS = 19;  // xant v1..3 f1..3 w1..3 cp cn mx mn q | hinv hmx hmy hmz
constexpr long long NOALLOC_CELLS = MPDATA_NOALLOC_MAX_CELLS;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_FIELDS * NOALLOC_CELLS];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
double* g_addr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device (looked up once
// per device; the host-side symbol itself is not a device address).
int scratch_on_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return MPDATA_E_CUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return MPDATA_E_CUDA;
    }
    g_addr[dev] = static_cast<double*>(p);
  }
  *out = g_addr[dev];
  return MPDATA_OK;
}

Arr<double> caller(const double* base, int ih, int n0, int n1) {
  const long sy = n0, sz = (long)n0 * n1;
  return Arr<double>{const_cast<double*>(base) + ih + ih * sy + ih * sz, (int)sy, (int)sz};
}

}  // namespace

extern "C" int mpdata_step_noalloc_f64(const mpdata_grid* grid, const mpdata_opts* opts, double* psi,
                                       const double* u1, const double* u2, const double* u3,
                                       const double* h, const double* rhr, const double* bcx,
                                       const double* bcy, void* stream) {
  // the same checks as a workspace, then this entry point's own limits
  int rc = grid_ok(grid);
  if (rc) return rc;
  rc = opts_ok(opts);
  if (rc) return rc;
  const mpdata_grid g = *grid;
  if ((long long)g.np * g.mp * g.lp > NOALLOC_CELLS) return MPDATA_E_TOO_LARGE;
  if (opts->precision != 64) return MPDATA_E_OPTS;
  if (!psi || !u1 || !u2 || !u3 || !h || !rhr) return MPDATA_E_NULL;
  if ((!g.ibcx && !bcx) || (!g.ibcy && !bcy)) return MPDATA_E_NULL;
  double* scratch = nullptr;
  rc = scratch_on_device(&scratch);
  if (rc) return rc;

  const int ih = g.ih, sx = g.np + 2 * ih, sy = g.mp + 2 * ih;
  const size_t ncell = (size_t)g.np * g.mp * g.lp;
  Prob<double> P;
  memset(&P, 0, sizeof P);
  P.g = Geo{g.np, g.mp, g.lp, g.ih, g.ibcx, g.ibcy, g.ibcz};
  P.stdf = opts->gauge ? 0 : 1;
  P.own_vel = 1;
  P.psi = caller(psi, ih, sx, sy);
  P.u1 = caller(u1, ih, sx + 1, sy);
  P.u2 = caller(u2, ih, sx, sy + 1);
  P.u3 = caller(u3, ih, sx, sy);
  P.h = caller(h, ih, sx, sy);
  P.rhr = caller(rhr, ih, sx, sy);
  P.bcx = bcx;
  P.bcy = bcy;
  Arr<double>* slots[NOALLOC_FIELDS] = {&P.xant, &P.v1, &P.v2, &P.v3, &P.f1, &P.f2, &P.f3,
                                        &P.w1,   &P.w2, &P.w3, &P.cp, &P.cn, &P.mx, &P.mn,
                                        &P.q,    &P.hinv, &P.hmx, &P.hmy, &P.hmz};
  for (int f = 0; f < NOALLOC_FIELDS; f++)
    *slots[f] = Arr<double>{scratch + (size_t)f * ncell, g.np, g.np * g.mp};
  return run_step<double>(P, opts->iord, opts->nonos, nullptr, static_cast<cudaStream_t>(stream)) == 0
             ? MPDATA_OK
             : MPDATA_E_CUDA;
}
