// Single-problem launch sequence of the MPDATA step (strict-IEEE path).
//
// One kernel per stage of the reference's antidiffusive iteration, one thread
// per cell, every face quantity computed exactly once (the reference
// recomputes shared faces per cell).  The per-cell arithmetic lives in
// mpdata_body.cuh.  Built with --fmad=false and IEEE division, so results are
// bit-identical to a strict-IEEE CPU evaluation of the reference's
// expressions (up to the sign of zero).
#include "mpdata_body.cuh"
#include "mpdata_stages.cuh"

namespace mpdata {

#define CELL_INDEX                                          \
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1; \
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1; \
  const int k = blockIdx.z + 1;                             \
  if (i > P.g.np || j > P.g.mp) return;

// Interior warps take the body without boundary maps (IN = true).
#define CELL_DISPATCH(BODY)                                 \
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1; \
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1; \
  const int k = blockIdx.z + 1;                             \
  const bool win = warp_interior(P.g, i, j, k);             \
  if (i > P.g.np || j > P.g.mp) return;                     \
  if (win) {                                                \
    BODY(true);                                             \
  } else {                                                  \
    BODY(false);                                            \
  }

// As CELL_DISPATCH, with the unit-density instantiation (BODY(IN, U)) for
// interior warps whose densities are all exactly 1.
#define CELL_DISPATCH_U(BODY)                               \
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1; \
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1; \
  const int k = blockIdx.z + 1;                             \
  const bool win = warp_interior(P.g, i, j, k);             \
  if (i > P.g.np || j > P.g.mp) return;                     \
  if (!win) {                                               \
    BODY(false, false);                                     \
  } else if (warp_unit_cell(P, i, j, k)) {                  \
    BODY(true, true);                                       \
  } else {                                                  \
    BODY(true, false);                                      \
  }

// Minimum resident 128-thread blocks per SM asked of the register allocator
// for the upwind, limiter-bounds and limited-flux kernels.  An explicit bound
// is always given: with none, or with 1, ptxas allots these kernels far more
// registers (k_limit 32 -> 56, k_upwind 48 -> 78 in FP32) and they run
// slower.  FP64 values from a sweep at 512x512x128 (upwind 8: -3%, bounds 12:
// -13% with a 12-byte spill, limit 16: -7%); FP32 from a sweep too (upwind
// 12: -12%, bounds 16: -4%, limit 16 and pseudo 8 as they were).
// Build-time overridable for tuning sweeps.
#ifndef MPDATA_MINB_UPWIND_F64
#define MPDATA_MINB_UPWIND_F64 8
#endif
#ifndef MPDATA_MINB_BOUNDS_F64
#define MPDATA_MINB_BOUNDS_F64 12
#endif
#ifndef MPDATA_MINB_LIMIT_F64
#define MPDATA_MINB_LIMIT_F64 16
#endif
#ifndef MPDATA_MINB_UPWIND_F32
#define MPDATA_MINB_UPWIND_F32 12
#endif
#ifndef MPDATA_MINB_BOUNDS_F32
#define MPDATA_MINB_BOUNDS_F32 16
#endif
#ifndef MPDATA_MINB_LIMIT_F32
#define MPDATA_MINB_LIMIT_F32 16
#endif
template <class R, int N64, int N32>
struct MinBlocks {
  static constexpr int v = sizeof(R) == 8 ? N64 : N32;
};

template <class R, bool ANTIDIFF>
__global__ void __launch_bounds__(128, (MinBlocks<R, MPDATA_MINB_UPWIND_F64, MPDATA_MINB_UPWIND_F32>::v)) k_upwind(const Prob<R> P) {
#define B(IN, U) upwind_body<R, ANTIDIFF, true, IN, U>(P, i, j, k)
  CELL_DISPATCH_U(B)
#undef B
}
template <class R>
__global__ void __launch_bounds__(128) k_copy(const Prob<R> P) {
  CELL_INDEX
  copy_body<R>(P, i, j, k);
}
// Minimum resident 128-thread blocks per SM asked of the register allocator
// for the pseudo-velocity kernel, whose interior path keeps ~60 neighbour
// loads in flight: FP32 is latency-bound and gains from 8 blocks (64
// registers, a 12-byte spill); FP64 takes 7 (72 registers, an 8-byte spill),
// which measured 5.02 ms per headline step at 512x512x128 against 5.32 with
// 5 blocks (88 registers) and 5.06 with 6 (80): the FP64 pipe waits on its
// loads (8 long-scoreboard stalls per issue at 5 blocks).  Build-time
// overridable for tuning sweeps.
#ifndef MPDATA_MINB_PSEUDO_F32
#define MPDATA_MINB_PSEUDO_F32 8
#endif
#ifndef MPDATA_MINB_PSEUDO_F64
#define MPDATA_MINB_PSEUDO_F64 7
#endif
template <class R>
struct PseudoMinBlocks {
  static constexpr int v = sizeof(R) == 4 ? MPDATA_MINB_PSEUDO_F32 : MPDATA_MINB_PSEUDO_F64;
};
// Whether the pseudo-velocity kernel issues every load before its stores
// (DEFER, see limit_form) or stores each face at once (fewer registers).
// FP64 measured the same either way, with 5 to 7 resident blocks (the FP64
// pipe is the bound); FP32 gains from DEFER.
#ifndef MPDATA_DEFER_PSEUDO_F64
#define MPDATA_DEFER_PSEUDO_F64 1
#endif
#ifndef MPDATA_DEFER_PSEUDO_F32
#define MPDATA_DEFER_PSEUDO_F32 1
#endif
template <class R>
struct PseudoDefer {
  static constexpr bool v = sizeof(R) == 4 ? MPDATA_DEFER_PSEUDO_F32 : MPDATA_DEFER_PSEUDO_F64;
};

template <class R, bool AIN>
__global__ void __launch_bounds__(128, PseudoMinBlocks<R>::v) k_pseudo(const Prob<R> P) {
  constexpr bool D = PseudoDefer<R>::v;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  const bool win = warp_interior(P.g, i, j, k);
  // FP64 with every pair sum stored: full warps at a boundary read them too,
  // through the boundary maps
  bool pin = false;
  if constexpr (sizeof(R) == 8)
    if (!win && P.pairs == 2) pin = warp_on_grid(P.g, i, j);
  if (i > P.g.np || j > P.g.mp) return;
  if (!win) {
    if constexpr (sizeof(R) == 8) {
      if (pin) {
        if (warp_unit_faces(P, i, j, k))
          pseudo_body<R, AIN, false, true, true, false, D, true>(P, i, j, k);
        else
          pseudo_body<R, AIN, false, false, true, false, D, true>(P, i, j, k);
        return;
      }
    }
    pseudo_body<R, AIN, false, false, false, false, D>(P, i, j, k);
  } else if constexpr (sizeof(R) == 8) {
    const bool unit = warp_unit_faces(P, i, j, k);
    if (P.pairs == 2) {
      if (unit)
        pseudo_body<R, AIN, true, true, true, false, D, true>(P, i, j, k);
      else
        pseudo_body<R, AIN, true, false, true, false, D, true>(P, i, j, k);
    } else if (P.pairs) {
      if (unit)
        pseudo_body<R, AIN, true, true, true, false, D>(P, i, j, k);
      else
        pseudo_body<R, AIN, true, false, true, false, D>(P, i, j, k);
    } else {
      if (unit)
        pseudo_body<R, AIN, true, true, false, false, D>(P, i, j, k);
      else
        pseudo_body<R, AIN, true, false, false, false, D>(P, i, j, k);
    }
  } else {
    pseudo_body<R, AIN, true, false, false, false, D>(P, i, j, k);
  }
}

template <class R, bool AIN, bool PV>
__global__ void __launch_bounds__(128) k_pairs(const Prob<R> P) {
  CELL_INDEX
  pairs_body<R, AIN, PV>(P, i, j, k);
}
template <class R, bool NONOS, bool FIRST, bool KEEP>
__global__ void __launch_bounds__(128, (MinBlocks<R, MPDATA_MINB_BOUNDS_F64, MPDATA_MINB_BOUNDS_F32>::v)) k_bounds(const Prob<R> P) {
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
    CELL_DISPATCH_U(B)
#undef B
  }
}
template <class R, bool NONOS>
__global__ void __launch_bounds__(128, (MinBlocks<R, MPDATA_MINB_LIMIT_F64, MPDATA_MINB_LIMIT_F32>::v)) k_limit(const Prob<R> P) {
#define B(IN) limit_body<R, NONOS, IN>(P, i, j, k)
  CELL_DISPATCH(B)
#undef B
}
template <class R, bool LAST>
__global__ void __launch_bounds__(128) k_update(const Prob<R> P) {
#define B(IN, U) update_body<R, LAST, IN, U>(P, i, j, k)
  CELL_DISPATCH_U(B)
#undef B
}

template <class R, bool LINER>
__global__ void __launch_bounds__(128) k_rho_out(const Prob<R> P) {
  CELL_INDEX
  rho_out_body<R, LINER>(P, i, j, k);
}

// ---- launch accounting ---------------------------------------------------
static unsigned long long g_launches = 0;
unsigned long long launch_count() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
void add_launches(int n) { __atomic_add_fetch(&g_launches, (unsigned long long)n, __ATOMIC_RELAXED); }

// launch wrapper: optional event pair around the kernel, launch accounting
#define LAUNCH(stage, ...)                   \
  do {                                       \
    if (prof) prof->begin(stage, s);         \
    __VA_ARGS__;                             \
    if (prof) prof->end(stage, s);           \
    add_launches(1);                         \
  } while (0)

template <class R>
int run_step(const Prob<R>& P, int iord, int nonos, Prof* prof, cudaStream_t s) {
  const Geo& g = P.g;
  const dim3 blk(32, 4, 1);
  const dim3 grd((g.np + 31) / 32, (g.mp + 3) / 4, g.lp);
  if (iord < 2) {
    LAUNCH(ST_UPWIND, (k_upwind<R, false><<<grd, blk, 0, s>>>(P)));
    if (P.rho) LAUNCH(ST_RHO_OUT, (k_rho_out<R, true><<<grd, blk, 0, s>>>(P)));
    else LAUNCH(ST_COPY, (k_copy<R><<<grd, blk, 0, s>>>(P)));
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
  }
  LAUNCH(ST_UPWIND, (k_upwind<R, true><<<grd, blk, 0, s>>>(P)));
  const bool keep = iord > 2;
  // FP64 gauge form: the pseudo-velocity stage reads precomputed pair sums of
  // xant (pairs 1) and, outside the density step, whose upwind fluxes hold
  // f1..f3, of the pass velocities too (pairs 2)
  Prob<R> Q = P;
  Q.pairs = (!P.stdf && sizeof(R) == 8) ? (P.rho ? 1 : 2) : 0;
  for (int pass = 2; pass <= iord; pass++) {
    const bool first = (pass == 2), last = (pass == iord);
    if (Q.pairs == 2 && first) LAUNCH(ST_PAIRS, (k_pairs<R, true, true><<<grd, blk, 0, s>>>(Q)));
    else if (Q.pairs == 2) LAUNCH(ST_PAIRS, (k_pairs<R, false, true><<<grd, blk, 0, s>>>(Q)));
    else if (Q.pairs) LAUNCH(ST_PAIRS, (k_pairs<R, true, false><<<grd, blk, 0, s>>>(Q)));
    if (first) LAUNCH(ST_PSEUDO, (k_pseudo<R, true><<<grd, blk, 0, s>>>(Q)));
    else LAUNCH(ST_PSEUDO, (k_pseudo<R, false><<<grd, blk, 0, s>>>(Q)));
    if (!nonos) LAUNCH(ST_BOUNDS, (k_bounds<R, false, true, false><<<grd, blk, 0, s>>>(P)));
    else if (first && keep) LAUNCH(ST_BOUNDS, (k_bounds<R, true, true, true><<<grd, blk, 0, s>>>(P)));
    else if (first) LAUNCH(ST_BOUNDS, (k_bounds<R, true, true, false><<<grd, blk, 0, s>>>(P)));
    else LAUNCH(ST_BOUNDS, (k_bounds<R, true, false, true><<<grd, blk, 0, s>>>(P)));
    if (nonos) LAUNCH(ST_LIMIT, (k_limit<R, true><<<grd, blk, 0, s>>>(P)));
    else LAUNCH(ST_LIMIT, (k_limit<R, false><<<grd, blk, 0, s>>>(P)));
    if (last) LAUNCH(ST_UPDATE, (k_update<R, true><<<grd, blk, 0, s>>>(P)));
    else LAUNCH(ST_UPDATE, (k_update<R, false><<<grd, blk, 0, s>>>(P)));
  }
  if (P.rho) LAUNCH(ST_RHO_OUT, (k_rho_out<R, false><<<grd, blk, 0, s>>>(P)));
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template int run_step<double>(const Prob<double>&, int, int, Prof*, cudaStream_t);
template int run_step<float>(const Prob<float>&, int, int, Prof*, cudaStream_t);

}  // namespace mpdata
