// Batched MPDATA step: many problems (tracers sharing one velocity, or
// independent domains of uneven sizes) advanced with ONE launch per stage.
//
// The reference advects up to 12 fields that share one velocity with a
// single fused upwind kernel and one antidiffusion call per field
// (advection/src_drivers/advection_CEtimestep_twostep_GPUBC.f90:193-339).
// Here every stage of every problem is one launch over the concatenated tile
// space of all problems: each block takes one tile, stages its problem's
// descriptor in shared memory and runs the same per-cell bodies as the
// single-problem path (mpdata_body.cuh).
// Problems of one velocity group share the velocity-derived scratch (1/h and
// the face reciprocal densities), computed once by the group's first problem.
#include "mpdata_body.cuh"
#include "mpdata_stages.cuh"

namespace mpdata {

// Stage the descriptor of problem p in shared memory (all threads call).
template <class R>
__device__ __forceinline__ void load_prob(Prob<R>& sP, const Prob<R>* __restrict__ probs, int p) {
  static_assert(sizeof(Prob<R>) % 8 == 0, "descriptor is copied as 8-byte words");
  const int nt = blockDim.x * blockDim.y, tid = threadIdx.y * blockDim.x + threadIdx.x;
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(probs + p);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sP);
  for (int w = tid; w < (int)(sizeof(Prob<R>) / 8); w += nt) dst[w] = __ldg(src + w);
}

// One tile per block.  tiles[blockIdx.x] packs the problem (bits 0-15) and
// the tile's x index (16-31), y index (32-47) and plane k-1 (48-63); the
// host builds the list for the current block shape.  BODY(IN) sees P
// (shared), i, j, k; interior warps take IN = true.
#define BATCH_TILE(BODY)                                                                     \
  __shared__ __align__(16) unsigned char sraw[sizeof(Prob<R>)];                              \
  Prob<R>& P = *reinterpret_cast<Prob<R>*>(sraw);                                            \
  const unsigned long long w = __ldg(tiles + blockIdx.x);                                    \
  load_prob<R>(P, probs, (int)(w & 0xffffu));                                                \
  __syncthreads();                                                                           \
  const int i = (int)((w >> 16) & 0xffffu) * (int)blockDim.x + (int)threadIdx.x + 1;         \
  const int j = (int)((w >> 32) & 0xffffu) * (int)blockDim.y + (int)threadIdx.y + 1;         \
  const int k = (int)(w >> 48) + 1;                                                          \
  const bool win = warp_interior(P.g, i, j, k);                                              \
  if (i <= P.g.np && j <= P.g.mp) {                                                          \
    if (win) {                                                                               \
      BODY(true);                                                                            \
    } else {                                                                                 \
      BODY(false);                                                                           \
    }                                                                                        \
  }

// As BATCH_TILE, with the unit-density instantiation BODY(IN, U) for interior
// warps whose densities are all exactly 1 (FP64).
#define BATCH_TILE_U(BODY)                                                                   \
  __shared__ __align__(16) unsigned char sraw[sizeof(Prob<R>)];                              \
  Prob<R>& P = *reinterpret_cast<Prob<R>*>(sraw);                                            \
  const unsigned long long w = __ldg(tiles + blockIdx.x);                                    \
  load_prob<R>(P, probs, (int)(w & 0xffffu));                                                \
  __syncthreads();                                                                           \
  const int i = (int)((w >> 16) & 0xffffu) * (int)blockDim.x + (int)threadIdx.x + 1;         \
  const int j = (int)((w >> 32) & 0xffffu) * (int)blockDim.y + (int)threadIdx.y + 1;         \
  const int k = (int)(w >> 48) + 1;                                                          \
  const bool win = warp_interior(P.g, i, j, k);                                              \
  if (i <= P.g.np && j <= P.g.mp) {                                                          \
    if (!win) {                                                                              \
      BODY(false, false);                                                                    \
    } else if (warp_unit_cell(P, i, j, k)) {                                                 \
      BODY(true, true);                                                                      \
    } else {                                                                                 \
      BODY(true, false);                                                                     \
    }                                                                                        \
  }

#define BATCH_ARGS const Prob<R>* __restrict__ probs, const unsigned long long* __restrict__ tiles

// Launch bounds of the tile kernels: minimum resident 256-thread blocks per
// SM (0: no explicit bound), the single-problem kernels' register budgets in
// 256-thread units.  Together they made the batch study 4-8% faster than no
// bound.  Build-time overridable for tuning sweeps.
#ifndef MPDATA_MINB_KB_UPWIND
#define MPDATA_MINB_KB_UPWIND 4
#endif
#ifndef MPDATA_MINB_KB_BOUNDS
#define MPDATA_MINB_KB_BOUNDS 6
#endif
#ifndef MPDATA_MINB_KB_LIMIT
#define MPDATA_MINB_KB_LIMIT 8
#endif
#if MPDATA_MINB_KB_UPWIND > 0
#define KB_LB_UPWIND __launch_bounds__(256, MPDATA_MINB_KB_UPWIND)
#else
#define KB_LB_UPWIND __launch_bounds__(256)
#endif
#if MPDATA_MINB_KB_BOUNDS > 0
#define KB_LB_BOUNDS __launch_bounds__(256, MPDATA_MINB_KB_BOUNDS)
#else
#define KB_LB_BOUNDS __launch_bounds__(256)
#endif
#if MPDATA_MINB_KB_LIMIT > 0
#define KB_LB_LIMIT __launch_bounds__(256, MPDATA_MINB_KB_LIMIT)
#else
#define KB_LB_LIMIT __launch_bounds__(256)
#endif

template <class R, bool ANTIDIFF, bool HALO>
__global__ void KB_LB_UPWIND kb_upwind(BATCH_ARGS) {
#define B(IN, U) upwind_body<R, ANTIDIFF, HALO, IN, U, false>(P, i, j, k)
  BATCH_TILE_U(B)
#undef B
}
// pair sums for the FP64 gauge problems (P.pairs), as k_pairs, with the
// velocity pairs except in the first pass of a gauge velocity group, whose
// interior warps read the group's precomputed sums (gvf) instead
template <class R>
__device__ __forceinline__ bool batch_vpairs(const Prob<R>& P, bool ain) {
  return P.pairs && !(ain && (P.gv & 1));
}
template <class R, bool AIN>
__global__ void __launch_bounds__(256) kb_pairs(BATCH_ARGS) {
#define B(IN)                                    \
  if (batch_vpairs(P, AIN))                      \
    pairs_body<R, AIN, true>(P, i, j, k);        \
  else if (P.pairs)                              \
    pairs_body<R, AIN, false>(P, i, j, k)
  BATCH_TILE(B)
#undef B
}
template <class R>
__global__ void __launch_bounds__(256) kb_copy(BATCH_ARGS) {
#define B(IN) copy_body<R>(P, i, j, k)
  BATCH_TILE(B)
#undef B
}
template <class R, bool AIN>
__device__ __forceinline__ void pseudo_dispatch(const Prob<R>& P, int i, int j, int k, bool win, bool pin) {
  if constexpr (AIN) {
    // first pass of a velocity group: its form's velocity-only terms are precomputed
    if (win && (P.stdf ? (P.gv & 2) : (P.gv & 1))) {
      if (warp_unit_faces(P, i, j, k)) {
        if (P.pairs)
          pseudo_body<R, AIN, true, true, true, true, false>(P, i, j, k);
        else
          pseudo_body<R, AIN, true, true, false, true, false>(P, i, j, k);
      } else {
        if (P.pairs)
          pseudo_body<R, AIN, true, false, true, true, false>(P, i, j, k);
        else
          pseudo_body<R, AIN, true, false, false, true, false>(P, i, j, k);
      }
      return;
    }
  }
  if (!win) {
    if constexpr (sizeof(R) == 8) {
      if (pin) {  // a full warp at a boundary: the stored pairs through the boundary maps
        if (warp_unit_faces(P, i, j, k))
          pseudo_body<R, AIN, false, true, true, false, false, true>(P, i, j, k);
        else
          pseudo_body<R, AIN, false, false, true, false, false, true>(P, i, j, k);
        return;
      }
    }
    pseudo_body<R, AIN, false, false, false, false, false>(P, i, j, k);
  } else if constexpr (sizeof(R) == 8) {
    const bool unit = warp_unit_faces(P, i, j, k);
    if (P.pairs) {  // outside the group branch above, the velocity pairs are stored too
      if (unit)
        pseudo_body<R, AIN, true, true, true, false, false, true>(P, i, j, k);
      else
        pseudo_body<R, AIN, true, false, true, false, false, true>(P, i, j, k);
    } else {
      if (unit)
        pseudo_body<R, AIN, true, true, false, false, false>(P, i, j, k);
      else
        pseudo_body<R, AIN, true, false, false, false, false>(P, i, j, k);
    }
  } else {
    pseudo_body<R, AIN, true, false, false, false, false>(P, i, j, k);
  }
}
template <class R, bool AIN>
__global__ void __launch_bounds__(256) kb_pseudo(BATCH_ARGS) {
  __shared__ __align__(16) unsigned char sraw[sizeof(Prob<R>)];
  Prob<R>& P = *reinterpret_cast<Prob<R>*>(sraw);
  const unsigned long long w = __ldg(tiles + blockIdx.x);
  load_prob<R>(P, probs, (int)(w & 0xffffu));
  __syncthreads();
  const int i = (int)((w >> 16) & 0xffffu) * (int)blockDim.x + (int)threadIdx.x + 1;
  const int j = (int)((w >> 32) & 0xffffu) * (int)blockDim.y + (int)threadIdx.y + 1;
  const int k = (int)(w >> 48) + 1;
  const bool win = warp_interior(P.g, i, j, k);
  // FP64 problems with every pair sum stored: full warps at a boundary read
  // them through the boundary maps (P is the block's problem: uniform)
  bool pin = false;
  if constexpr (sizeof(R) == 8)
    if (!win && batch_vpairs(P, AIN)) pin = warp_on_grid(P.g, i, j);
  if (i <= P.g.np && j <= P.g.mp) pseudo_dispatch<R, AIN>(P, i, j, k, win, pin);
}
template <class R, bool NONOS, bool FIRST, bool KEEP>
__global__ void KB_LB_BOUNDS kb_bounds(BATCH_ARGS) {
  if constexpr (NONOS && sizeof(R) == 8) {  // FP32: per-lane quotients are cheaper than the barriers
    __shared__ __align__(16) unsigned char sraw[sizeof(Prob<R>)];
    Prob<R>& P = *reinterpret_cast<Prob<R>*>(sraw);
    const unsigned long long w = __ldg(tiles + blockIdx.x);
    load_prob<R>(P, probs, (int)(w & 0xffffu));
    __syncthreads();
    const int i = (int)((w >> 16) & 0xffffu) * (int)blockDim.x + (int)threadIdx.x + 1;
    const int j = (int)((w >> 32) & 0xffffu) * (int)blockDim.y + (int)threadIdx.y + 1;
    const int k = (int)(w >> 48) + 1;
    const bool win = warp_interior(P.g, i, j, k);
    const bool valid = i <= P.g.np && j <= P.g.mp;
    RatioOps<R> r{};
    if (valid) {
      if (!win)
        r = bounds_body<R, true, FIRST, KEEP, false, 2, false, false>(P, i, j, k);
      else if (warp_unit_cell(P, i, j, k))
        r = bounds_body<R, true, FIRST, KEEP, true, 2, true, false>(P, i, j, k);
      else
        r = bounds_body<R, true, FIRST, KEEP, true, 2, false, false>(P, i, j, k);
    }
    block_ratios(P, i, j, k, valid, r);
  } else {
#define B(IN, U) bounds_body<R, NONOS, FIRST, KEEP, IN, 1, U, false>(P, i, j, k)
    BATCH_TILE_U(B)
#undef B
  }
}
template <class R, bool NONOS>
__global__ void KB_LB_LIMIT kb_limit(BATCH_ARGS) {
#define B(IN) limit_body<R, NONOS, IN, false>(P, i, j, k)
  BATCH_TILE(B)
#undef B
}
template <class R, bool LAST>
__global__ void __launch_bounds__(256) kb_update(BATCH_ARGS) {
#define B(IN, U) update_body<R, LAST, IN, U>(P, i, j, k)
  BATCH_TILE_U(B)
#undef B
}

#define BLAUNCH(stage, ...)                  \
  do {                                       \
    if (prof) prof->begin(stage, s);         \
    __VA_ARGS__;                             \
    if (prof) prof->end(stage, s);           \
    add_launches(1);                         \
  } while (0)

template <class R>
int run_batch(const BatchLaunch<R>& B, Prof* prof, cudaStream_t s) {
  const dim3 blk(B.bx, B.by, 1);
  const int G = B.ntiles;
#define A B.probs, B.tiles
  if (B.iord < 2) {
    if (B.halo) {
      BLAUNCH(ST_UPWIND, (kb_upwind<R, false, true><<<G, blk, 0, s>>>(A)));
      BLAUNCH(ST_COPY, (kb_copy<R><<<G, blk, 0, s>>>(A)));
    } else {
      BLAUNCH(ST_UPWIND, (kb_upwind<R, false, false><<<G, blk, 0, s>>>(A)));
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
  }
  if (B.halo) BLAUNCH(ST_UPWIND, (kb_upwind<R, true, true><<<G, blk, 0, s>>>(A)));
  else BLAUNCH(ST_UPWIND, (kb_upwind<R, true, false><<<G, blk, 0, s>>>(A)));
  const bool keep = B.iord > 2;
  for (int pass = 2; pass <= B.iord; pass++) {
    const bool first = (pass == 2), last = (pass == B.iord) && B.halo;
    if (B.pairs && first) BLAUNCH(ST_PAIRS, (kb_pairs<R, true><<<G, blk, 0, s>>>(A)));
    else if (B.pairs) BLAUNCH(ST_PAIRS, (kb_pairs<R, false><<<G, blk, 0, s>>>(A)));
    if (first) BLAUNCH(ST_PSEUDO, (kb_pseudo<R, true><<<G, blk, 0, s>>>(A)));
    else BLAUNCH(ST_PSEUDO, (kb_pseudo<R, false><<<G, blk, 0, s>>>(A)));
    if (!B.nonos) BLAUNCH(ST_BOUNDS, (kb_bounds<R, false, true, false><<<G, blk, 0, s>>>(A)));
    else if (first && keep) BLAUNCH(ST_BOUNDS, (kb_bounds<R, true, true, true><<<G, blk, 0, s>>>(A)));
    else if (first) BLAUNCH(ST_BOUNDS, (kb_bounds<R, true, true, false><<<G, blk, 0, s>>>(A)));
    else BLAUNCH(ST_BOUNDS, (kb_bounds<R, true, false, true><<<G, blk, 0, s>>>(A)));
    if (B.nonos) BLAUNCH(ST_LIMIT, (kb_limit<R, true><<<G, blk, 0, s>>>(A)));
    else BLAUNCH(ST_LIMIT, (kb_limit<R, false><<<G, blk, 0, s>>>(A)));
    if (last) BLAUNCH(ST_UPDATE, (kb_update<R, true><<<G, blk, 0, s>>>(A)));
    else BLAUNCH(ST_UPDATE, (kb_update<R, false><<<G, blk, 0, s>>>(A)));
  }
#undef A
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

template int run_batch<double>(const BatchLaunch<double>&, Prof*, cudaStream_t);
template int run_batch<float>(const BatchLaunch<float>&, Prof*, cudaStream_t);


}  // namespace mpdata
