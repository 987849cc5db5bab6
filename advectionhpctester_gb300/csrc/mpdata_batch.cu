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

#define BATCH_ARGS const Prob<R>* __restrict__ probs, const unsigned long long* __restrict__ tiles

template <class R, bool ANTIDIFF, bool HALO>
__global__ void __launch_bounds__(256) kb_upwind(BATCH_ARGS) {
#define B(IN) upwind_body<R, ANTIDIFF, HALO, IN>(P, i, j, k)
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
__global__ void __launch_bounds__(256) kb_pseudo(BATCH_ARGS) {
#define B(IN) pseudo_body<R, AIN, IN>(P, i, j, k)
  BATCH_TILE(B)
#undef B
}
template <class R, bool NONOS, bool FIRST, bool KEEP>
__global__ void __launch_bounds__(256) kb_bounds(BATCH_ARGS) {
#define B(IN) bounds_body<R, NONOS, FIRST, KEEP, IN, true>(P, i, j, k)
  BATCH_TILE(B)
#undef B
}
template <class R, bool NONOS>
__global__ void __launch_bounds__(256) kb_limit(BATCH_ARGS) {
#define B(IN) limit_body<R, NONOS, IN>(P, i, j, k)
  BATCH_TILE(B)
#undef B
}
template <class R, bool LAST>
__global__ void __launch_bounds__(256) kb_update(BATCH_ARGS) {
#define B(IN) update_body<R, LAST, IN>(P, i, j, k)
  BATCH_TILE(B)
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
