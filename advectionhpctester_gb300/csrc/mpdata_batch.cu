// Batched MPDATA step: many problems (tracers sharing one velocity, or
// independent domains of uneven sizes) advanced with ONE launch per stage.
//
// The reference advects up to 12 fields that share one velocity with a
// single fused upwind kernel and one antidiffusion call per field
// (advection/src_drivers/advection_CEtimestep_twostep_GPUBC.f90:193-339).
// Here every stage of every problem is one persistent launch: each block
// takes a contiguous chunk of tiles from the concatenated tile space of all
// problems and runs the same per-cell bodies as the single-problem path
// (mpdata_body.cuh) on the problem descriptor it stages in shared memory.
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

// Walk this block's chunk of tiles; BODY sees P (shared), i, j, k.
#define BATCH_LOOP(BODY)                                                                     \
  __shared__ __align__(16) unsigned char sraw[sizeof(Prob<R>)];                              \
  Prob<R>& P = *reinterpret_cast<Prob<R>*>(sraw);                                            \
  const long long chunk = (tiles + gridDim.x - 1) / gridDim.x;                               \
  const long long t0 = (long long)blockIdx.x * chunk;                                        \
  const long long t1 = t0 + chunk < tiles ? t0 + chunk : tiles;                              \
  int p = -1;                                                                                \
  long long pend = -1, pbeg = 0;                                                             \
  int ntx = 1, nty = 1;                                                                      \
  for (long long t = t0; t < t1; t++) {                                                      \
    if (t >= pend) {                                                                         \
      if (p < 0) {                                                                           \
        int lo = 0, hi = nprob - 1;                                                          \
        while (lo < hi) {                                                                    \
          const int mid = (lo + hi + 1) >> 1;                                                \
          if (__ldg(prefix + mid) <= t) lo = mid; else hi = mid - 1;                         \
        }                                                                                    \
        p = lo;                                                                              \
      } else {                                                                               \
        do { p++; } while (__ldg(prefix + p + 1) <= t);                                      \
      }                                                                                      \
      pbeg = __ldg(prefix + p);                                                              \
      pend = __ldg(prefix + p + 1);                                                          \
      __syncthreads();                                                                       \
      load_prob<R>(P, probs, p);                                                             \
      __syncthreads();                                                                       \
      ntx = (P.g.np + blockDim.x - 1) / blockDim.x;                                          \
      nty = (P.g.mp + blockDim.y - 1) / blockDim.y;                                          \
    }                                                                                        \
    long long lt = t - pbeg;                                                                 \
    const int tx = (int)(lt % ntx);                                                          \
    lt /= ntx;                                                                               \
    const int ty = (int)(lt % nty);                                                          \
    const int k = (int)(lt / nty) + 1;                                                       \
    const int i = tx * blockDim.x + threadIdx.x + 1;                                         \
    const int j = ty * blockDim.y + threadIdx.y + 1;                                         \
    if (i <= P.g.np && j <= P.g.mp) { BODY; }                                                \
  }

#define BATCH_ARGS const Prob<R>* __restrict__ probs, const long long* __restrict__ prefix, int nprob, \
                   long long tiles

template <class R, bool ANTIDIFF, bool HALO>
__global__ void __launch_bounds__(256) kb_upwind(BATCH_ARGS) {
  BATCH_LOOP((upwind_body<R, ANTIDIFF, HALO>(P, i, j, k)))
}
template <class R>
__global__ void __launch_bounds__(256) kb_copy(BATCH_ARGS) {
  BATCH_LOOP((copy_body<R>(P, i, j, k)))
}
template <class R, bool AIN>
__global__ void __launch_bounds__(256) kb_pseudo(BATCH_ARGS) {
  BATCH_LOOP((pseudo_body<R, AIN>(P, i, j, k)))
}
template <class R, bool NONOS, bool FIRST, bool KEEP>
__global__ void __launch_bounds__(256) kb_bounds(BATCH_ARGS) {
  BATCH_LOOP((bounds_body<R, NONOS, FIRST, KEEP>(P, i, j, k)))
}
template <class R, bool NONOS>
__global__ void __launch_bounds__(256) kb_limit(BATCH_ARGS) {
  BATCH_LOOP((limit_body<R, NONOS>(P, i, j, k)))
}
template <class R, bool LAST>
__global__ void __launch_bounds__(256) kb_update(BATCH_ARGS) {
  BATCH_LOOP((update_body<R, LAST>(P, i, j, k)))
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
  const int G = B.grid;
#define A B.probs, B.prefix, B.nprob, B.tiles
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

// Resident blocks per SM of the heaviest batched kernel for a block shape.
template <class R>
int batch_occupancy(int threads) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_pseudo<R, true>, threads, 0) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}
template int batch_occupancy<double>(int);
template int batch_occupancy<float>(int);

}  // namespace mpdata
