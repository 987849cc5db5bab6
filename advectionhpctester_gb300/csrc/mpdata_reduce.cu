// FP64 compensated reductions over the interior of psi-shaped arrays: the
// global mass sum(h*psi[/rhr]) and the error norms of one field against
// another (e.g. an FP32 run against the FP64 run).  The reference reduces
// with MPI_ALLREDUCE over plain sums (common/mpi_parallel.f90:826-880,
// advection_test_setup.f90:472-617); here every partial sum is an FP64
// Neumaier (sum, compensation) pair, merged with two-sum at every level, so
// the result is independent of the field's precision and nearly of the
// reduction order.
#include "mpdata_common.cuh"
#include "mpdata_stages.cuh"

namespace mpdata {

// Neumaier accumulator (Neumaier 1974, "Rundungsfehleranalyse einiger
// Verfahren zur Summation endlicher Summen"): s + c carries the sum.
struct Neu {
  double s, c;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ void merge(const Neu& o) {
    add(o.s);
    c += o.c;
  }
};

template <class T>
__device__ __forceinline__ double ldv(const T* p, long idx) { return (double)p[idx]; }

// Each block folds a grid-stride range of cells into one Neumaier pair per
// quantity and writes it to part[blockIdx.x * NQ + q].
template <class R, int MODE>
__global__ void __launch_bounds__(256) k_sums(Geo g, const R* __restrict__ a, const R* __restrict__ h,
                                              const R* __restrict__ rhr, const void* __restrict__ b,
                                              int b_is_f64, double* __restrict__ part) {
  // MODE 0: mass  [sum h*a(/rhr)]
  // MODE 1: norms [sum (a-b)^2, sum b^2, max|a-b|, max|b|]
  const long sx = g.np + 2 * g.ih, sy = g.mp + 2 * g.ih;
  const long n = (long)g.np * g.mp * g.lp;
  Neu s0{0.0, 0.0}, s1{0.0, 0.0};
  double m0 = 0.0, m1 = 0.0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
    const long i = c % g.np, j = (c / g.np) % g.mp, k = c / ((long)g.np * g.mp);
    const long idx = (i + g.ih) + (j + g.ih) * sx + (k + g.ih) * sx * sy;
    const double av = ldv(a, idx);
    if (MODE == 0) {
      double v = av * ldv(h, idx);
      if (rhr) v = v / ldv(rhr, idx);
      s0.add(v);
    } else {
      const double bv = b_is_f64 ? ldv((const double*)b, idx) : ldv((const float*)b, idx);
      const double d = av - bv;
      s0.add(d * d);
      s1.add(bv * bv);
      m0 = fmax(m0, fabs(d));
      m1 = fmax(m1, fabs(bv));
    }
  }
  __shared__ double sh[256][6];
  const int t = threadIdx.x;
  sh[t][0] = s0.s; sh[t][1] = s0.c; sh[t][2] = s1.s; sh[t][3] = s1.c; sh[t][4] = m0; sh[t][5] = m1;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      Neu x{sh[t][0], sh[t][1]}, y{sh[t][2], sh[t][3]};
      x.merge(Neu{sh[t + w][0], sh[t + w][1]});
      y.merge(Neu{sh[t + w][2], sh[t + w][3]});
      sh[t][0] = x.s; sh[t][1] = x.c; sh[t][2] = y.s; sh[t][3] = y.c;
      sh[t][4] = fmax(sh[t][4], sh[t + w][4]);
      sh[t][5] = fmax(sh[t][5], sh[t + w][5]);
    }
    __syncthreads();
  }
  if (t == 0)
    for (int q = 0; q < 6; q++) part[blockIdx.x * 6 + q] = sh[0][q];
}

// Final fold of the per-block pairs by one block.
__global__ void __launch_bounds__(256) k_fold(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  __shared__ double sh[256][6];
  const int t = threadIdx.x;
  Neu x{0.0, 0.0}, y{0.0, 0.0};
  double m0 = 0.0, m1 = 0.0;
  for (int b = t; b < nblk; b += blockDim.x) {
    x.merge(Neu{part[b * 6 + 0], part[b * 6 + 1]});
    y.merge(Neu{part[b * 6 + 2], part[b * 6 + 3]});
    m0 = fmax(m0, part[b * 6 + 4]);
    m1 = fmax(m1, part[b * 6 + 5]);
  }
  sh[t][0] = x.s; sh[t][1] = x.c; sh[t][2] = y.s; sh[t][3] = y.c; sh[t][4] = m0; sh[t][5] = m1;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      Neu a{sh[t][0], sh[t][1]}, c{sh[t][2], sh[t][3]};
      a.merge(Neu{sh[t + w][0], sh[t + w][1]});
      c.merge(Neu{sh[t + w][2], sh[t + w][3]});
      sh[t][0] = a.s; sh[t][1] = a.c; sh[t][2] = c.s; sh[t][3] = c.c;
      sh[t][4] = fmax(sh[t][4], sh[t + w][4]);
      sh[t][5] = fmax(sh[t][5], sh[t + w][5]);
    }
    __syncthreads();
  }
  if (t == 0) {
    out[0] = sh[0][0] + sh[0][1];  // compensated sum 0
    out[1] = sh[0][2] + sh[0][3];  // compensated sum 1
    out[2] = sh[0][4];
    out[3] = sh[0][5];
  }
}

constexpr int RED_BLOCKS = 1216;  // 8 blocks per SM on 152 SMs

// out (device, 4 doubles): MODE 0 -> [mass, 0, 0, 0]; MODE 1 -> [sum d^2, sum b^2, max|d|, max|b|]
template <class R>
int run_reduce(Geo g, int mode, const R* a, const R* h, const R* rhr, const void* b, int b_is_f64,
               double* part, double* out, cudaStream_t s) {
  if (mode == 0)
    k_sums<R, 0><<<RED_BLOCKS, 256, 0, s>>>(g, a, h, rhr, b, b_is_f64, part);
  else
    k_sums<R, 1><<<RED_BLOCKS, 256, 0, s>>>(g, a, h, rhr, b, b_is_f64, part);
  k_fold<<<1, 256, 0, s>>>(part, RED_BLOCKS, out);
  add_launches(2);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
template int run_reduce<double>(Geo, int, const double*, const double*, const double*, const void*, int,
                                double*, double*, cudaStream_t);
template int run_reduce<float>(Geo, int, const float*, const float*, const float*, const void*, int,
                               double*, double*, cudaStream_t);
int reduce_blocks() { return RED_BLOCKS; }

// Limiter-bound violations: interior cells whose value lies outside
// [mn - tol, mx + tol], mn/mx the running extrema the nonoscillatory limiter
// kept over the step.  psi, mx and mn are views (logical (1,1,1) bases).
template <class R>
__global__ void __launch_bounds__(256) k_bound_violations(Geo g, Arr<R> psi, Arr<R> mx, Arr<R> mn, double tol,
                                                           unsigned long long* count) {
  unsigned long long c = 0;
  const long n = (long)g.np * g.mp * g.lp;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.np) + 1;
    const long r = t / g.np;
    const int j = (int)(r % g.mp) + 1, k = (int)(r / g.mp) + 1;
    const double v = (double)psi.ld(i, j, k);
    if (v > (double)mx.ld(i, j, k) + tol || v < (double)mn.ld(i, j, k) - tol) c++;
  }
  for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(0xffffffffu, c, d);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

template <class R>
int run_bound_violations(Geo g, const Arr<R>& psi, const Arr<R>& mx, const Arr<R>& mn, double tol,
                         unsigned long long* count, cudaStream_t s) {
  k_bound_violations<R><<<RED_BLOCKS, 256, 0, s>>>(g, psi, mx, mn, tol, count);
  add_launches(1);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
template int run_bound_violations<double>(Geo, const Arr<double>&, const Arr<double>&, const Arr<double>&,
                                          double, unsigned long long*, cudaStream_t);
template int run_bound_violations<float>(Geo, const Arr<float>&, const Arr<float>&, const Arr<float>&, double,
                                         unsigned long long*, cudaStream_t);

}  // namespace mpdata
