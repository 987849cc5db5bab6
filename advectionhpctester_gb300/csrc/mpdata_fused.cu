// Fused single-precision MPDATA step on z-marching tiles (periodic grids,
// infinite-gauge form, nonoscillatory limiter).
//
// The stage path runs one kernel per stage of the reference's antidiffusive
// iteration and keeps every intermediate field in HBM; here a step is
//   K1  upwind (upwind3d-gpubc.f90:101-198) + first-pass pseudo-velocities
//       (antidiff3d-gauge-gpubc.f90:157-203)
//   K2  limiter bounds and ratios (:238-324) + limited velocities (:343-363)
//       + corrective update (:364-428), one launch per pass
//   K3  pseudo-velocities of every later pass (the MPDATA recursion)
// so iord=3 is four launches instead of nine.  A block owns a 32x8 column of
// cells and marches it through a chunk of planes.  Every field it reads is
// staged plane by plane in shared memory (40x12 cells: the tile, two halo
// rows and four halo columns, so that a staged row starts on a 16-byte
// boundary), in a ring of as many planes as the stencils reach in z plus one
// plane of prefetch; intermediate fields that only a neighbour needs (the
// upwind field on the tile's one-cell ring, the limiter ratios, the limited
// velocities) never leave shared memory.  Neighbour offsets inside a plane
// are compile-time constants.
//
// Staging: arena fields (this file's own scratch, rows padded to 16 bytes)
// arrive by TMA (cp.async.bulk.tensor, one 40x12 box per field and plane,
// completion on an mbarrier) on tiles whose boxes lie inside the grid; the
// caller's arrays (whose rows need not start on 16-byte boundaries) and the
// tiles at a periodic seam are staged with 4-byte cp.async, each thread
// copying two cells of the box from precomputed wrapped coordinates.  The z
// wrap is the plane index taken modulo lp.
//
// Arithmetic: every expression is the FP32 stage bodies' (mpdata_body.cuh,
// interior path), in the same order, built with --fmad=false, so the result
// is bit for bit that of the stage path and of the FP32 oracle.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdlib>

#include "mpdata_fused.cuh"

namespace mpdata {
namespace {

constexpr int TX = 32, TY = 8, NT = TX * TY;  // tile of output cells, one thread each
constexpr int HX = 4, HY = 2;                 // staged halo columns and rows
constexpr int P = TX + 2 * HX;                // plane pitch: 40
constexpr int NR = TY + 2 * HY;               // plane rows: 12
constexpr int PLANE = P * NR;                 // 480 cells, 1920 bytes
constexpr uint32_t BOX_BYTES = PLANE * 4;
constexpr int NRING1 = 2 * (TX + 2) + 2 * TY;  // the tile's one-cell ring: 84 cells
constexpr int NRINGW = TX + TY;                // faces beyond the tile's last row / column: 40

__device__ __forceinline__ int wrapn(int i, int n) {
  int r = (i - 1) % n;
  if (r < 0) r += n;
  return r + 1;
}
// ring slot of plane k (k >= -2; 12 is a multiple of every ring size)
template <int N>
__device__ __forceinline__ int slot(int k) {
  return (k + 12) % N;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint64_t* m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* m, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait on an mbarrier phase: false when the limit ran out (each
// try_wait suspends for a bounded time, so the limit is a few seconds).
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t parity) {
  for (int it = 0; it < (1 << 22); it++)
    if (mbar_try_wait(m, parity)) return true;
  return false;
}
// One 40x12 box of arena field f, plane z (0-based), into dst.  x must be a
// multiple of 4 (16 bytes of FP32).
__device__ __forceinline__ void tma_box(float* dst, const CUtensorMap* map, int x, int y, int z, int f,
                                        uint64_t* m) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(f), "r"(smem_u32(m))
      : "memory");
}

// Dynamic shared memory rounded up to 128 bytes, the alignment a TMA box
// destination needs (every staged plane is a multiple of 128 bytes from it).
__device__ __forceinline__ float* smem_base() {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const uint32_t off = smem_u32(smem_raw);
  return reinterpret_cast<float*>(smem_raw + ((128u - (off & 127u)) & 127u));
}

struct FzArgs {
  Geo g;
  Arr<float> psi, u1, u2, u3, h, rhr;
  float* arena;
  int px;
  long fs;
  int kchunk;
  int fin, fout;                      // pass input / output field
  int fmx_in, fmn_in, fmx_out, fmn_out;
  int* err;
};

// The two staged cells of thread t: box cells t and t+NT (the second exists
// for t < PLANE-NT), as wrapped 1-based grid coordinates.
struct Box {
  int i0, j0, i1, j1;
  bool two;
};
__device__ __forceinline__ Box box_cells(const Geo& g, int x0, int y0, int t) {
  Box b;
  b.i0 = wrapn(x0 - HX + t % P, g.np);
  b.j0 = wrapn(y0 - HY + t / P, g.mp);
  const int e = t + NT;
  b.two = e < PLANE;
  b.i1 = wrapn(x0 - HX + e % P, g.np);
  b.j1 = wrapn(y0 - HY + e / P, g.mp);
  return b;
}
// a plane of a caller array (any strides) into a staged plane
__device__ __forceinline__ void stage_caller(float* dst, const Arr<float>& A, int kw, const Box& b, int t) {
  const float* base = A.p + (long)(kw - 1) * A.sz;
  cp_async4(dst + t, base + (b.i0 - 1) + (long)(b.j0 - 1) * A.sy);
  if (b.two) cp_async4(dst + t + NT, base + (b.i1 - 1) + (long)(b.j1 - 1) * A.sy);
}
// a plane of an arena field through the wrapped coordinates (seam tiles)
__device__ __forceinline__ void stage_arena(float* dst, const float* fbase, int px, int mp, int kw, const Box& b,
                                            int t) {
  const float* base = fbase + (long)(kw - 1) * px * mp;
  cp_async4(dst + t, base + (b.i0 - 1) + (long)(b.j0 - 1) * px);
  if (b.two) cp_async4(dst + t + NT, base + (b.i1 - 1) + (long)(b.j1 - 1) * px);
}

// smem index of ring cell q of the tile's one-cell ring
__device__ __forceinline__ int ring1_index(int q) {
  int c, r;
  if (q < TX + 2) {
    c = HX - 1 + q;
    r = HY - 1;
  } else if (q < 2 * (TX + 2)) {
    c = HX - 1 + (q - (TX + 2));
    r = HY + TY;
  } else {
    const int s = q - 2 * (TX + 2);
    c = s < TY ? HX - 1 : HX + TX;
    r = HY + (s % TY);
  }
  return r * P + c;
}
// Faces the tile's update reads beyond its cells: the y faces of the row past
// the tile (q < TX) and the x faces of the column past it.
__device__ __forceinline__ int ringw_index(int q) {
  return q < TX ? (HY + TY) * P + HX + q : (HY + (q - TX)) * P + HX + TX;
}

// ---- the stage arithmetic on staged planes (FP32 bodies, interior path) ----

// upwind3d_gpubc at smem cell b of plane k: x0/xm/xp = psi at k, k-1, k+1;
// w3p = u3 at k+1 (the cell's upper face).
__device__ __forceinline__ float upwind_cell(int b, const float* x0, const float* xm, const float* xp,
                                             const float* a1, const float* a2, const float* a3, const float* a3p,
                                             const float* h, const float* rh) {
  const float x = x0[b];
  const float hi = 1.0f / h[b];
  const float f1p = donor(x, x0[b + 1], a1[b + 1]);
  const float f1 = donor(x0[b - 1], x, a1[b]);
  const float f2p = donor(x, x0[b + P], a2[b + P]);
  const float f2 = donor(x0[b - P], x, a2[b]);
  const float f3p = donor(x, xp[b], a3p[b]);
  const float f3 = donor(xm[b], x, a3[b]);
  const float sum = f1p - f1 + f2p - f2 + f3p - f3;
  return (x - sum * hi) * rh[b];
}

// Gauge pseudo-velocities of the cell's three lower faces at plane k:
// X at k-1, k, k+1; A1, A2 (x and y velocities) at k-1, k; A3 at k, k+1;
// h at k-1, k.  pseudo_form<float, false, ...> with IN.
__device__ __forceinline__ void pseudo_cell(int b, const float* xm, const float* x0, const float* xp,
                                            const float* a1m, const float* a10, const float* a2m,
                                            const float* a20, const float* a30, const float* a3p,
                                            const float* hm, const float* h0, float& v1, float& v2, float& v3) {
  const float xc = x0[b];
  {  // x face
    const float hmx = 2.0f / (h0[b - 1] + h0[b]);
    const float a = a10[b];
    const float d2 = (x0[b + P] + x0[b - 1 + P]) - (x0[b - P] + x0[b - 1 - P]);
    const float s2 = (a20[b - 1] + a20[b - 1 + P]) + (a20[b] + a20[b + P]);
    const float d3 = (xp[b] + xp[b - 1]) - (xm[b] + xm[b - 1]);
    const float s3 = (a30[b - 1] + a3p[b - 1]) + (a30[b] + a3p[b]);
    const float cr = s2 * d2 + s3 * d3;
    v1 = (fabsf(a) - a * a * hmx) * (xc - x0[b - 1]) * 0.5f - 0.03125f * a * hmx * cr;
  }
  {  // y face
    const float hmy = 2.0f / (h0[b - P] + h0[b]);
    const float a = a20[b];
    const float d1 = (x0[b + 1] + x0[b + 1 - P]) - (x0[b - 1] + x0[b - 1 - P]);
    const float s1 = (a10[b - P] + a10[b + 1 - P]) + (a10[b] + a10[b + 1]);
    const float d3 = (xp[b] + xp[b - P]) - (xm[b] + xm[b - P]);
    const float s3 = (a30[b - P] + a3p[b - P]) + (a30[b] + a3p[b]);
    const float cr = s1 * d1 + s3 * d3;
    v2 = (fabsf(a) - a * a * hmy) * (xc - x0[b - P]) * 0.5f - 0.03125f * a * hmy * cr;
  }
  {  // z face
    const float hmz = 2.0f / (hm[b] + h0[b]);
    const float a = a30[b];
    const float d1 = (x0[b + 1] + xm[b + 1]) - (x0[b - 1] + xm[b - 1]);
    const float d2 = (x0[b + P] + xm[b + P]) - (x0[b - P] + xm[b - P]);
    const float s1 = (a1m[b] + a1m[b + 1]) + (a10[b] + a10[b + 1]);
    const float s2 = (a2m[b] + a2m[b + P]) + (a20[b] + a20[b + P]);
    const float cr = s1 * d1 + s2 * d2;
    v3 = (fabsf(a) - a * a * hmz) * (xc - xm[b]) * 0.5f - 0.03125f * a * hmz * cr;
  }
}

// Limiter bounds and ratios of cell b at plane k (bounds_body, FP32, IN):
// FIRST folds the star of x_in (s0/sm/sp) before the field's own star;
// later passes start from the running extrema (s0 = mx, sm = mn at k).
template <bool FIRST>
__device__ __forceinline__ void bounds_cell(int b, const float* xm, const float* x0, const float* xp,
                                            const float* s0, const float* sm, const float* sp, const float* v1,
                                            const float* v2, const float* v3, const float* v3p, const float* h,
                                            float& cp, float& cn, float& ma, float& mi) {
  const float x = x0[b];
  if (FIRST) {
    Extrema<float> e(s0[b]);
    e.add(s0[b - 1]);
    e.add(s0[b + 1]);
    e.add(s0[b - P]);
    e.add(s0[b + P]);
    e.add(sm[b]);
    e.add(sp[b]);
    e.add(x);
    e.add(x0[b - 1]);
    e.add(x0[b + 1]);
    e.add(x0[b - P]);
    e.add(x0[b + P]);
    e.add(xm[b]);
    e.add(xp[b]);
    ma = e.max();
    mi = e.min();
  } else {
    Extrema<float> e(x);
    e.add(x0[b - 1]);
    e.add(x0[b + 1]);
    e.add(x0[b - P]);
    e.add(x0[b + P]);
    e.add(xm[b]);
    e.add(xp[b]);
    ma = mx2(s0[b], e.max());
    mi = mn2(sm[b], e.min());
  }
  const float e1 = v1[b + 1], w1 = v1[b], e2 = v2[b + P], w2 = v2[b], e3 = v3p[b], w3 = v3[b];
  const float hc = h[b];
  const float ep = Eps<float>::v;
  const float np_ = (ma - x) * hc, nn = (x - mi) * hc;
  const float dp = pn(e1) + pp(w1) + pn(e2) + pp(w2) + pn(e3) + pp(w3) + ep;
  const float dn = pp(e1) + pn(w1) + pp(e2) + pn(w2) + pp(e3) + pn(w3) + ep;
  cp = lim_ratio(np_, dp);
  cn = lim_ratio(nn, dn);
}

// ---- K1: upwind + first-pass pseudo-velocities ----------------------------
// smem planes: psi 4, u1 4, u2 4, u3 4, h 4, rhr 2, xant 3
constexpr int K1_PLANES = 25;

__global__ void __launch_bounds__(NT, 4) k_fz_upwind_pseudo(const FzArgs A) {
  float* const sm = smem_base();
  float* const PSI = sm;
  float* const U1 = PSI + 4 * PLANE;
  float* const U2 = U1 + 4 * PLANE;
  float* const U3 = U2 + 4 * PLANE;
  float* const H = U3 + 4 * PLANE;
  float* const RH = H + 4 * PLANE;
  float* const XA = RH + 2 * PLANE;
  const Geo& g = A.g;
  const int t = threadIdx.x, tx = t % TX, ty = t / TX;
  const int x0 = blockIdx.x * TX + 1, y0 = blockIdx.y * TY + 1;
  const int kb = blockIdx.z * A.kchunk + 1;
  if (kb > g.lp) return;
  const int ke = min(g.lp, kb + A.kchunk - 1);
  const Box bx = box_cells(g, x0, y0, t);
  const int b = (ty + HY) * P + tx + HX;
  const int br = t < NRING1 ? ring1_index(t) : -1;
  const int ig = x0 + tx, jg = y0 + ty;
  const bool own = ig <= g.np && jg <= g.mp;
  const long pl = (long)A.px * g.mp;
  const long go = (long)(ig - 1) + (long)(jg - 1) * A.px;
  float* const fxin = A.arena + FZ_XIN * A.fs;
  float* const fxa = A.arena + FZ_X0 * A.fs;
  float* const fv1 = A.arena + FZ_V1 * A.fs;
  float* const fv2 = A.arena + FZ_V2 * A.fs;
  float* const fv3 = A.arena + FZ_V3 * A.fs;
#define ST4(R, F, k) stage_caller(R + slot<4>(k) * PLANE, A.F, wrapn((k), g.lp), bx, t)
#define ST2(R, F, k) stage_caller(R + slot<2>(k) * PLANE, A.F, wrapn((k), g.lp), bx, t)
  // what the first step (ko = kb-2) reads and does not stage itself
  for (int k = kb - 2; k <= kb; k++) ST4(PSI, psi, k);
  for (int k = kb - 1; k <= kb; k++) ST4(U3, u3, k);
  ST4(U1, u1, kb - 1);
  ST4(U2, u2, kb - 1);
  ST4(H, h, kb - 1);
  ST2(RH, rhr, kb - 1);
  cp_commit();
  for (int ko = kb - 2; ko <= ke; ko++) {
    cp_wait_all();
    __syncthreads();
    if (ko < ke) {
      ST4(PSI, psi, ko + 3);
      ST4(U3, u3, ko + 3);
      ST4(U1, u1, ko + 2);
      ST4(U2, u2, ko + 2);
      ST4(H, h, ko + 2);
      ST2(RH, rhr, ko + 2);
      cp_commit();
    }
    {  // xant at plane ko+1 on the tile and its ring
      const int k = ko + 1;
      const float* p0 = PSI + slot<4>(k) * PLANE;
      const float* pm = PSI + slot<4>(k - 1) * PLANE;
      const float* pp_ = PSI + slot<4>(k + 1) * PLANE;
      const float* a1 = U1 + slot<4>(k) * PLANE;
      const float* a2 = U2 + slot<4>(k) * PLANE;
      const float* a3 = U3 + slot<4>(k) * PLANE;
      const float* a3p = U3 + slot<4>(k + 1) * PLANE;
      const float* h = H + slot<4>(k) * PLANE;
      const float* rh = RH + slot<2>(k) * PLANE;
      float* xa = XA + slot<3>(k) * PLANE;
      const float v = upwind_cell(b, p0, pm, pp_, a1, a2, a3, a3p, h, rh);
      xa[b] = v;
      if (br >= 0) xa[br] = upwind_cell(br, p0, pm, pp_, a1, a2, a3, a3p, h, rh);
      if (own && k >= kb && k <= ke) {
        fxa[go + (k - 1) * pl] = v;
        fxin[go + (k - 1) * pl] = p0[b];
      }
    }
    __syncthreads();
    if (ko >= kb) {
      float v1, v2, v3;
      pseudo_cell(b, XA + slot<3>(ko - 1) * PLANE, XA + slot<3>(ko) * PLANE, XA + slot<3>(ko + 1) * PLANE,
                  U1 + slot<4>(ko - 1) * PLANE, U1 + slot<4>(ko) * PLANE, U2 + slot<4>(ko - 1) * PLANE,
                  U2 + slot<4>(ko) * PLANE, U3 + slot<4>(ko) * PLANE, U3 + slot<4>(ko + 1) * PLANE,
                  H + slot<4>(ko - 1) * PLANE, H + slot<4>(ko) * PLANE, v1, v2, v3);
      if (own) {
        const long o = go + (ko - 1) * pl;
        fv1[o] = v1;
        fv2[o] = v2;
        fv3[o] = v3;
      }
    }
  }
#undef ST4
#undef ST2
}

// ---- staging of arena fields: TMA on interior tiles, wrapped cp.async else ----
struct Stager {
  const CUtensorMap* map;
  const float* arena;
  long fs;
  int px, mp, lp;
  int xc, yc;  // box origin (0-based) of the tile
  bool tma;
  Box bx;
  int t;
  __device__ __forceinline__ void plane(float* dst, int f, int k, uint64_t* m) const {
    const int kw = wrapn(k, lp);
    if (tma) {
      if (t == 0) tma_box(dst, map, xc, yc, kw - 1, f, m);
    } else {
      stage_arena(dst, arena + f * fs, px, mp, kw, bx, t);
    }
  }
};

// Interior tile: every staged box lies inside the grid, so TMA needs no wrap.
__device__ __forceinline__ bool tile_inside(const Geo& g) {
  return blockIdx.x >= 1 && (int)blockIdx.x * TX + TX + HX <= g.np && blockIdx.y >= 1 &&
         (int)blockIdx.y * TY + TY + HY <= g.mp;
}

// Waits for the staging of the previous iteration (cp.async groups of this
// thread, and the TMA phase of the block), then the block barrier.  Returns
// false (in every thread) when a TMA wait ran out: the error word is set.
__device__ __forceinline__ bool stage_sync(bool tma, uint64_t* mbar, int n, int* s_abort, int* err) {
  cp_wait_all();
  if (tma && n >= 1) {
    if (!mbar_wait(&mbar[(n - 1) & 1], ((n - 1) >> 1) & 1)) {
      *s_abort = 1;
      atomicOr(err, 2);
    }
  }
  __syncthreads();
  return *s_abort == 0;
}

// ---- K2: limiter bounds + limited velocities + update of one pass ----------
// smem planes: x 4, x_in 4 (or mx 2 + mn 2), v1 2, v2 2, v3 3, h 3, cp 2,
// cn 2, w1 2, w2 2; tiles: w3 2, rhr 2
constexpr int K2_PLANES = 26;
constexpr int K2_TILES = 4;

template <bool FIRST, bool LAST, bool KEEP>
__global__ void __launch_bounds__(NT, 4) k_fz_limit(const FzArgs A, const __grid_constant__ CUtensorMap tm) {
  float* const sm = smem_base();
  float* const X = sm;
  float* const S = X + 4 * PLANE;
  float* const V1 = S + 4 * PLANE;
  float* const V2 = V1 + 2 * PLANE;
  float* const V3 = V2 + 2 * PLANE;
  float* const H = V3 + 3 * PLANE;
  float* const CP = H + 3 * PLANE;
  float* const CN = CP + 2 * PLANE;
  float* const W1 = CN + 2 * PLANE;
  float* const W2 = W1 + 2 * PLANE;
  float* const W3 = W2 + 2 * PLANE;
  float* const RH = W3 + 2 * NT;
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ int s_abort;
  const Geo& g = A.g;
  const int t = threadIdx.x, tx = t % TX, ty = t / TX;
  const int x0 = blockIdx.x * TX + 1, y0 = blockIdx.y * TY + 1;
  const int kb = blockIdx.z * A.kchunk + 1;
  if (kb > g.lp) return;
  const int ke = min(g.lp, kb + A.kchunk - 1);
  const bool tma = tile_inside(g);
  const Stager st{&tm, A.arena, A.fs, A.px, g.mp, g.lp, x0 - 1 - HX, y0 - 1 - HY, tma, box_cells(g, x0, y0, t), t};
  const int b = (ty + HY) * P + tx + HX;
  const int br = t < NRING1 ? ring1_index(t) : -1;
  const int bw = t < NRINGW ? ringw_index(t) : -1;
  const int ig = x0 + tx, jg = y0 + ty;
  const bool own = ig <= g.np && jg <= g.mp;
  const int ipw = wrapn(ig, g.np), jpw = wrapn(jg, g.mp);
  const long pl = (long)A.px * g.mp;
  const long go = (long)(ig - 1) + (long)(jg - 1) * A.px;
  if (t == 0) {
    s_abort = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  constexpr int NBOX_PRO = FIRST ? 10 : 9;  // boxes staged before the first step
  constexpr int NBOX = FIRST ? 5 : 6;       // boxes staged by each step
  const int fs_ = FIRST ? FZ_XIN : A.fmx_in;
  // staging of the first step's reads
  if (tma && t == 0) mbar_expect_tx(&mbar[0], NBOX_PRO * BOX_BYTES);
  for (int k = kb - 2; k <= kb; k++) {
    st.plane(X + slot<4>(k) * PLANE, A.fin, k, &mbar[0]);
    if (FIRST) st.plane(S + slot<4>(k) * PLANE, FZ_XIN, k, &mbar[0]);
  }
  for (int k = kb - 1; k <= kb; k++) st.plane(V3 + slot<3>(k) * PLANE, FZ_V3, k, &mbar[0]);
  st.plane(V1 + slot<2>(kb - 1) * PLANE, FZ_V1, kb - 1, &mbar[0]);
  st.plane(V2 + slot<2>(kb - 1) * PLANE, FZ_V2, kb - 1, &mbar[0]);
  if (!FIRST) {
    st.plane(S + slot<2>(kb - 1) * PLANE, fs_, kb - 1, &mbar[0]);
    st.plane(S + (2 + slot<2>(kb - 1)) * PLANE, A.fmn_in, kb - 1, &mbar[0]);
  }
  stage_caller(H + slot<3>(kb - 1) * PLANE, A.h, wrapn(kb - 1, g.lp), st.bx, t);
  cp_commit();
  for (int ko = kb - 2; ko <= ke; ko++) {
    const int n = ko - kb + 3;
    if (!stage_sync(tma, mbar, n, &s_abort, A.err)) return;
    if (ko < ke) {
      uint64_t* m = &mbar[n & 1];
      if (tma && t == 0) mbar_expect_tx(m, NBOX * BOX_BYTES);
      st.plane(X + slot<4>(ko + 3) * PLANE, A.fin, ko + 3, m);
      if (FIRST) st.plane(S + slot<4>(ko + 3) * PLANE, FZ_XIN, ko + 3, m);
      st.plane(V3 + slot<3>(ko + 3) * PLANE, FZ_V3, ko + 3, m);
      st.plane(V1 + slot<2>(ko + 2) * PLANE, FZ_V1, ko + 2, m);
      st.plane(V2 + slot<2>(ko + 2) * PLANE, FZ_V2, ko + 2, m);
      if (!FIRST) {
        st.plane(S + slot<2>(ko + 2) * PLANE, fs_, ko + 2, m);
        st.plane(S + (2 + slot<2>(ko + 2)) * PLANE, A.fmn_in, ko + 2, m);
      }
      stage_caller(H + slot<3>(ko + 2) * PLANE, A.h, wrapn(ko + 2, g.lp), st.bx, t);
      {
        const int kw = wrapn(ko + 1, g.lp);
        cp_async4(RH + slot<2>(ko + 1) * NT + t, &A.rhr.p[A.rhr.off(ipw, jpw, kw)]);
      }
      cp_commit();
    }
    // limiter bounds and ratios at plane ko+1, on the tile and its ring
    const int kc = ko + 1;
    {
      const float* xm = X + slot<4>(kc - 1) * PLANE;
      const float* xc = X + slot<4>(kc) * PLANE;
      const float* xp = X + slot<4>(kc + 1) * PLANE;
      const float *s0, *s1, *s2;
      if (FIRST) {
        s0 = S + slot<4>(kc) * PLANE;
        s1 = S + slot<4>(kc - 1) * PLANE;
        s2 = S + slot<4>(kc + 1) * PLANE;
      } else {
        s0 = S + slot<2>(kc) * PLANE;        // mx
        s1 = S + (2 + slot<2>(kc)) * PLANE;  // mn
        s2 = nullptr;
      }
      const float* v1 = V1 + slot<2>(kc) * PLANE;
      const float* v2 = V2 + slot<2>(kc) * PLANE;
      const float* v3 = V3 + slot<3>(kc) * PLANE;
      const float* v3p = V3 + slot<3>(kc + 1) * PLANE;
      const float* h = H + slot<3>(kc) * PLANE;
      float* cp = CP + slot<2>(kc) * PLANE;
      float* cn = CN + slot<2>(kc) * PLANE;
      float rp, rn, ma, mi;
      bounds_cell<FIRST>(b, xm, xc, xp, s0, s1, s2, v1, v2, v3, v3p, h, rp, rn, ma, mi);
      cp[b] = rp;
      cn[b] = rn;
      if (KEEP && own && kc >= kb && kc <= ke) {
        A.arena[A.fmx_out * A.fs + go + (kc - 1) * pl] = ma;
        A.arena[A.fmn_out * A.fs + go + (kc - 1) * pl] = mi;
      }
      if (br >= 0) {
        bounds_cell<FIRST>(br, xm, xc, xp, s0, s1, s2, v1, v2, v3, v3p, h, rp, rn, ma, mi);
        cp[br] = rp;
        cn[br] = rn;
      }
    }
    __syncthreads();
    // limited velocities at plane ko+1 (limit_form, gauge, nonos)
    if (kc >= kb) {
      const float* cp = CP + slot<2>(kc) * PLANE;
      const float* cn = CN + slot<2>(kc) * PLANE;
      const float* cpm = CP + slot<2>(kc - 1) * PLANE;
      const float* cnm = CN + slot<2>(kc - 1) * PLANE;
      const float* v1 = V1 + slot<2>(kc) * PLANE;
      const float* v2 = V2 + slot<2>(kc) * PLANE;
      const float* v3 = V3 + slot<3>(kc) * PLANE;
      float* w1 = W1 + slot<2>(kc) * PLANE;
      float* w2 = W2 + slot<2>(kc) * PLANE;
      const float cpc = cp[b], cnc = cn[b];
      const float r1 = donor(min3(cpc, cn[b - 1]), min3(cp[b - 1], cnc), v1[b]);
      const float r2 = donor(min3(cpc, cn[b - P]), min3(cp[b - P], cnc), v2[b]);
      const float r3 = donor(min3(cpc, cnm[b]), min3(cpm[b], cnc), v3[b]);
      w1[b] = r1;
      w2[b] = r2;
      W3[slot<2>(kc) * NT + t] = r3;
      if (!LAST && own && kc <= ke) {
        const long o = go + (kc - 1) * pl;
        A.arena[FZ_W1 * A.fs + o] = r1;
        A.arena[FZ_W2 * A.fs + o] = r2;
        A.arena[FZ_W3 * A.fs + o] = r3;
      }
      if (bw >= 0) {
        const float cq = cp[bw], nq = cn[bw];
        if (t < TX)
          w2[bw] = donor(min3(cq, cn[bw - P]), min3(cp[bw - P], nq), v2[bw]);
        else
          w1[bw] = donor(min3(cq, cn[bw - 1]), min3(cp[bw - 1], nq), v1[bw]);
      }
    }
    __syncthreads();
    // corrective update of plane ko (update_body, gauge)
    if (ko >= kb) {
      const float* w1 = W1 + slot<2>(ko) * PLANE;
      const float* w2 = W2 + slot<2>(ko) * PLANE;
      const float* w3 = W3 + slot<2>(ko) * NT;
      const float* w3p = W3 + slot<2>(ko + 1) * NT;
      const float* xc = X + slot<4>(ko) * PLANE;
      const float* h = H + slot<3>(ko) * PLANE;
      const float rh = RH[slot<2>(ko) * NT + t];
      const float d = w1[b + 1] - w1[b] + w2[b + P] - w2[b] + w3p[t] - w3[t];
      const float q = xc[b] / rh;
      const float out = (q - d / h[b]) * rh;
      if (own) {
        if (LAST)
          A.psi.at(ig, jg, ko) = out;
        else
          A.arena[A.fout * A.fs + go + (ko - 1) * pl] = out;
      }
    }
  }
}

// ---- K3: pseudo-velocities of a later pass ---------------------------------
// smem planes: x 4, w1 3, w2 3, w3 3, h 3
constexpr int K3_PLANES = 16;

__global__ void __launch_bounds__(NT, 4) k_fz_pseudo(const FzArgs A, const __grid_constant__ CUtensorMap tm) {
  float* const sm = smem_base();
  float* const X = sm;
  float* const A1 = X + 4 * PLANE;
  float* const A2 = A1 + 3 * PLANE;
  float* const A3 = A2 + 3 * PLANE;
  float* const H = A3 + 3 * PLANE;
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ int s_abort;
  const Geo& g = A.g;
  const int t = threadIdx.x, tx = t % TX, ty = t / TX;
  const int x0 = blockIdx.x * TX + 1, y0 = blockIdx.y * TY + 1;
  const int kb = blockIdx.z * A.kchunk + 1;
  if (kb > g.lp) return;
  const int ke = min(g.lp, kb + A.kchunk - 1);
  const bool tma = tile_inside(g);
  const Stager st{&tm, A.arena, A.fs, A.px, g.mp, g.lp, x0 - 1 - HX, y0 - 1 - HY, tma, box_cells(g, x0, y0, t), t};
  const int b = (ty + HY) * P + tx + HX;
  const int ig = x0 + tx, jg = y0 + ty;
  const bool own = ig <= g.np && jg <= g.mp;
  const long pl = (long)A.px * g.mp;
  const long go = (long)(ig - 1) + (long)(jg - 1) * A.px;
  if (t == 0) {
    s_abort = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tma && t == 0) mbar_expect_tx(&mbar[0], 9 * BOX_BYTES);
  for (int k = kb - 1; k <= kb + 1; k++) st.plane(X + slot<4>(k) * PLANE, A.fin, k, &mbar[0]);
  for (int k = kb; k <= kb + 1; k++) st.plane(A3 + slot<3>(k) * PLANE, FZ_W3, k, &mbar[0]);
  for (int k = kb - 1; k <= kb; k++) {
    st.plane(A1 + slot<3>(k) * PLANE, FZ_W1, k, &mbar[0]);
    st.plane(A2 + slot<3>(k) * PLANE, FZ_W2, k, &mbar[0]);
    stage_caller(H + slot<3>(k) * PLANE, A.h, wrapn(k, g.lp), st.bx, t);
  }
  cp_commit();
  for (int ko = kb; ko <= ke; ko++) {
    const int n = ko - kb + 1;
    if (!stage_sync(tma, mbar, n, &s_abort, A.err)) return;
    if (ko < ke) {
      uint64_t* m = &mbar[n & 1];
      if (tma && t == 0) mbar_expect_tx(m, 4 * BOX_BYTES);
      st.plane(X + slot<4>(ko + 2) * PLANE, A.fin, ko + 2, m);
      st.plane(A3 + slot<3>(ko + 2) * PLANE, FZ_W3, ko + 2, m);
      st.plane(A1 + slot<3>(ko + 1) * PLANE, FZ_W1, ko + 1, m);
      st.plane(A2 + slot<3>(ko + 1) * PLANE, FZ_W2, ko + 1, m);
      stage_caller(H + slot<3>(ko + 1) * PLANE, A.h, wrapn(ko + 1, g.lp), st.bx, t);
      cp_commit();
    }
    float v1, v2, v3;
    pseudo_cell(b, X + slot<4>(ko - 1) * PLANE, X + slot<4>(ko) * PLANE, X + slot<4>(ko + 1) * PLANE,
                A1 + slot<3>(ko - 1) * PLANE, A1 + slot<3>(ko) * PLANE, A2 + slot<3>(ko - 1) * PLANE,
                A2 + slot<3>(ko) * PLANE, A3 + slot<3>(ko) * PLANE, A3 + slot<3>(ko + 1) * PLANE,
                H + slot<3>(ko - 1) * PLANE, H + slot<3>(ko) * PLANE, v1, v2, v3);
    if (own) {
      const long o = go + (ko - 1) * pl;
      A.arena[FZ_V1 * A.fs + o] = v1;
      A.arena[FZ_V2 * A.fs + o] = v2;
      A.arena[FZ_V3 * A.fs + o] = v3;
    }
  }
}

constexpr size_t K1_SMEM = (size_t)K1_PLANES * PLANE * 4 + 128;
constexpr size_t K2_SMEM = (size_t)K2_PLANES * PLANE * 4 + (size_t)K2_TILES * NT * 4 + 128;
constexpr size_t K3_SMEM = (size_t)K3_PLANES * PLANE * 4 + 128;

template <class K>
int set_smem(K kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess ? 0
                                                                                                                : -5;
}

int init_kernels() {
  static int rc = [] {
    int r = 0;
    r |= set_smem(k_fz_upwind_pseudo, K1_SMEM);
    r |= set_smem(k_fz_limit<true, true, false>, K2_SMEM);
    r |= set_smem(k_fz_limit<true, false, true>, K2_SMEM);
    r |= set_smem(k_fz_limit<false, false, true>, K2_SMEM);
    r |= set_smem(k_fz_limit<false, true, true>, K2_SMEM);
    r |= set_smem(k_fz_pseudo, K3_SMEM);
    return r;
  }();
  return rc;
}

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

}  // namespace

bool fused_eligible(const Geo& g, int precision, int gauge, int nonos, int iord, int rho) {
  if (const char* e = std::getenv("MPDATA_FUSED")) {
    if (e[0] == '0') return false;  // stage path forced (comparisons and tests)
  }
  return precision == 32 && gauge && nonos && iord >= 2 && !rho && g.bx && g.by && g.bz;
}

size_t fused_arena_elems(const Geo& g, int* px) {
  const int p = (g.np + 3) / 4 * 4;
  if (px) *px = p;
  return (size_t)FZ_NF * p * g.mp * g.lp;
}

int fused_make_tmap(CUtensorMap* map, float* arena, int px, const Geo& g) {
  static EncodeTiled enc = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<EncodeTiled>(fn);
  }();
  if (!enc) return -5;
  const cuuint64_t dims[4] = {(cuuint64_t)px, (cuuint64_t)g.mp, (cuuint64_t)g.lp, (cuuint64_t)FZ_NF};
  const cuuint64_t strides[3] = {(cuuint64_t)px * 4, (cuuint64_t)px * g.mp * 4, (cuuint64_t)px * g.mp * g.lp * 4};
  const cuuint32_t box[4] = {(cuuint32_t)P, (cuuint32_t)NR, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, arena, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -5;
}

int fused_kchunk(const Geo& g) {
  if (const char* e = std::getenv("MPDATA_FUSED_KCHUNK")) {
    const int v = std::atoi(e);
    if (v > 0) return v;
  }
  // enough blocks for several waves of 4 resident blocks on every SM, with
  // chunks long enough that the march's start-up planes stay a small share
  const long tiles = (long)((g.np + TX - 1) / TX) * ((g.mp + TY - 1) / TY);
  const long want = 152L * 4 * 6;  // about six waves
  int nz = (int)((want + tiles - 1) / tiles);
  if (nz < 1) nz = 1;
  int kc = (g.lp + nz - 1) / nz;
  if (kc < 16) kc = 16;
  if (kc > g.lp) kc = g.lp;
  return kc;
}

#define FZ_LAUNCH(stage, ...)              \
  do {                                     \
    if (prof) prof->begin(stage, s);       \
    __VA_ARGS__;                           \
    if (prof) prof->end(stage, s);         \
    add_launches(1);                       \
  } while (0)

int run_step_fused(const FusedPlan& F, int iord, Prof* prof, cudaStream_t s, int* mx_field, int* mn_field) {
  if (init_kernels()) return -5;
  const Geo& g = F.g;
  FzArgs A;
  A.g = g;
  A.psi = F.psi;
  A.u1 = F.u1;
  A.u2 = F.u2;
  A.u3 = F.u3;
  A.h = F.h;
  A.rhr = F.rhr;
  A.arena = F.arena;
  A.px = F.px;
  A.fs = F.fs;
  A.kchunk = F.kchunk;
  A.err = F.err;
  A.fin = FZ_X0;
  A.fout = FZ_X1;
  A.fmx_in = FZ_MX0;
  A.fmn_in = FZ_MN0;
  A.fmx_out = FZ_MX0;
  A.fmn_out = FZ_MN0;
  const dim3 grid((g.np + TX - 1) / TX, (g.mp + TY - 1) / TY, (g.lp + F.kchunk - 1) / F.kchunk);
  const dim3 blk(NT);
  const CUtensorMap& tm = *F.tmap;
  FZ_LAUNCH(ST_FZ_UPWIND_PSEUDO, (k_fz_upwind_pseudo<<<grid, blk, K1_SMEM, s>>>(A)));
  *mx_field = *mn_field = -1;
  for (int pass = 2; pass <= iord; pass++) {
    const bool first = pass == 2, last = pass == iord;
    if (!first) FZ_LAUNCH(ST_FZ_PSEUDO, (k_fz_pseudo<<<grid, blk, K3_SMEM, s>>>(A, tm)));
    if (first && last)
      FZ_LAUNCH(ST_FZ_LIMIT, (k_fz_limit<true, true, false><<<grid, blk, K2_SMEM, s>>>(A, tm)));
    else if (first)
      FZ_LAUNCH(ST_FZ_LIMIT, (k_fz_limit<true, false, true><<<grid, blk, K2_SMEM, s>>>(A, tm)));
    else if (!last)
      FZ_LAUNCH(ST_FZ_LIMIT, (k_fz_limit<false, false, true><<<grid, blk, K2_SMEM, s>>>(A, tm)));
    else
      FZ_LAUNCH(ST_FZ_LIMIT, (k_fz_limit<false, true, true><<<grid, blk, K2_SMEM, s>>>(A, tm)));
    if (iord > 2) {
      *mx_field = A.fmx_out;
      *mn_field = A.fmn_out;
    }
    // the next pass reads this pass's output field and extrema
    A.fin = A.fout;
    A.fout = A.fout == FZ_X1 ? FZ_X0 : FZ_X1;
    A.fmx_in = A.fmx_out;
    A.fmn_in = A.fmn_out;
    A.fmx_out = A.fmx_out == FZ_MX0 ? FZ_MX1 : FZ_MX0;
    A.fmn_out = A.fmn_out == FZ_MN0 ? FZ_MN1 : FZ_MN0;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

}  // namespace mpdata
