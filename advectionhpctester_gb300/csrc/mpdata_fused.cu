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

// Tile heights (build-time, for tuning sweeps).  A tile of 32 x TY cells is
// one block of 32*TY threads, one output cell each; 1024 threads stay
// resident per SM (four blocks of 8 rows, two of 16).  The upwind+pseudo
// kernel, bound by shared-memory traffic, measured 13% faster with 16 rows
// (its one-cell ring of recomputed upwind cells is a smaller share); the
// other two measured 4-15% faster with 8 rows.
#ifndef MPDATA_FZ_TY_UP
#define MPDATA_FZ_TY_UP 16
#endif
#ifndef MPDATA_FZ_TY
#define MPDATA_FZ_TY 8
#endif
constexpr int TX = 32;
constexpr int HX = 4, HY = 2;   // staged halo columns and rows
constexpr int P = TX + 2 * HX;  // plane pitch: 40
template <int TY>
struct Tl {
  static constexpr int NT = TX * TY;                     // threads = output cells per plane
  static constexpr int MINB = 1024 / NT;                 // resident blocks per SM asked of ptxas
  static constexpr int NR = TY + 2 * HY;                 // staged rows
  static constexpr int PLANE = P * NR;                   // staged cells per plane
  static constexpr uint32_t BOX_BYTES = PLANE * 4;
  static constexpr int NRING1 = 2 * (TX + 2) + 2 * TY;  // the tile's one-cell ring
  static constexpr int NRINGW = TX + TY;                // faces beyond the tile's last row / column
};
constexpr int TY_UP = MPDATA_FZ_TY_UP, TY2 = MPDATA_FZ_TY;

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
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity), "r"(1000000u)
      : "memory");
  return ok != 0;
}
// Bounded wait on an mbarrier phase: false when the limit ran out.  Each
// try_wait suspends the thread until the phase completes or about 1 ms has
// passed, so a waiting warp issues almost nothing and the limit is seconds.
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t parity) {
  for (int it = 0; it < 4096; it++)
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

typedef FusedArgs FzArgs;

// The fields of one pass: which arena fields hold its input field, its
// output field and the running extrema it reads and writes (the same for
// every problem of a batch).
struct FzPass {
  int fin, fout, fmx_in, fmn_in, fmx_out, fmn_out;
  __device__ __forceinline__ void apply(FzArgs& a) const {
    a.fin = fin;
    a.fout = fout;
    a.fmx_in = fmx_in;
    a.fmn_in = fmn_in;
    a.fmx_out = fmx_out;
    a.fmn_out = fmn_out;
  }
};

// The two staged cells of thread t: box cells t and t+NT (the second exists
// for t < PLANE-NT), as wrapped 1-based grid coordinates.
struct Box {
  int i0, j0, i1, j1;
  bool two;
};
template <int TY>
__device__ __forceinline__ Box box_cells(const Geo& g, int x0, int y0, int t) {
  constexpr int NT = Tl<TY>::NT, PLANE = Tl<TY>::PLANE;
  Box b;
  b.i0 = wrapn(x0 - HX + t % P, g.np);
  b.j0 = wrapn(y0 - HY + t / P, g.mp);
  const int e = t + NT;
  b.two = e < PLANE;
  b.i1 = wrapn(x0 - HX + e % P, g.np);
  b.j1 = wrapn(y0 - HY + e / P, g.mp);
  return b;
}
// In-plane offsets of the thread's two box cells in a layout with row
// stride sy (every plane of every array used here is below 2^31 elements).
struct Offs {
  int o0, o1;
};
__device__ __forceinline__ Offs box_offs(const Box& b, int sy) {
  return Offs{(b.i0 - 1) + (b.j0 - 1) * sy, (b.i1 - 1) + (b.j1 - 1) * sy};
}
// the thread's two box cells of one plane (base = the plane's cell (1,1))
template <int NT>
__device__ __forceinline__ void stage2(float* dst, const float* base, const Offs& o, bool two, int t) {
  cp_async4(dst + t, base + o.o0);
  if (two) cp_async4(dst + t + NT, base + o.o1);
}
__device__ __forceinline__ const float* caller_plane(const Arr<float>& A, int kw) {
  return A.p + (long)(kw - 1) * A.sz;
}
// the wrapped plane after kw
__device__ __forceinline__ int next_plane(int kw, int lp) { return kw == lp ? 1 : kw + 1; }
__device__ __forceinline__ int mod3(int a) { return a >= 3 ? a - 3 : a; }  // a in [0, 5]
__device__ __forceinline__ bool is1(float v) { return __float_as_int(v) == 0x3f800000; }

// smem index of ring cell q of the tile's one-cell ring
template <int TY>
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
template <int TY>
__device__ __forceinline__ int ringw_index(int q) {
  return q < TX ? (HY + TY) * P + HX + q : (HY + (q - TX)) * P + HX + TX;
}

// ---- the stage arithmetic on staged planes (FP32 bodies, interior path) ----
// U: every density the stage reads is exactly 1 (block-uniform), so the
// products and quotients by it are dropped; x*1 == x/1 == x and
// 2/(1+1) == 1 hold exactly in IEEE arithmetic, so no bit changes.

// upwind3d_gpubc at smem cell b of plane k: x0/xm/xp = psi at k, k-1, k+1;
// a3p = u3 at k+1 (the cell's upper face).
template <bool U>
__device__ __forceinline__ float upwind_cell(int b, const float* x0, const float* xm, const float* xp,
                                             const float* a1, const float* a2, const float* a3, const float* a3p,
                                             const float* h, const float* rh) {
  const float x = x0[b];
  const float f1p = donor(x, x0[b + 1], a1[b + 1]);
  const float f1 = donor(x0[b - 1], x, a1[b]);
  const float f2p = donor(x, x0[b + P], a2[b + P]);
  const float f2 = donor(x0[b - P], x, a2[b]);
  const float f3p = donor(x, xp[b], a3p[b]);
  const float f3 = donor(xm[b], x, a3[b]);
  const float sum = f1p - f1 + f2p - f2 + f3p - f3;
  if (U) return x - sum;
  const float hi = 1.0f / h[b];
  return (x - sum * hi) * rh[b];
}

// Gauge pseudo-velocities of the cell's three lower faces at plane k:
// X at k-1, k, k+1; A1, A2 (x and y velocities) at k-1, k; A3 at k, k+1;
// h at k-1, k.  pseudo_form<float, false, ...> with IN.
template <bool U>
__device__ __forceinline__ void pseudo_cell(int b, const float* xm, const float* x0, const float* xp,
                                            const float* a1m, const float* a10, const float* a2m,
                                            const float* a20, const float* a30, const float* a3p,
                                            const float* hm, const float* h0, float& v1, float& v2, float& v3) {
  const float xc = x0[b];
  {  // x face
    const float hmx = U ? 1.0f : 2.0f / (h0[b - 1] + h0[b]);
    const float a = a10[b];
    const float d2 = (x0[b + P] + x0[b - 1 + P]) - (x0[b - P] + x0[b - 1 - P]);
    const float s2 = (a20[b - 1] + a20[b - 1 + P]) + (a20[b] + a20[b + P]);
    const float d3 = (xp[b] + xp[b - 1]) - (xm[b] + xm[b - 1]);
    const float s3 = (a30[b - 1] + a3p[b - 1]) + (a30[b] + a3p[b]);
    const float cr = s2 * d2 + s3 * d3;
    v1 = (fabsf(a) - hmul<U>(a * a, hmx)) * (xc - x0[b - 1]) * 0.5f - hmul<U>(0.03125f * a, hmx) * cr;
  }
  {  // y face
    const float hmy = U ? 1.0f : 2.0f / (h0[b - P] + h0[b]);
    const float a = a20[b];
    const float d1 = (x0[b + 1] + x0[b + 1 - P]) - (x0[b - 1] + x0[b - 1 - P]);
    const float s1 = (a10[b - P] + a10[b + 1 - P]) + (a10[b] + a10[b + 1]);
    const float d3 = (xp[b] + xp[b - P]) - (xm[b] + xm[b - P]);
    const float s3 = (a30[b - P] + a3p[b - P]) + (a30[b] + a3p[b]);
    const float cr = s1 * d1 + s3 * d3;
    v2 = (fabsf(a) - hmul<U>(a * a, hmy)) * (xc - x0[b - P]) * 0.5f - hmul<U>(0.03125f * a, hmy) * cr;
  }
  {  // z face
    const float hmz = U ? 1.0f : 2.0f / (hm[b] + h0[b]);
    const float a = a30[b];
    const float d1 = (x0[b + 1] + xm[b + 1]) - (x0[b - 1] + xm[b - 1]);
    const float d2 = (x0[b + P] + xm[b + P]) - (x0[b - P] + xm[b - P]);
    const float s1 = (a1m[b] + a1m[b + 1]) + (a10[b] + a10[b + 1]);
    const float s2 = (a2m[b] + a2m[b + P]) + (a20[b] + a20[b + P]);
    const float cr = s1 * d1 + s2 * d2;
    v3 = (fabsf(a) - hmul<U>(a * a, hmz)) * (xc - xm[b]) * 0.5f - hmul<U>(0.03125f * a, hmz) * cr;
  }
}

// NaN-propagating max and min (one instruction each).
__device__ __forceinline__ float maxn(float a, float b) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float minn(float a, float b) {
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// Star extrema of the limiter bounds.  The reference folds them with
// compare-and-select in a fixed tree (ties between +0 and -0 keep the earlier
// operand; a NaN propagates from some positions and not from others).  The
// fast path takes max/min instructions, which give the same bits whenever no
// operand is a NaN and the result is not a zero: the largest value is then
// unique.  Otherwise the select tree runs in the reference's order.
template <bool FIRST>
__device__ __forceinline__ void star_extrema(int b, const float* xm, const float* x0, const float* xp,
                                             const float* s0, const float* sm, const float* sp, float& ma,
                                             float& mi) {
  const float x = x0[b];
  const float b0 = x0[b - 1], b2 = x0[b + 1], b3 = x0[b - P], b4 = x0[b + P], b5 = xm[b], b6 = xp[b];
  float m0, n0;  // extrema folded before the current field's star
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, a4 = 0.f, a5 = 0.f, a6 = 0.f;
  if (FIRST) {
    a0 = s0[b - 1];
    a1 = s0[b];
    a2 = s0[b + 1];
    a3 = s0[b - P];
    a4 = s0[b + P];
    a5 = sm[b];
    a6 = sp[b];
    m0 = maxn(maxn(maxn(maxn(maxn(maxn(a0, a1), a2), a3), a4), a5), a6);
    n0 = minn(minn(minn(minn(minn(minn(a0, a1), a2), a3), a4), a5), a6);
  } else {
    m0 = s0[b];
    n0 = sm[b];
  }
  ma = maxn(maxn(maxn(maxn(maxn(maxn(maxn(m0, b0), x), b2), b3), b4), b5), b6);
  mi = minn(minn(minn(minn(minn(minn(minn(n0, b0), x), b2), b3), b4), b5), b6);
  if (ma == 0.0f || mi == 0.0f || ma != ma || mi != mi) {
    if (FIRST) {
      m0 = mx2(mx2(mx2(mx2(mx2(a0, a1), mx2(a2, a3)), a4), a5), a6);
      n0 = mn2(mn2(mn2(mn2(mn2(a0, a1), mn2(a2, a3)), a4), a5), a6);
    } else {
      m0 = s0[b];
      n0 = sm[b];
    }
    ma = mx2(mx2(mx2(mx2(mx2(m0, b0), mx2(x, b2)), mx2(b3, b4)), b5), b6);
    mi = mn2(mn2(mn2(mn2(mn2(n0, b0), mn2(x, b2)), mn2(b3, b4)), b5), b6);
  }
}

// Limiter bounds and ratios of cell b at plane k (bounds_body, FP32, IN):
// FIRST folds the star of x_in (s0/sm/sp) before the field's own star;
// later passes start from the running extrema (s0 = mx, sm = mn at k).
template <bool FIRST, bool U>
__device__ __forceinline__ void bounds_cell(int b, const float* xm, const float* x0, const float* xp,
                                            const float* s0, const float* sm, const float* sp, const float* v1,
                                            const float* v2, const float* v3, const float* v3p, const float* h,
                                            float& cp, float& cn, float& ma, float& mi) {
  star_extrema<FIRST>(b, xm, x0, xp, s0, sm, sp, ma, mi);
  const float x = x0[b];
  const float e1 = v1[b + 1], w1 = v1[b], e2 = v2[b + P], w2 = v2[b], e3 = v3p[b], w3 = v3[b];
  const float ep = Eps<float>::v;
  const float np_ = U ? ma - x : (ma - x) * h[b], nn = U ? x - mi : (x - mi) * h[b];
  const float dp = pn(e1) + pp(w1) + pn(e2) + pp(w2) + pn(e3) + pp(w3) + ep;
  const float dn = pp(e1) + pn(w1) + pp(e2) + pn(w2) + pp(e3) + pn(w3) + ep;
  cp = lim_ratio(np_, dp);
  cn = lim_ratio(nn, dn);
}

// ---- K1: upwind + first-pass pseudo-velocities ----------------------------
// smem planes: psi 4, u1 4, u2 4, u3 4, h 4, rhr 2, xant 4
constexpr int K1_PLANES = 26;

// Each kernel is a device body over one work item (tile bxi, byi of the
// problem's grid, z chunk bzi) and two entry points: a grid over one
// problem's tiles and chunks (arguments as kernel parameters), and a grid
// over a batch's work list (one packed item per block: problem in bits 0-15,
// bxi 16-31, byi 32-47, bzi 48-63), whose block stages its problem's
// arguments in shared memory.
template <int TY>
__device__ __forceinline__ void body_upwind_pseudo(const FzArgs& A, int bxi, int byi, int bzi) {
  constexpr int NT = Tl<TY>::NT, PLANE = Tl<TY>::PLANE, NRING1 = Tl<TY>::NRING1;
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
  const int x0 = bxi * TX + 1, y0 = byi * TY + 1;
  const int kb = bzi * A.kchunk + 1;
  if (kb > g.lp) return;
  const int ke = min(g.lp, kb + A.kchunk - 1);
  const Box bx = box_cells<TY>(g, x0, y0, t);
  const bool two = bx.two;
  const Offs os = box_offs(bx, A.psi.sy), o1 = box_offs(bx, A.u1.sy), o2 = box_offs(bx, A.u2.sy);
  const int b = (ty + HY) * P + tx + HX;
  const int br = t < NRING1 ? ring1_index<TY>(t) : -1;
  const int ig = x0 + tx, jg = y0 + ty;
  const bool own = ig <= g.np && jg <= g.mp;
  const long pl = (long)A.px * g.mp;
  const long go = (long)(ig - 1) + (long)(jg - 1) * A.px;
  float* const fxin = A.arena + FZ_XIN * A.fs + go;
  float* const fxa = A.arena + FZ_X0 * A.fs + go;
  float* const fv1 = A.arena + FZ_V1 * A.fs + go;
  float* const fv2 = A.arena + FZ_V2 * A.fs + go;
  float* const fv3 = A.arena + FZ_V3 * A.fs + go;
#define S4(k) (((k) + 12) & 3)
#define S2(k) ((k) & 1)
  // what the first step (ko = kb-2) reads and does not stage itself
  {
    int kw = wrapn(kb - 2, g.lp);
    for (int k = kb - 2; k <= kb; k++, kw = next_plane(kw, g.lp)) {
      stage2<NT>(PSI + S4(k) * PLANE, caller_plane(A.psi, kw), os, two, t);
      if (k >= kb - 1) stage2<NT>(U3 + S4(k) * PLANE, caller_plane(A.u3, kw), os, two, t);
      if (k == kb - 1) {
        stage2<NT>(U1 + S4(k) * PLANE, caller_plane(A.u1, kw), o1, two, t);
        stage2<NT>(U2 + S4(k) * PLANE, caller_plane(A.u2, kw), o2, two, t);
        stage2<NT>(H + S4(k) * PLANE, caller_plane(A.h, kw), os, two, t);
        stage2<NT>(RH + S2(k) * PLANE, caller_plane(A.rhr, kw), os, two, t);
      }
    }
  }
  cp_commit();
  int kw3 = wrapn(kb + 1, g.lp), kw2 = wrapn(kb, g.lp);  // wrapped planes ko+3 and ko+2
  unsigned umask = 0;  // bit d: h and rhr of plane ko+1-d are exactly 1 on the whole box
  for (int ko = kb - 2; ko <= ke; ko++) {
    cp_wait_all();
    bool one = is1(H[S4(ko + 1) * PLANE + t]) && is1(RH[S2(ko + 1) * PLANE + t]);
    if (two) one = one && is1(H[S4(ko + 1) * PLANE + t + NT]) && is1(RH[S2(ko + 1) * PLANE + t + NT]);
    umask = (umask << 1) | (__syncthreads_and(one) ? 1u : 0u);
    const bool unit = umask & 1u;                 // the upwind at ko+1: h and rhr at ko+1
    const bool unit_ps = (umask & 6u) == 6u;      // the pseudo-velocities at ko: h at ko-1 and ko
    if (ko < ke) {
      stage2<NT>(PSI + S4(ko + 3) * PLANE, caller_plane(A.psi, kw3), os, two, t);
      stage2<NT>(U3 + S4(ko + 3) * PLANE, caller_plane(A.u3, kw3), os, two, t);
      stage2<NT>(U1 + S4(ko + 2) * PLANE, caller_plane(A.u1, kw2), o1, two, t);
      stage2<NT>(U2 + S4(ko + 2) * PLANE, caller_plane(A.u2, kw2), o2, two, t);
      stage2<NT>(H + S4(ko + 2) * PLANE, caller_plane(A.h, kw2), os, two, t);
      stage2<NT>(RH + S2(ko + 2) * PLANE, caller_plane(A.rhr, kw2), os, two, t);
      cp_commit();
      kw3 = next_plane(kw3, g.lp);
      kw2 = next_plane(kw2, g.lp);
    }
    {  // xant at plane ko+1 on the tile and its ring
      const int k = ko + 1;
      const float* p0 = PSI + S4(k) * PLANE;
      const float* pm = PSI + S4(k - 1) * PLANE;
      const float* pp_ = PSI + S4(k + 1) * PLANE;
      const float* a1 = U1 + S4(k) * PLANE;
      const float* a2 = U2 + S4(k) * PLANE;
      const float* a3 = U3 + S4(k) * PLANE;
      const float* a3p = U3 + S4(k + 1) * PLANE;
      const float* h = H + S4(k) * PLANE;
      const float* rh = RH + S2(k) * PLANE;
      float* xa = XA + S4(k) * PLANE;
      float v;
      if (unit) {
        v = upwind_cell<true>(b, p0, pm, pp_, a1, a2, a3, a3p, h, rh);
        if (br >= 0) xa[br] = upwind_cell<true>(br, p0, pm, pp_, a1, a2, a3, a3p, h, rh);
      } else {
        v = upwind_cell<false>(b, p0, pm, pp_, a1, a2, a3, a3p, h, rh);
        if (br >= 0) xa[br] = upwind_cell<false>(br, p0, pm, pp_, a1, a2, a3, a3p, h, rh);
      }
      xa[b] = v;
      if (own && k >= kb && k <= ke) {
        fxa[(k - 1) * pl] = v;
        fxin[(k - 1) * pl] = p0[b];
      }
    }
    __syncthreads();
    if (ko >= kb) {
      float v1, v2, v3;
      const float *xm = XA + S4(ko - 1) * PLANE, *xc = XA + S4(ko) * PLANE, *xp = XA + S4(ko + 1) * PLANE;
      const float *a1m = U1 + S4(ko - 1) * PLANE, *a10 = U1 + S4(ko) * PLANE;
      const float *a2m = U2 + S4(ko - 1) * PLANE, *a20 = U2 + S4(ko) * PLANE;
      const float *a30 = U3 + S4(ko) * PLANE, *a3p = U3 + S4(ko + 1) * PLANE;
      const float *hm = H + S4(ko - 1) * PLANE, *h0 = H + S4(ko) * PLANE;
      if (unit_ps)
        pseudo_cell<true>(b, xm, xc, xp, a1m, a10, a2m, a20, a30, a3p, hm, h0, v1, v2, v3);
      else
        pseudo_cell<false>(b, xm, xc, xp, a1m, a10, a2m, a20, a30, a3p, hm, h0, v1, v2, v3);
      if (own) {
        const long o = (ko - 1) * pl;
        fv1[o] = v1;
        fv2[o] = v2;
        fv3[o] = v3;
      }
    }
  }
}

template <int TY>
__global__ void __launch_bounds__(Tl<TY>::NT, Tl<TY>::MINB) k_fz_upwind_pseudo(const FzArgs A) {
  body_upwind_pseudo<TY>(A, blockIdx.x, blockIdx.y, blockIdx.z);
}

// One work item of a batch.
struct Item {
  int p, bxi, byi, bzi;
};
__device__ __forceinline__ Item item_of(const unsigned long long* items) {
  const unsigned long long w = items[blockIdx.x];
  return Item{(int)(w & 0xffffu), (int)((w >> 16) & 0xffffu), (int)((w >> 32) & 0xffffu), (int)(w >> 48)};
}

template <int TY>
__global__ void __launch_bounds__(Tl<TY>::NT, Tl<TY>::MINB)
    kb_fz_upwind_pseudo(const FzArgs* __restrict__ probs, const unsigned long long* __restrict__ items) {
  __shared__ FzArgs sa;
  const Item it = item_of(items);
  if (threadIdx.x == 0) sa = probs[it.p];
  __syncthreads();
  body_upwind_pseudo<TY>(sa, it.bxi, it.byi, it.bzi);
}

// ---- staging of arena fields: TMA on interior tiles, wrapped cp.async else ----
template <int NT>
struct Stager {
  const CUtensorMap* map;
  const float* arena;
  long fs;
  long pl;     // elements per arena plane
  int xc, yc;  // box origin (0-based) of the tile
  bool tma, two;
  Offs o;      // the thread's two box cells in the arena layout (seam tiles)
  int t;
  // plane kw (1-based, wrapped) of arena field f into dst
  __device__ __forceinline__ void plane(float* dst, int f, int kw, uint64_t* m) const {
    if (tma) {
      if (t == 0) tma_box(dst, map, xc, yc, kw - 1, f, m);
    } else {
      stage2<NT>(dst, arena + f * fs + (kw - 1) * pl, o, two, t);
    }
  }
  // the two forms separately, for a step that stages several planes under one
  // branch (box: thread 0 of an interior tile; cp: every thread of a seam tile)
  __device__ __forceinline__ void box(float* dst, int f, int kw, uint64_t* m) const {
    tma_box(dst, map, xc, yc, kw - 1, f, m);
  }
  __device__ __forceinline__ void cp(float* dst, int f, int kw) const {
    stage2<NT>(dst, arena + f * fs + (kw - 1) * pl, o, two, t);
  }
};

// Interior tile: every staged box lies inside the grid, so TMA needs no wrap.
template <int TY>
__device__ __forceinline__ bool tile_inside(const Geo& g, int bxi, int byi) {
  return bxi >= 1 && bxi * TX + TX + HX <= g.np && byi >= 1 && byi * TY + TY + HY <= g.mp;
}

// Waits for the TMA phase of the previous iteration (bounded); false when the
// limit ran out, after setting the block's abort flag and the error word.
__device__ __forceinline__ void tma_wait(bool tma, uint64_t* mbar, int n, int* s_abort, int* err) {
  if (tma && n >= 1) {
    if (!mbar_wait(&mbar[(n - 1) & 1], ((n - 1) >> 1) & 1)) {
      *s_abort = 1;
      atomicOr(err, 2);
    }
  }
}

// ---- K2: limiter bounds + limited velocities + update of one pass ----------
// smem planes: x 4, x_in 4 (or mx 2 + mn 2), v1 2, v2 2, v3 3, h 3, cp 2,
// cn 2, w1 2, w2 2; tiles: w3 2, rhr 2
constexpr int K2_PLANES = 26;
constexpr int K2_TILES = 4;

template <int TY, bool FIRST, bool LAST, bool KEEP>
__device__ __forceinline__ void body_limit(const FzArgs& A, const CUtensorMap* tm, int bxi, int byi, int bzi) {
  constexpr int NT = Tl<TY>::NT, PLANE = Tl<TY>::PLANE, NRING1 = Tl<TY>::NRING1, NRINGW = Tl<TY>::NRINGW;
  constexpr uint32_t BOX_BYTES = Tl<TY>::BOX_BYTES;
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
  const int x0 = bxi * TX + 1, y0 = byi * TY + 1;
  const int kb = bzi * A.kchunk + 1;
  if (kb > g.lp) return;
  const int ke = min(g.lp, kb + A.kchunk - 1);
  const bool tma = tile_inside<TY>(g, bxi, byi);
  const Box bx = box_cells<TY>(g, x0, y0, t);
  const bool two = bx.two;
  const long pl = (long)A.px * g.mp;
  const Stager<NT> st{tm, A.arena, A.fs, pl, x0 - 1 - HX, y0 - 1 - HY, tma, two, box_offs(bx, A.px), t};
  const Offs oh = box_offs(bx, A.h.sy);
  const int b = (ty + HY) * P + tx + HX;
  const int br = t < NRING1 ? ring1_index<TY>(t) : -1;
  const int bw = t < NRINGW ? ringw_index<TY>(t) : -1;
  const int ig = x0 + tx, jg = y0 + ty;
  const bool own = ig <= g.np && jg <= g.mp;
  const int orh = (wrapn(ig, g.np) - 1) + (wrapn(jg, g.mp) - 1) * A.rhr.sy;
  const long go = (long)(ig - 1) + (long)(jg - 1) * A.px;
  float* const fmx = A.arena + A.fmx_out * A.fs + go;
  float* const fmn = A.arena + A.fmn_out * A.fs + go;
  float* const fw1 = A.arena + FZ_W1 * A.fs + go;
  float* const fw2 = A.arena + FZ_W2 * A.fs + go;
  float* const fw3 = A.arena + FZ_W3 * A.fs + go;
  float* const fout = A.arena + A.fout * A.fs + go;
  if (t == 0) {
    s_abort = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  constexpr int NBOX_PRO = FIRST ? 10 : 9;  // boxes staged before the first step
  constexpr int NBOX = FIRST ? 5 : 6;       // boxes staged by each step
  const int fsx = FIRST ? FZ_XIN : A.fmx_in;
#define S4(k) (((k) + 12) & 3)
#define S2(k) ((k) & 1)
  // staging of the first step's reads
  if (tma && t == 0) mbar_expect_tx(&mbar[0], NBOX_PRO * BOX_BYTES);
  {
    int kw = wrapn(kb - 2, g.lp);
    for (int k = kb - 2; k <= kb; k++, kw = next_plane(kw, g.lp)) {
      st.plane(X + S4(k) * PLANE, A.fin, kw, &mbar[0]);
      if (FIRST) st.plane(S + S4(k) * PLANE, FZ_XIN, kw, &mbar[0]);
      if (k >= kb - 1) st.plane(V3 + mod3(k - kb + 5) * PLANE, FZ_V3, kw, &mbar[0]);
      if (k == kb - 1) {
        st.plane(V1 + S2(k) * PLANE, FZ_V1, kw, &mbar[0]);
        st.plane(V2 + S2(k) * PLANE, FZ_V2, kw, &mbar[0]);
        if (!FIRST) {
          st.plane(S + S2(k) * PLANE, fsx, kw, &mbar[0]);
          st.plane(S + (2 + S2(k)) * PLANE, A.fmn_in, kw, &mbar[0]);
        }
        stage2<NT>(H + mod3(k - kb + 5) * PLANE, caller_plane(A.h, kw), oh, two, t);
      }
    }
  }
  cp_commit();
  // ring slots of the 3-plane rings: r3 = slot of plane ko (planes ko-kb+5 mod 3)
  int r3 = 0;  // plane ko = kb-2 has slot (kb-2-kb+5) mod 3 = 0
  int kw3 = wrapn(kb + 1, g.lp), kw2 = wrapn(kb, g.lp), kw1 = wrapn(kb - 1, g.lp);  // planes ko+3, +2, +1
  for (int ko = kb - 2; ko <= ke; ko++) {
    const int n = ko - kb + 3;
    const int q0 = r3, q1 = mod3(r3 + 1), q2 = mod3(r3 + 2);  // slots of planes ko, ko+1, ko+2 (= ko-1)
    cp_wait_all();
    tma_wait(tma, mbar, n, &s_abort, A.err);
    // densities of this step (h at ko and ko+1, rhr at ko) all exactly 1?
    bool one = is1(H[q0 * PLANE + t]) && is1(H[q1 * PLANE + t]) && is1(RH[S2(ko) * NT + t]);
    if (two) one = one && is1(H[q0 * PLANE + t + NT]) && is1(H[q1 * PLANE + t + NT]);
    const bool unit = __syncthreads_and(one);
    if (s_abort) return;
    if (ko < ke) {
      uint64_t* m = &mbar[n & 1];
      float* const dx = X + S4(ko + 3) * PLANE;
      float* const ds = S + S4(ko + 3) * PLANE;
      float* const d3 = V3 + q0 * PLANE;  // plane ko+3 takes the slot of ko
      float* const d1 = V1 + S2(ko + 2) * PLANE;
      float* const d2 = V2 + S2(ko + 2) * PLANE;
      float* const dmx = S + S2(ko + 2) * PLANE;
      float* const dmn = S + (2 + S2(ko + 2)) * PLANE;
      if (tma) {
        if (t == 0) {
          mbar_expect_tx(m, NBOX * BOX_BYTES);
          st.box(dx, A.fin, kw3, m);
          if (FIRST) st.box(ds, FZ_XIN, kw3, m);
          st.box(d3, FZ_V3, kw3, m);
          st.box(d1, FZ_V1, kw2, m);
          st.box(d2, FZ_V2, kw2, m);
          if (!FIRST) {
            st.box(dmx, fsx, kw2, m);
            st.box(dmn, A.fmn_in, kw2, m);
          }
        }
      } else {
        st.cp(dx, A.fin, kw3);
        if (FIRST) st.cp(ds, FZ_XIN, kw3);
        st.cp(d3, FZ_V3, kw3);
        st.cp(d1, FZ_V1, kw2);
        st.cp(d2, FZ_V2, kw2);
        if (!FIRST) {
          st.cp(dmx, fsx, kw2);
          st.cp(dmn, A.fmn_in, kw2);
        }
      }
      stage2<NT>(H + q2 * PLANE, caller_plane(A.h, kw2), oh, two, t);  // plane ko+2 takes the slot of ko-1
      cp_async4(RH + S2(ko + 1) * NT + t, caller_plane(A.rhr, kw1) + orh);
      cp_commit();
      kw3 = next_plane(kw3, g.lp);
      kw2 = next_plane(kw2, g.lp);
      kw1 = next_plane(kw1, g.lp);
    }
    // limiter bounds and ratios at plane ko+1, on the tile and its ring
    const int kc = ko + 1;
    {
      const float* xm = X + S4(kc - 1) * PLANE;
      const float* xc = X + S4(kc) * PLANE;
      const float* xp = X + S4(kc + 1) * PLANE;
      const float *s0, *s1, *s2;
      if (FIRST) {
        s0 = S + S4(kc) * PLANE;
        s1 = S + S4(kc - 1) * PLANE;
        s2 = S + S4(kc + 1) * PLANE;
      } else {
        s0 = S + S2(kc) * PLANE;        // mx
        s1 = S + (2 + S2(kc)) * PLANE;  // mn
        s2 = nullptr;
      }
      const float* v1 = V1 + S2(kc) * PLANE;
      const float* v2 = V2 + S2(kc) * PLANE;
      const float* v3 = V3 + q1 * PLANE;
      const float* v3p = V3 + q2 * PLANE;
      const float* h = H + q1 * PLANE;
      float* cp = CP + S2(kc) * PLANE;
      float* cn = CN + S2(kc) * PLANE;
      float rp, rn, ma, mi;
      if (unit)
        bounds_cell<FIRST, true>(b, xm, xc, xp, s0, s1, s2, v1, v2, v3, v3p, h, rp, rn, ma, mi);
      else
        bounds_cell<FIRST, false>(b, xm, xc, xp, s0, s1, s2, v1, v2, v3, v3p, h, rp, rn, ma, mi);
      cp[b] = rp;
      cn[b] = rn;
      if (KEEP && own && kc >= kb && kc <= ke) {
        fmx[(kc - 1) * pl] = ma;
        fmn[(kc - 1) * pl] = mi;
      }
      if (br >= 0) {
        if (unit)
          bounds_cell<FIRST, true>(br, xm, xc, xp, s0, s1, s2, v1, v2, v3, v3p, h, rp, rn, ma, mi);
        else
          bounds_cell<FIRST, false>(br, xm, xc, xp, s0, s1, s2, v1, v2, v3, v3p, h, rp, rn, ma, mi);
        cp[br] = rp;
        cn[br] = rn;
      }
    }
    __syncthreads();
    // limited velocities at plane ko+1 (limit_form, gauge, nonos)
    if (kc >= kb) {
      const float* cp = CP + S2(kc) * PLANE;
      const float* cn = CN + S2(kc) * PLANE;
      const float* cpm = CP + S2(kc - 1) * PLANE;
      const float* cnm = CN + S2(kc - 1) * PLANE;
      const float* v1 = V1 + S2(kc) * PLANE;
      const float* v2 = V2 + S2(kc) * PLANE;
      const float* v3 = V3 + q1 * PLANE;
      float* w1 = W1 + S2(kc) * PLANE;
      float* w2 = W2 + S2(kc) * PLANE;
      const float cpc = cp[b], cnc = cn[b];
      const float r1 = donor(min3(cpc, cn[b - 1]), min3(cp[b - 1], cnc), v1[b]);
      const float r2 = donor(min3(cpc, cn[b - P]), min3(cp[b - P], cnc), v2[b]);
      const float r3v = donor(min3(cpc, cnm[b]), min3(cpm[b], cnc), v3[b]);
      w1[b] = r1;
      w2[b] = r2;
      W3[S2(kc) * NT + t] = r3v;
      if (!LAST && own && kc <= ke) {
        const long o = (kc - 1) * pl;
        fw1[o] = r1;
        fw2[o] = r2;
        fw3[o] = r3v;
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
      const float* w1 = W1 + S2(ko) * PLANE;
      const float* w2 = W2 + S2(ko) * PLANE;
      const float* w3 = W3 + S2(ko) * NT;
      const float* w3p = W3 + S2(ko + 1) * NT;
      const float xc = X[S4(ko) * PLANE + b];
      const float d = w1[b + 1] - w1[b] + w2[b + P] - w2[b] + w3p[t] - w3[t];
      float out;
      if (unit) {
        out = xc - d;
      } else {
        const float rh = RH[S2(ko) * NT + t];
        const float q = xc / rh;
        out = (q - d / H[q0 * PLANE + b]) * rh;
      }
      if (own) {
        if (LAST)
          A.psi.at(ig, jg, ko) = out;
        else
          fout[(ko - 1) * pl] = out;
      }
    }
    r3 = q1;
  }
}

// ---- K3: pseudo-velocities of a later pass ---------------------------------
// smem planes: x 4, w1 4, w2 4, w3 4, h 4
constexpr int K3_PLANES = 20;

template <int TY>
__device__ __forceinline__ void body_pseudo(const FzArgs& A, const CUtensorMap* tm, int bxi, int byi, int bzi) {
  constexpr int NT = Tl<TY>::NT, PLANE = Tl<TY>::PLANE;
  constexpr uint32_t BOX_BYTES = Tl<TY>::BOX_BYTES;
  float* const sm = smem_base();
  float* const X = sm;
  float* const A1 = X + 4 * PLANE;
  float* const A2 = A1 + 4 * PLANE;
  float* const A3 = A2 + 4 * PLANE;
  float* const H = A3 + 4 * PLANE;
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ int s_abort;
  const Geo& g = A.g;
  const int t = threadIdx.x, tx = t % TX, ty = t / TX;
  const int x0 = bxi * TX + 1, y0 = byi * TY + 1;
  const int kb = bzi * A.kchunk + 1;
  if (kb > g.lp) return;
  const int ke = min(g.lp, kb + A.kchunk - 1);
  const bool tma = tile_inside<TY>(g, bxi, byi);
  const Box bx = box_cells<TY>(g, x0, y0, t);
  const bool two = bx.two;
  const long pl = (long)A.px * g.mp;
  const Stager<NT> st{tm, A.arena, A.fs, pl, x0 - 1 - HX, y0 - 1 - HY, tma, two, box_offs(bx, A.px), t};
  const Offs oh = box_offs(bx, A.h.sy);
  const int b = (ty + HY) * P + tx + HX;
  const int ig = x0 + tx, jg = y0 + ty;
  const bool own = ig <= g.np && jg <= g.mp;
  const long go = (long)(ig - 1) + (long)(jg - 1) * A.px;
  float* const fv1 = A.arena + FZ_V1 * A.fs + go;
  float* const fv2 = A.arena + FZ_V2 * A.fs + go;
  float* const fv3 = A.arena + FZ_V3 * A.fs + go;
  if (t == 0) {
    s_abort = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tma && t == 0) mbar_expect_tx(&mbar[0], 9 * BOX_BYTES);
  {
    int kw = wrapn(kb - 1, g.lp);
    for (int k = kb - 1; k <= kb + 1; k++, kw = next_plane(kw, g.lp)) {
      st.plane(X + S4(k) * PLANE, A.fin, kw, &mbar[0]);
      if (k >= kb) st.plane(A3 + S4(k) * PLANE, FZ_W3, kw, &mbar[0]);
      if (k <= kb) {
        st.plane(A1 + S4(k) * PLANE, FZ_W1, kw, &mbar[0]);
        st.plane(A2 + S4(k) * PLANE, FZ_W2, kw, &mbar[0]);
        stage2<NT>(H + S4(k) * PLANE, caller_plane(A.h, kw), oh, two, t);
      }
    }
  }
  cp_commit();
  int kw2 = wrapn(kb + 2, g.lp), kw1 = wrapn(kb + 1, g.lp);  // planes ko+2, ko+1
  for (int ko = kb; ko <= ke; ko++) {
    const int n = ko - kb + 1;
    cp_wait_all();
    tma_wait(tma, mbar, n, &s_abort, A.err);
    bool one = is1(H[S4(ko - 1) * PLANE + t]) && is1(H[S4(ko) * PLANE + t]);
    if (two) one = one && is1(H[S4(ko - 1) * PLANE + t + NT]) && is1(H[S4(ko) * PLANE + t + NT]);
    const bool unit = __syncthreads_and(one);
    if (s_abort) return;
    if (ko < ke) {
      uint64_t* m = &mbar[n & 1];
      float* const dx = X + S4(ko + 2) * PLANE;
      float* const d3 = A3 + S4(ko + 2) * PLANE;
      float* const d1 = A1 + S4(ko + 1) * PLANE;
      float* const d2 = A2 + S4(ko + 1) * PLANE;
      if (tma) {
        if (t == 0) {
          mbar_expect_tx(m, 4 * BOX_BYTES);
          st.box(dx, A.fin, kw2, m);
          st.box(d3, FZ_W3, kw2, m);
          st.box(d1, FZ_W1, kw1, m);
          st.box(d2, FZ_W2, kw1, m);
        }
      } else {
        st.cp(dx, A.fin, kw2);
        st.cp(d3, FZ_W3, kw2);
        st.cp(d1, FZ_W1, kw1);
        st.cp(d2, FZ_W2, kw1);
      }
      stage2<NT>(H + S4(ko + 1) * PLANE, caller_plane(A.h, kw1), oh, two, t);
      cp_commit();
      kw2 = next_plane(kw2, g.lp);
      kw1 = next_plane(kw1, g.lp);
    }
    float v1, v2, v3;
    const float *xm = X + S4(ko - 1) * PLANE, *xc = X + S4(ko) * PLANE, *xp = X + S4(ko + 1) * PLANE;
    const float *a1m = A1 + S4(ko - 1) * PLANE, *a10 = A1 + S4(ko) * PLANE;
    const float *a2m = A2 + S4(ko - 1) * PLANE, *a20 = A2 + S4(ko) * PLANE;
    const float *a30 = A3 + S4(ko) * PLANE, *a3p = A3 + S4(ko + 1) * PLANE;
    const float *hm = H + S4(ko - 1) * PLANE, *h0 = H + S4(ko) * PLANE;
    if (unit)
      pseudo_cell<true>(b, xm, xc, xp, a1m, a10, a2m, a20, a30, a3p, hm, h0, v1, v2, v3);
    else
      pseudo_cell<false>(b, xm, xc, xp, a1m, a10, a2m, a20, a30, a3p, hm, h0, v1, v2, v3);
    if (own) {
      const long o = (ko - 1) * pl;
      fv1[o] = v1;
      fv2[o] = v2;
      fv3[o] = v3;
    }
  }
#undef S4
#undef S2
}

template <int TY, bool FIRST, bool LAST, bool KEEP>
__global__ void __launch_bounds__(Tl<TY>::NT, Tl<TY>::MINB)
    k_fz_limit(const FzArgs A, const __grid_constant__ CUtensorMap tm) {
  body_limit<TY, FIRST, LAST, KEEP>(A, &tm, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <int TY, bool FIRST, bool LAST, bool KEEP>
__global__ void __launch_bounds__(Tl<TY>::NT, Tl<TY>::MINB)
    kb_fz_limit(const FzArgs* __restrict__ probs, const CUtensorMap* __restrict__ maps,
                const unsigned long long* __restrict__ items, FzPass pass) {
  __shared__ FzArgs sa;
  const Item it = item_of(items);
  if (threadIdx.x == 0) {
    sa = probs[it.p];
    pass.apply(sa);
  }
  __syncthreads();
  body_limit<TY, FIRST, LAST, KEEP>(sa, maps + it.p, it.bxi, it.byi, it.bzi);
}
template <int TY>
__global__ void __launch_bounds__(Tl<TY>::NT, Tl<TY>::MINB)
    k_fz_pseudo(const FzArgs A, const __grid_constant__ CUtensorMap tm) {
  body_pseudo<TY>(A, &tm, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <int TY>
__global__ void __launch_bounds__(Tl<TY>::NT, Tl<TY>::MINB)
    kb_fz_pseudo(const FzArgs* __restrict__ probs, const CUtensorMap* __restrict__ maps,
                 const unsigned long long* __restrict__ items, FzPass pass) {
  __shared__ FzArgs sa;
  const Item it = item_of(items);
  if (threadIdx.x == 0) {
    sa = probs[it.p];
    pass.apply(sa);
  }
  __syncthreads();
  body_pseudo<TY>(sa, maps + it.p, it.bxi, it.byi, it.bzi);
}

constexpr size_t K1_SMEM = (size_t)K1_PLANES * Tl<TY_UP>::PLANE * 4 + 128;
constexpr size_t K2_SMEM = (size_t)K2_PLANES * Tl<TY2>::PLANE * 4 + (size_t)K2_TILES * Tl<TY2>::NT * 4 + 128;
constexpr size_t K3_SMEM = (size_t)K3_PLANES * Tl<TY2>::PLANE * 4 + 128;

template <class K>
int set_smem(K kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess ? 0
                                                                                                                : -5;
}

int init_kernels() {
  static int rc = [] {
    int r = 0;
    r |= set_smem(kb_fz_upwind_pseudo<TY_UP>, K1_SMEM);
    r |= set_smem(kb_fz_limit<TY2, true, true, false>, K2_SMEM);
    r |= set_smem(kb_fz_limit<TY2, true, false, true>, K2_SMEM);
    r |= set_smem(kb_fz_limit<TY2, false, false, true>, K2_SMEM);
    r |= set_smem(kb_fz_limit<TY2, false, true, true>, K2_SMEM);
    r |= set_smem(kb_fz_pseudo<TY2>, K3_SMEM);
    r |= set_smem(k_fz_upwind_pseudo<TY_UP>, K1_SMEM);
    r |= set_smem(k_fz_limit<TY2, true, true, false>, K2_SMEM);
    r |= set_smem(k_fz_limit<TY2, true, false, true>, K2_SMEM);
    r |= set_smem(k_fz_limit<TY2, false, false, true>, K2_SMEM);
    r |= set_smem(k_fz_limit<TY2, false, true, true>, K2_SMEM);
    r |= set_smem(k_fz_pseudo<TY2>, K3_SMEM);
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
  const cuuint32_t box[4] = {(cuuint32_t)P, (cuuint32_t)Tl<TY2>::NR, 1, 1};
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
  const long tiles = (long)((g.np + TX - 1) / TX) * ((g.mp + TY2 - 1) / TY2);
  const long want = 152L * Tl<TY2>::MINB * 6;  // about six waves
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

FusedArgs fused_args(const FusedPlan& F) {
  FzArgs A;
  A.g = F.g;
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
  A.fin = FZ_X0;  // the first pass reads the upwind field and writes X1
  A.fout = FZ_X1;
  A.fmx_in = FZ_MX0;
  A.fmn_in = FZ_MN0;
  A.fmx_out = FZ_MX0;
  A.fmn_out = FZ_MN0;
  return A;
}

int fused_init() { return init_kernels(); }

void fused_items(const Geo& g, int kchunk, int p, std::vector<unsigned long long>& up,
                 std::vector<unsigned long long>& rest) {
  const int nz = (g.lp + kchunk - 1) / kchunk;
  const int ntx = (g.np + TX - 1) / TX;
  const int nty1 = (g.mp + TY_UP - 1) / TY_UP, nty2 = (g.mp + TY2 - 1) / TY2;
  for (int z = 0; z < nz; z++) {
    for (int y = 0; y < nty1; y++)
      for (int x = 0; x < ntx; x++)
        up.push_back((unsigned long long)p | ((unsigned long long)x << 16) | ((unsigned long long)y << 32) |
                     ((unsigned long long)z << 48));
    for (int y = 0; y < nty2; y++)
      for (int x = 0; x < ntx; x++)
        rest.push_back((unsigned long long)p | ((unsigned long long)x << 16) | ((unsigned long long)y << 32) |
                       ((unsigned long long)z << 48));
  }
}

// the arena fields of the next pass: it reads this pass's output field and extrema
static void next_pass(int& fin, int& fout, int& mxi, int& mni, int& mxo, int& mno) {
  fin = fout;
  fout = fout == FZ_X1 ? FZ_X0 : FZ_X1;
  mxi = mxo;
  mni = mno;
  mxo = mxo == FZ_MX0 ? FZ_MX1 : FZ_MX0;
  mno = mno == FZ_MN0 ? FZ_MN1 : FZ_MN0;
}

int run_batch_fused(const FusedArgs* probs, const CUtensorMap* maps, const unsigned long long* items_up, int n_up,
                    const unsigned long long* items, int n, int iord, Prof* prof, cudaStream_t s) {
  if (init_kernels()) return -5;
  if (n_up < 1 || n < 1) return 0;
  const dim3 blk1(Tl<TY_UP>::NT), blk(Tl<TY2>::NT);
  FZ_LAUNCH(ST_FZ_UPWIND_PSEUDO, (kb_fz_upwind_pseudo<TY_UP><<<n_up, blk1, K1_SMEM, s>>>(probs, items_up)));
  FzPass ps{FZ_X0, FZ_X1, FZ_MX0, FZ_MN0, FZ_MX0, FZ_MN0};
  for (int pass = 2; pass <= iord; pass++) {
    const bool first = pass == 2, last = pass == iord;
    if (!first) FZ_LAUNCH(ST_FZ_PSEUDO, (kb_fz_pseudo<TY2><<<n, blk, K3_SMEM, s>>>(probs, maps, items, ps)));
    if (first && last)
      FZ_LAUNCH(ST_FZ_LIMIT, (kb_fz_limit<TY2, true, true, false><<<n, blk, K2_SMEM, s>>>(probs, maps, items, ps)));
    else if (first)
      FZ_LAUNCH(ST_FZ_LIMIT, (kb_fz_limit<TY2, true, false, true><<<n, blk, K2_SMEM, s>>>(probs, maps, items, ps)));
    else if (!last)
      FZ_LAUNCH(ST_FZ_LIMIT, (kb_fz_limit<TY2, false, false, true><<<n, blk, K2_SMEM, s>>>(probs, maps, items, ps)));
    else
      FZ_LAUNCH(ST_FZ_LIMIT, (kb_fz_limit<TY2, false, true, true><<<n, blk, K2_SMEM, s>>>(probs, maps, items, ps)));
    next_pass(ps.fin, ps.fout, ps.fmx_in, ps.fmn_in, ps.fmx_out, ps.fmn_out);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

int run_step_fused(const FusedPlan& F, int iord, Prof* prof, cudaStream_t s, int* mx_field, int* mn_field) {
  if (init_kernels()) return -5;
  const Geo& g = F.g;
  FzArgs A = fused_args(F);
  const int nz = (g.lp + F.kchunk - 1) / F.kchunk;
  const dim3 grid1((g.np + TX - 1) / TX, (g.mp + TY_UP - 1) / TY_UP, nz), blk1(Tl<TY_UP>::NT);
  const dim3 grid((g.np + TX - 1) / TX, (g.mp + TY2 - 1) / TY2, nz), blk(Tl<TY2>::NT);
  const CUtensorMap& tm = *F.tmap;
  FZ_LAUNCH(ST_FZ_UPWIND_PSEUDO, (k_fz_upwind_pseudo<TY_UP><<<grid1, blk1, K1_SMEM, s>>>(A)));
  *mx_field = *mn_field = -1;
  for (int pass = 2; pass <= iord; pass++) {
    const bool first = pass == 2, last = pass == iord;
    if (!first) FZ_LAUNCH(ST_FZ_PSEUDO, (k_fz_pseudo<TY2><<<grid, blk, K3_SMEM, s>>>(A, tm)));
    if (first && last)
      FZ_LAUNCH(ST_FZ_LIMIT, (k_fz_limit<TY2, true, true, false><<<grid, blk, K2_SMEM, s>>>(A, tm)));
    else if (first)
      FZ_LAUNCH(ST_FZ_LIMIT, (k_fz_limit<TY2, true, false, true><<<grid, blk, K2_SMEM, s>>>(A, tm)));
    else if (!last)
      FZ_LAUNCH(ST_FZ_LIMIT, (k_fz_limit<TY2, false, false, true><<<grid, blk, K2_SMEM, s>>>(A, tm)));
    else
      FZ_LAUNCH(ST_FZ_LIMIT, (k_fz_limit<TY2, false, true, true><<<grid, blk, K2_SMEM, s>>>(A, tm)));
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
