// Launch sequences of the MPDATA kernels (host side).
#pragma once
#include "mpdata_body.cuh"

namespace mpdata {

// Stage ids for the optional per-launch CUDA-event timing.
enum Stage { ST_UPWIND = 0, ST_PSEUDO, ST_BOUNDS, ST_LIMIT, ST_UPDATE, ST_COPY, ST_PRED_LEVEL,
             ST_PRED_CGRID, ST_RHO_OUT, ST_PAIRS, ST_FZ_UPWIND_PSEUDO, ST_FZ_PSEUDO, ST_FZ_LIMIT, NSTAGE };

// Records a pair of CUDA events around each launch when enabled (the events
// live on the launching stream, so they time exactly that kernel).
struct Prof {
  virtual void begin(int stage, cudaStream_t s) = 0;
  virtual void end(int stage, cudaStream_t s) = 0;
  virtual ~Prof() {}
};

// One step of one problem: upwind, then iord-1 corrective passes (and the
// outputs of the density step when P.rho is set).
template <class R>
int run_step(const Prob<R>& P, int iord, int nonos, Prof* prof, cudaStream_t stream);

// One step of every problem of a batch.  probs and tiles live in device
// memory: tiles[t] packs the problem (bits 0-15), the x and y tile indices
// (16-31, 32-47) and the plane k-1 (48-63) of tile t, tiles of bx*by cells in
// one plane.  Each stage is one launch of ntiles blocks of bx*by threads.
template <class R>
struct BatchLaunch {
  const Prob<R>* probs;
  const unsigned long long* tiles;
  int ntiles;
  int bx, by;
  int iord, nonos;
  int halo;  // 0 while autotuning: psi (interior and halo) is not written
  int pairs; // some FP64 gauge problem reads pair sums: launch kb_pairs
};
template <class R>
int run_batch(const BatchLaunch<R>& B, Prof* prof, cudaStream_t stream);

// Velocity predictor (velprd_traj0 + velprdA_to_C + level roll).
template <class R>
struct PredPlan {
  Geo g;
  long lev;  // elements per psi-shaped level
  R* ox;
  R* oy;
  R* oz;  // logical (1,1,1) of level 0 of the three-level stacks (caller layout)
  R* u;
  R* v;
  R* w;  // optional physical velocity stacks
  Arr<R> h, u1, u2, u3;
  R gc1, gc2, gc3, dt_ratio;
  Prof* prof;
};

template <class R>
int run_predictor(const PredPlan<R>& plan, cudaStream_t stream);
// The pieces separately: level = the n+1/2 momenta into level 1
// (velprd_traj0_adapt_dt), cgrid = velprdA_to_C of level 1, roll = the
// driver's level roll; roll without cgrid runs the roll alone.
template <class R>
int run_pred_parts(const PredPlan<R>& plan, bool level, bool cgrid, bool roll, cudaStream_t stream);
// compute_courants of momentum level 1 (gc*ox at level 0) or 2 (ox at level 1
// over h): folds the seven maxima into keys[0..6] (unsigned order keys of
// doubles, atomicMax), which the caller initialises.
template <class R>
int run_courants(const PredPlan<R>& plan, int level, R dxi, R dyi, R dzi, R dt, unsigned long long* keys,
                 cudaStream_t stream);
template <class R>
int run_halve(R* p, long n, cudaStream_t stream);
// Adjoint of run_predictor: plan.ox/oy/oz are the gradient level stacks,
// plan.u1..u3 the C-grid gradients dJ/du (see k_pred_adjoint).
template <class R>
int run_pred_adjoint(const PredPlan<R>& plan, cudaStream_t stream);

// Adjoint of one step (mpdata_adjoint.cu), gauge form, iord >= 2.
// Reverse-kernel arguments of one corrective pass: where each adjoint lives.
template <class R>
struct AdjArr {
  Arr<R> lxant;             // adjoint of the pass's input field (written first by the update's reverse)
  Arr<R> lv1, lv2, lv3;     // adjoints of the pseudo-velocities
  Arr<R> lw1, lw2, lw3;     // adjoints of the limited velocities (the next pass's pseudo adds too)
  Arr<R> lcp, lcn;          // adjoints of the limiter ratios
  Arr<R> lx;                // adjoint of the step's input psi
  Arr<R> lam;               // adjoint of the pass's output (the caller's lambda for the last pass)
  Arr<R> gu1, gu2, gu3;     // caller gradients of u1..u3 (C-grid shaped), accumulated
  Arr<R> la1, la2, la3;     // adjoint of the pass's "a" velocities: gu (first pass) or the previous lw
  Arr<R> lmx, lmn;          // adjoint of this pass's running extrema carried from the next pass
  Arr<R> lmxp, lmnp;        // ... of the previous pass's extrema (added when they win the fold)
  Arr<R> mxp, mnp;          // the previous pass's running extrema (values)
  // standard form only
  Arr<R> lg1, lg2, lg3;     // adjoints of the limited donor fluxes of x/rhr
  Arr<R> lf1, lf2, lf3;     // adjoints of the unlimited donor fluxes f*ns
  Arr<R> lq;                // adjoint of q = x/rhr
  // density step: cotangents of its mass fluxes (caller C-grid arrays, faces 1..n+1)
  Arr<R> lm1, lm2, lm3;
};

// Arena of the step adjoint: per-pass forward records and accumulators.
constexpr int kAdjMaxPass = 7;  // iord <= 8
template <class R>
struct AdjPlan {
  int npass;                                    // iord - 1
  Arr<R> x[kAdjMaxPass];                        // each pass's input field
  Arr<R> v[kAdjMaxPass][3], w[kAdjMaxPass][3];  // pseudo and limited velocities
  Arr<R> cp[kAdjMaxPass], cn[kAdjMaxPass];
  Arr<R> mx[kAdjMaxPass], mn[kAdjMaxPass];      // running extrema after each pass
  Arr<R> fns[kAdjMaxPass][3], q[kAdjMaxPass];   // standard form: unlimited donor fluxes, x/rhr
  Arr<R> lx[kAdjMaxPass], lw[kAdjMaxPass][3], lmx[kAdjMaxPass], lmn[kAdjMaxPass];
  Arr<R> lv[3], lcp, lcn;                       // reused by every pass
  Arr<R> lg[3], lf[3], lq;                      // reused by every pass (standard form)
  Arr<R> lxin;                                  // adjoint of the step's input psi
  Arr<R> lam;                                   // caller lambda: in dJ/dpsi_new, out dJ/dpsi_in
  Arr<R> gu1, gu2, gu3;                         // caller gradients of u1..u3
  R* acc;                                       // the accumulators, contiguous
  size_t acc_elems, pass_acc_elems;             // all of them; the per-pass block (lv, lcp, lcn)
  R* pass_acc;
  // density step (mpdata_rho_gauge_adjoint_*): the upwind divides by h
  // without rhr, and the mass fluxes (upwind flux + the last pass's limited
  // flux on every face) take the cotangents lm1..lm3 (p null when absent)
  bool rho;
  Arr<R> lm1, lm2, lm3;
};
// Fields of the arena for iord passes: records, then accumulators.
// records per pass: x, v*3, w*3, cp, cn, mx, mn, fns*3, q
inline size_t adj_record_fields(int iord) { return (size_t)(iord - 1) * 15; }
// accumulators: per pass lx, lw*3, lmx, lmn; shared lv*3, lcp, lcn, lg*3, lf*3, lq; lxin
inline size_t adj_acc_fields(int iord) { return (size_t)(iord - 1) * 6 + 12 + 1; }

template <class R>
int run_step_adjoint(const Prob<R>& P, const AdjPlan<R>& A, int nonos, cudaStream_t s);
template <class R>
int run_step_record(const Prob<R>& P, const AdjPlan<R>& A, int nonos, const Arr<R>* out, cudaStream_t s);
template <class R>
int run_step_reverse(const Prob<R>& P, const AdjPlan<R>& A, int nonos, cudaStream_t s);
template <class R>
int run_seed(const Prob<R>& P, const Arr<R>& psi, const Arr<R>& target, const Arr<R>& lam, cudaStream_t s);
// Reverse of the density step's outputs (x_incomp, pexr1/2, rhr) from the
// step's output field `out`: adds h*dJ/dx_incomp into lam and writes
// dJ/d(x_incomp input) and dJ/dpexe (null cotangent arrays are zeros).
template <class R>
int run_rho_out_adjoint(const Prob<R>& P, const Arr<R>& out, const Arr<R>& lxc, const Arr<R>& lp1,
                        const Arr<R>& lp2, const Arr<R>& lrh, const Arr<R>& lam, const Arr<R>& g_xinc,
                        const Arr<R>& g_pexe, cudaStream_t s);

unsigned long long launch_count();
void add_launches(int n);

}  // namespace mpdata
