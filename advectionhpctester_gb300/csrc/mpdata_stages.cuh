// Launch sequences of the MPDATA kernels (host side).
#pragma once
#include "mpdata_body.cuh"

namespace mpdata {

// Stage ids for the optional per-launch CUDA-event timing.
enum Stage { ST_UPWIND = 0, ST_PSEUDO, ST_BOUNDS, ST_LIMIT, ST_UPDATE, ST_COPY, ST_PRED_LEVEL,
             ST_PRED_CGRID, ST_RHO_OUT, NSTAGE };

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

// Adjoint scratch of one problem (mpdata_adjoint.cu).
template <class R>
struct AdjArr {
  Arr<R> lxant, lv1, lv2, lv3, lw1, lw2, lw3, lcp, lcn, lx;
  Arr<R> lam;            // caller lambda: in dJ/dpsi_new, out dJ/dpsi_in (psi-shaped)
  Arr<R> gu1, gu2, gu3;  // caller gradients of u1..u3 (C-grid shaped), accumulated
};
template <class R>
int run_step_adjoint(const Prob<R>& P, const AdjArr<R>& A, int nonos, R* zero, size_t ncell, cudaStream_t s);
template <class R>
int run_seed(const Prob<R>& P, const Arr<R>& psi, const Arr<R>& target, const Arr<R>& lam, cudaStream_t s);

unsigned long long launch_count();
void add_launches(int n);

}  // namespace mpdata
