// Launch plans for the MPDATA stage kernels.
#pragma once
#include "mpdata_common.cuh"

namespace mpdata {

// Stage ids for the optional per-launch CUDA-event timing.
enum Stage { ST_UPWIND = 0, ST_PSEUDO, ST_BOUNDS, ST_LIMIT, ST_UPDATE, ST_COPY, ST_PRED_LEVEL,
             ST_PRED_CGRID, NSTAGE };

// Records a pair of CUDA events around each launch when enabled (the events
// live on the launching stream, so they time exactly that kernel).
struct Prof {
  virtual void begin(int stage, cudaStream_t s) = 0;
  virtual void end(int stage, cudaStream_t s) = 0;
  virtual ~Prof() {}
};

// Everything one step needs: caller arrays (Fortran layout views) and the
// workspace scratch (interior-shaped views).
template <class R>
struct StepPlan {
  Geo g;
  int iord, nonos, gauge;
  Arr<R> psi, u1, u2, u3, h, rhr;
  const R* bcx;
  const R* bcy;
  // scratch
  Arr<R> xant, hinv, v1, v2, v3, f1, f2, f3, w1, w2, w3, cp, cn, mx, mn, q;
  Prof* prof;  // NULL = no timing
};

template <class R>
int run_step(const StepPlan<R>& plan, cudaStream_t stream);

// Velocity predictor (velprd_traj0 + velprdA_to_C + level roll).
template <class R>
struct PredPlan {
  Geo g;
  long lev;  // elements per psi-shaped level
  R* ox;
  R* oy;
  R* oz;  // base pointers of the three-level stacks (caller layout)
  R* u;
  R* v;
  R* w;  // optional physical velocity stacks
  Arr<R> h, u1, u2, u3;
  R gc1, gc2, gc3, dt_ratio;
  Prof* prof;
};

template <class R>
int run_predictor(const PredPlan<R>& plan, cudaStream_t stream);

unsigned long long launch_count();
void add_launches(int n);

}  // namespace mpdata
