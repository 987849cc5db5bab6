// Host interface of the fused single-precision MPDATA step (mpdata_fused.cu).
#pragma once
#include <cuda.h>

#include <vector>

#include "mpdata_stages.cuh"

namespace mpdata {

// Fields of the fused step's arena, each px*mp*lp floats (rows padded to a
// multiple of 4 elements so that every row starts on a 16-byte boundary, as
// TMA requires): the step's input field, the two ping-pong fields of the
// passes, pseudo and limited velocities, and two ping-pong pairs of running
// extrema.
enum FusedField { FZ_XIN = 0, FZ_X0, FZ_X1, FZ_V1, FZ_V2, FZ_V3, FZ_W1, FZ_W2, FZ_W3, FZ_MX0, FZ_MN0, FZ_MX1,
                  FZ_MN1, FZ_NF };

// Arguments of the fused kernels for one problem: caller arrays, the arena,
// the z-march chunk, and the arena fields of the current pass.
struct FusedArgs {
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

struct FusedPlan {
  Geo g;
  Arr<float> psi, u1, u2, u3, h, rhr;  // caller arrays
  float* arena;
  int px;       // arena row pitch (elements)
  long fs;      // elements per arena field
  int kchunk;   // planes per block of the z-march
  int* err;     // device error word (bit 1: a staging wait timed out)
  const CUtensorMap* tmap;  // one 4-D map over the arena (x, y, z, field)
};

// Whether a step takes the fused path: FP32, infinite gauge, nonoscillatory,
// iord >= 2, every axis periodic, not the density step.
bool fused_eligible(const Geo& g, int precision, int gauge, int nonos, int iord, int rho);
// Arena geometry: the row pitch and the total elements of the FZ_NF fields.
size_t fused_arena_elems(const Geo& g, int* px);
// Encodes the arena's tensor map (box 40 x 12 x 1 x 1).  0 on success.
int fused_make_tmap(CUtensorMap* map, float* arena, int px, const Geo& g);
// Planes per block of the z-march for this grid (MPDATA_FUSED_KCHUNK overrides).
int fused_kchunk(const Geo& g);
// One step; on return *mx_field / *mn_field name the arena fields that hold
// the running extrema of the step (-1 when iord = 2 keeps none).
int run_step_fused(const FusedPlan& F, int iord, Prof* prof, cudaStream_t s, int* mx_field, int* mn_field);

// Batches.  Each problem of the fused table gets work items (a tile of the
// upwind+pseudo kernel's height, or of the other kernels' height, and a z
// chunk) packed as problem | tile x << 16 | tile y << 32 | chunk << 48; one
// launch per fused kernel then covers every problem.
FusedArgs fused_args(const FusedPlan& F);
void fused_items(const Geo& g, int kchunk, int p, std::vector<unsigned long long>& up,
                 std::vector<unsigned long long>& rest);
int fused_init();
// One step of every problem of the table (device arrays: args, tensor maps,
// the two item lists).
int run_batch_fused(const FusedArgs* probs, const CUtensorMap* maps, const unsigned long long* items_up, int n_up,
                    const unsigned long long* items, int n, int iord, Prof* prof, cudaStream_t s);

}  // namespace mpdata
