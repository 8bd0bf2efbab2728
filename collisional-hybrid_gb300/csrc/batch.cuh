// batch.cuh -- device descriptors of the ensemble (ch_batch) potential solve.
#pragma once

#include "solver_dev.cuh"

namespace ch {

// One multigrid level of one run (FP32).  Level 0 uses n and dinv; x, b
// are the level's V-cycle unknown and right-hand side below level 0; r and t
// are the residual and smoother scratch.
struct BLevel {
  GridDesc g;
  DevCoefs<float> C;
  int hx, hy, hz;   // halving to level l + 1
  float sR;         // residual scale into level l + 1
  float *n, *dinv, *x, *b, *r, *t;
};

struct BSolveOut {
  int iterations, refinements, status, flags;
  double rnorm, bnorm;
};

// Everything one cluster needs to solve the potential of one run: the RHS
// from the moments, FP64 iterative refinement around FP32 MG-PCG, and the
// node field of the next push.
struct BSolveRun {
  GridDesc g;
  DevCoefs<double> C64;
  RhsCoefs K;
  double rtol, atol;
  int maxit;          // inner Krylov iterations per refinement
  int L;              // multigrid levels
  double tscale;      // (q/m) dt/2 of the push
  BLevel lv[CH_MG_MAX_LEVELS];
  const double* mom;  // n, Gx, Gy, Gz (SoA, 4 N)
  double *phi, *b64, *r64;
  float *b32, *x32, *r32, *z32, *p32, *q32;
  float4* E32;
  BSolveOut* out;
};

// Coarsest-level bound of the in-cluster solve (shared memory per CTA).
constexpr int BATCH_COARSE_MAX = 2048;

// One launch: run r is solved by the cluster of `cluster` CTAs starting at
// block r * cluster.
cudaError_t launch_batch_solve(const BSolveRun* runs, int nruns, int cluster, cudaStream_t s);
// Allows clusters of 16 CTAs for the solve on the current device (false if refused).
bool batch_solve_allow_wide();

}  // namespace ch
