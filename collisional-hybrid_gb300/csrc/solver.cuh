// solver.cuh -- potential solve of the hybrid-PIC hot path (src/potential.c,
// src/lhs.c, src/rhs.c) as matrix-free sm_103a kernels.
#pragma once

#include <vector>

#include "common.cuh"

namespace ch {

// Stencil scale factors of ComputeFullLHS (src/lhs.c:404-447) or of the
// Laplacian/identity operators, by --lhs-type.
struct OpCoefs {
  int type;                 // CH_LHS_*
  double sxx, syy, szz, sxy, sxz, syz, syx, szx, szy;
};
OpCoefs op_coefs(const ch_params& p, const GridDesc& g);

// One level of the operator: grid, coefficients, density.
template <typename T>
struct Level {
  GridDesc g;
  OpCoefs c;
  const T* n;               // density the operator is built from
};

struct SolveStats {
  int iterations;
  int refinements;
  double rnorm, bnorm;
};

// Device coefficients of one operator level (defined in solver.cu).
template <typename T>
struct DevCoefs {
  T sxx, syy, szz, sxy, sxz, syz, syx, szx, szy;
  int type;
  int cross;
};

// Geometric multigrid hierarchy in precision T.  Level 0 is the fine grid;
// level l+1 halves every axis of level l that stays >= 4 nodes when halved.
constexpr int CH_MG_MAX_LEVELS = 16;
template <typename T>
struct MGHier {
  int L = 0;
  GridDesc g[CH_MG_MAX_LEVELS];
  DevCoefs<T> C[CH_MG_MAX_LEVELS];
  int hx[CH_MG_MAX_LEVELS], hy[CH_MG_MAX_LEVELS], hz[CH_MG_MAX_LEVELS];  // halving to level l+1
  double sR[CH_MG_MAX_LEVELS];                                           // residual scale into l+1
  T *n[CH_MG_MAX_LEVELS], *dinv[CH_MG_MAX_LEVELS], *x[CH_MG_MAX_LEVELS], *b[CH_MG_MAX_LEVELS],
      *r[CH_MG_MAX_LEVELS], *t[CH_MG_MAX_LEVELS];
  int tail = -1;          // first level of the one-CTA tail cycle (k_mg_tail), or -1
  size_t tail_smem = 0;   // its shared memory
  bool built = false;
};

// Workspace and driver for the Krylov solves of one run.
class PotentialSolver {
 public:
  ch_status init(const ch_params& p, const GridDesc& g, int sms);
  void release();
  // RHS from the moments (SoA n, Gx, Gy, Gz; FP64), mean removed.
  void build_rhs(const double* mom, double* b, cudaStream_t s);
  // Solve A(n) phi = b; phi holds the warm start.  n is FP64.
  ch_status solve(const double* n, const double* b, double* phi, SolveStats* st, cudaStream_t s);
  // y = A(n) x in FP64.
  void apply64(const double* n, const double* x, double* y, cudaStream_t s);
  // Applied field of the RHS (varied by the adjoint's gradient and
  // finite-difference runs).
  void set_E0(const double E0[3]) {
    for (int d = 0; d < 3; ++d) p_.E0[d] = E0[d];
  }
  // Krylov method, preconditioner and tolerances for the following solves
  // (the multigrid hierarchy is built on the first solve that needs it).
  void set_options(int32_t ksp_type, int32_t pc_type, double rtol, double atol, int32_t max_it) {
    p_.ksp_type = ksp_type;
    p_.pc_type = pc_type;
    p_.ksp_rtol = rtol;
    p_.ksp_atol = atol;
    p_.ksp_max_it = max_it;
  }

 private:
  ch_status solve_fp64(const double* n, const double* b, double* phi, SolveStats* st, cudaStream_t s);
  ch_status solve_mixed(const double* n, const double* b, double* phi, SolveStats* st, cudaStream_t s);
  template <typename T>
  ch_status krylov(const GridDesc& g, const T* n, const T* b, T* x, double rtol, int maxit, bool zero_guess,
                   int* its, double* rnorm_out, MGHier<T>* mg, cudaStream_t s,
                   double bnorm_known = -1.0);
  double dot64(const double* a, const double* b, cudaStream_t s);
  template <typename T>
  ch_status mg_build(MGHier<T>& h);
  template <typename T>
  void mg_update(MGHier<T>& h, const T* n_fine, cudaStream_t s);
  template <typename T>
  void mg_vcycle(MGHier<T>& h, int l, const T* b, T* x, cudaStream_t s, double* part = nullptr);
  template <typename T>
  void mg_release(MGHier<T>& h);
  void remove_mean64(double* v, cudaStream_t s);

  ch_params p_{};
  GridDesc g_{};
  OpCoefs c_{};
  int sms_ = 0;
  int64_t N_ = 0;
  int nb_ = 0;              // blocks of the vector kernels
  // FP64 workspace
  double *r_ = nullptr, *z_ = nullptr, *pd_ = nullptr, *q_ = nullptr, *rh_ = nullptr, *s_ = nullptr, *t_ = nullptr,
         *sh_ = nullptr, *dinv_ = nullptr;
  // FP32 workspace (mixed form)
  float *n32_ = nullptr, *b32_ = nullptr, *x32_ = nullptr, *r32_ = nullptr, *z32_ = nullptr, *p32_ = nullptr,
        *q32_ = nullptr, *rh32_ = nullptr, *s32_ = nullptr, *t32_ = nullptr, *sh32_ = nullptr, *dinv32_ = nullptr;
  // one captured Krylov iteration per (precision, method, buffers)
  struct GraphKey {
    int tsize, ksp;
    const void *mg, *n, *b, *x;
    bool operator==(const GraphKey& o) const {
      return tsize == o.tsize && ksp == o.ksp && mg == o.mg && n == o.n && b == o.b && x == o.x;
    }
  };
  struct GraphEntry {
    GraphKey k;
    cudaGraphExec_t exec;
    long long nodes;
  };
  std::vector<GraphEntry> graphs_;
  cudaEvent_t evs_[4] = {nullptr, nullptr, nullptr, nullptr};
  double* hring_ = nullptr;
  MGHier<float> mg32_;
  MGHier<double> mg64_;
  double* part_ = nullptr;  // block partials
  double* scal_ = nullptr;  // device scalars
  double* hscal_ = nullptr; // pinned host mirror
};

}  // namespace ch
