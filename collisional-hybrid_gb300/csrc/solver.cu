// solver.cu -- matrix-free 19-point potential solve on sm_103a.
//
// The operator is ComputeFullLHS (src/lhs.c:350-543) applied without ever
// assembling it: each row's 19 values are rebuilt on the fly from the
// density at the node and its six face neighbours, so one application reads
// x and n once and writes y once.  ComputeLaplacianLHS (:168-347) and
// ComputeIdentityLHS (:144) are selectable.  The RHS is ComputeFullRHS
// (src/rhs.c:133-303) with its null-space removal.  Krylov drivers: CG for
// the symmetric (kappa_e = 0) operator, BiCGStab otherwise, Jacobi
// preconditioned, constant null space projected out of b and phi; the
// mixed form runs the Krylov iterations in FP32 inside an FP64 iterative
// refinement of phi.  Reductions use fixed block partials summed in fixed
// order, so every solve is deterministic.
#include <math.h>
#include <string.h>

#include "solver_dev.cuh"

namespace ch {

OpCoefs op_coefs(const ch_params& p, const GridDesc& g) {
  OpCoefs c;
  memset(&c, 0, sizeof(c));
  c.type = p.lhs_type;
  if (p.lhs_type == CH_LHS_LAPLACIAN) {
    // src/lhs.c:204-218 (finite-volume scaled)
    c.sxx = g.dy * g.dz / g.dx;
    c.syy = g.dx * g.dz / g.dy;
    c.szz = g.dx * g.dy / g.dz;
    return c;
  }
  const double Kx = p.kappa_e[0], Ky = p.kappa_e[1], Kz = p.kappa_e[2];
  const double det = 1 + Kx * Kx + Ky * Ky + Kz * Kz;
  const double rxx = 1 + Kx * Kx, rxy = Ky * Kx - Kz, rxz = Kz * Kx + Ky;
  const double ryx = Kx * Ky + Kz, ryy = 1 + Ky * Ky, ryz = Kz * Ky - Kx;
  const double rzx = Kx * Kz - Ky, rzy = Ky * Kz + Kx, rzz = 1 + Kz * Kz;
  const double hxx = 1.0 / (2.0 * g.dx * g.dx), hyy = 1.0 / (2.0 * g.dy * g.dy), hzz = 1.0 / (2.0 * g.dz * g.dz);
  const double hxy = 1.0 / (8.0 * g.dy * g.dx), hxz = 1.0 / (8.0 * g.dz * g.dx), hyz = 1.0 / (8.0 * g.dy * g.dz);
  const double scale = 1.0 / det;
  c.sxx = scale * rxx * hxx; c.syy = scale * ryy * hyy; c.szz = scale * rzz * hzz;
  c.sxy = scale * rxy * hxy; c.sxz = scale * rxz * hxz; c.syz = scale * ryz * hyz;
  c.syx = scale * ryx * hxy; c.szx = scale * rzx * hxz; c.szy = scale * rzy * hyz;
  return c;
}

#define GRID_LOOP(c, N) for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < (N); c += (int64_t)gridDim.x * blockDim.x)

// Programmatic dependent launch.  The solver is a chain of short dependent
// kernels, so each one is launched with programmatic stream serialization:
// it may be scheduled while the kernel before it finishes, waits in
// pdl_enter (griddepcontrol.wait: the previous grid has completed and its
// writes are visible) before its first read, and then lets the next kernel be
// scheduled.  The next kernel is released only when every block of this one
// has done so, so blocks waiting there never hold back a grid still running.
// Launched without the attribute, the wait returns at once.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <typename... KP, typename... A>
static void launch(void (*k)(KP...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args) {
  static_assert(sizeof...(KP) == sizeof...(A), "kernel arguments");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, (KP)args...);  // errors surface at the stream's next check, as with <<<>>>
  ::ch::note_launch();
}

// ------------------------------------------------------------------ kernels
// y = A x; partial w.y (w may be null).
template <typename T>
__global__ void __launch_bounds__(256) k_apply(GridDesc g, DevCoefs<T> C, const T* __restrict__ n,
                                               const T* __restrict__ x, T* __restrict__ y, const T* __restrict__ w,
                                               double* part) {
  pdl_enter();
  T d0 = T(0);
  GRID_LOOP(c, g.N) {
    const Nb b = neighbours(g, c);
    const T v = apply_row<T>(C, n, x, b);
    y[c] = v;
    if (w) d0 += w[c] * v;
  }
  if (part) {
    double d[1] = {(double)d0};
    partials<1>(d, part);
  }
}

// t = A x; partials (t.s, t.t).
template <typename T>
__global__ void __launch_bounds__(256) k_apply_dot2(GridDesc g, DevCoefs<T> C, const T* __restrict__ n,
                                                    const T* __restrict__ x, T* __restrict__ t,
                                                    const T* __restrict__ s, double* part) {
  pdl_enter();
  T d0 = T(0), d1 = T(0);
  GRID_LOOP(c, g.N) {
    const Nb b = neighbours(g, c);
    const T v = apply_row<T>(C, n, x, b);
    t[c] = v;
    d0 += v * s[c];
    d1 += v * v;
  }
  double d[2] = {(double)d0, (double)d1};
  partials<2>(d, part);
}

// r = b - A x; partial r.r
template <typename T>
__global__ void __launch_bounds__(256) k_residual(GridDesc g, DevCoefs<T> C, const T* __restrict__ n,
                                                  const T* __restrict__ b, const T* __restrict__ x,
                                                  T* __restrict__ r, double* part) {
  pdl_enter();
  T d0 = T(0);
  GRID_LOOP(c, g.N) {
    const Nb nb = neighbours(g, c);
    const T v = b[c] - apply_row<T>(C, n, x, nb);
    r[c] = v;
    d0 += v * v;
  }
  double d[1] = {(double)d0};
  partials<1>(d, part);
}

template <typename T>
__global__ void k_jacobi(GridDesc g, DevCoefs<T> C, const T* __restrict__ n, T* __restrict__ dinv, int jacobi) {
  pdl_enter();
  GRID_LOOP(c, g.N) {
    const T d = jacobi ? diag_row<T>(C, n, neighbours(g, c)) : T(1);
    dinv[c] = d != T(0) ? T(1) / d : T(1);
  }
}

// z = dinv r; partials (r.z, r.r)
template <typename T>
__global__ void k_prec_dot(int64_t N, const T* __restrict__ dinv, const T* __restrict__ r, T* __restrict__ z,
                           double* part) {
  pdl_enter();
  T d0 = T(0), d1 = T(0);
  GRID_LOOP(c, N) {
    const T rv = r[c];
    const T zv = dinv[c] * rv;
    z[c] = zv;
    d0 += rv * zv;
    d1 += rv * rv;
  }
  double d[2] = {(double)d0, (double)d1};
  partials<2>(d, part);
}

// scalar slots
enum {
  S_RZ = 0, S_PQ, S_ALPHA, S_BETA, S_RR, S_RHO, S_OMEGA, S_TS, S_TT, S_RV, S_SS, S_RR0, S_MEAN, S_TMP, S_NSLOT
};
enum { OP_SET_RZ_RR = 0, OP_CG_ALPHA, OP_CG_BETA, OP_RR, OP_BI_ALPHA, OP_BI_OMEGA, OP_BI_BETA, OP_SS, OP_MEAN, OP_TMP,
       OP_SET_BICG };

// Fixed-order reduction of K partials and the scalar update of one step.
__global__ void k_scalar(const double* __restrict__ part, int nb, int K, int op, double* scal, double invN) {
  pdl_enter();
  __shared__ double sm[3][32];
  __shared__ double red[3];
  for (int q = 0; q < K; ++q) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[(size_t)b * K + q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[q][threadIdx.x >> 5] = s;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    for (int q = 0; q < K; ++q) {
      double t = threadIdx.x < (blockDim.x >> 5) ? sm[q][threadIdx.x] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (threadIdx.x == 0) red[q] = t;
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  switch (op) {
    case OP_SET_RZ_RR: scal[S_RZ] = red[0]; scal[S_RR] = red[1]; break;
    case OP_CG_ALPHA: scal[S_PQ] = red[0]; scal[S_ALPHA] = red[0] != 0.0 ? scal[S_RZ] / red[0] : 0.0; break;
    case OP_CG_BETA:
      scal[S_BETA] = scal[S_RZ] != 0.0 ? red[0] / scal[S_RZ] : 0.0;
      scal[S_RZ] = red[0];
      scal[S_RR] = red[1];
      break;
    case OP_RR: scal[S_RR] = red[0]; break;
    case OP_BI_ALPHA: scal[S_RV] = red[0]; scal[S_ALPHA] = red[0] != 0.0 ? scal[S_RHO] / red[0] : 0.0; break;
    case OP_SS: scal[S_SS] = red[0]; break;
    case OP_BI_OMEGA:
      scal[S_TS] = red[0]; scal[S_TT] = red[1];
      scal[S_OMEGA] = red[1] != 0.0 ? red[0] / red[1] : 0.0;
      break;
    case OP_BI_BETA: {
      // red[0] = r.r, red[1] = rh.r (rho new)
      scal[S_RR] = red[0];
      const double rho1 = red[1];
      scal[S_BETA] = (scal[S_RHO] != 0.0 && scal[S_OMEGA] != 0.0)
                         ? (rho1 / scal[S_RHO]) * (scal[S_ALPHA] / scal[S_OMEGA]) : 0.0;
      scal[S_RHO] = rho1;
      break;
    }
    case OP_MEAN: scal[S_MEAN] = red[0] * invN; break;
    case OP_TMP: scal[S_TMP] = red[0]; break;
    case OP_SET_BICG: scal[S_RHO] = scal[S_RR]; scal[S_BETA] = 0.0; scal[S_OMEGA] = 0.0; scal[S_ALPHA] = 0.0; break;
  }
}

// CG: x += a p; r -= a q; z = dinv r; partials (r.z, r.r)
template <typename T>
__global__ void k_cg_xr(int64_t N, const double* __restrict__ scal, T* __restrict__ x, T* __restrict__ r,
                        const T* __restrict__ p, const T* __restrict__ q, const T* __restrict__ dinv,
                        T* __restrict__ z, double* part) {
  pdl_enter();
  const T a = (T)scal[S_ALPHA];
  T d0 = T(0), d1 = T(0);
  GRID_LOOP(c, N) {
    x[c] += a * p[c];
    const T rv = r[c] - a * q[c];
    r[c] = rv;
    const T zv = dinv[c] * rv;
    z[c] = zv;
    d0 += rv * zv;
    d1 += rv * rv;
  }
  double d[2] = {(double)d0, (double)d1};
  partials<2>(d, part);
}

// CG: x += a p; r -= a q (the preconditioner runs after)
template <typename T>
__global__ void k_cg_xr_plain(int64_t N, const double* __restrict__ scal, T* __restrict__ x, T* __restrict__ r,
                              const T* __restrict__ p, const T* __restrict__ q) {
  pdl_enter();
  const T a = (T)scal[S_ALPHA];
  GRID_LOOP(c, N) {
    x[c] += a * p[c];
    r[c] -= a * q[c];
  }
}

template <typename T>
__global__ void k_cg_p(int64_t N, const double* __restrict__ scal, const T* __restrict__ z, T* __restrict__ p,
                       int first) {
  pdl_enter();
  const T b = first ? T(0) : (T)scal[S_BETA];
  GRID_LOOP(c, N) p[c] = z[c] + b * p[c];
}

// BiCGStab: p = r + beta (p - omega v); y = dinv p
template <typename T>
__global__ void k_bi_p(int64_t N, const double* __restrict__ scal, const T* __restrict__ r, T* __restrict__ p,
                       const T* __restrict__ v, const T* __restrict__ dinv, T* __restrict__ y, int first) {
  pdl_enter();
  const T b = first ? T(0) : (T)scal[S_BETA], w = first ? T(0) : (T)scal[S_OMEGA];
  GRID_LOOP(c, N) {
    const T pv = r[c] + b * (p[c] - w * v[c]);
    p[c] = pv;
    if (dinv) y[c] = dinv[c] * pv;
  }
}

// s = r - alpha v; sh = dinv s; partial s.s
template <typename T>
__global__ void k_bi_s(int64_t N, const double* __restrict__ scal, const T* __restrict__ r, const T* __restrict__ v,
                       const T* __restrict__ dinv, T* __restrict__ s, T* __restrict__ sh, double* part) {
  pdl_enter();
  const T a = (T)scal[S_ALPHA];
  T d0 = T(0);
  GRID_LOOP(c, N) {
    const T sv = r[c] - a * v[c];
    s[c] = sv;
    if (dinv) sh[c] = dinv[c] * sv;
    d0 += sv * sv;
  }
  double d[1] = {(double)d0};
  partials<1>(d, part);
}

// x += alpha y + omega sh; r = s - omega t; partials (r.r, rh.r)
template <typename T>
__global__ void k_bi_xr(int64_t N, const double* __restrict__ scal, T* __restrict__ x, const T* __restrict__ y,
                        const T* __restrict__ sh, T* __restrict__ r, const T* __restrict__ s, const T* __restrict__ t,
                        const T* __restrict__ rh, double* part) {
  pdl_enter();
  const T a = (T)scal[S_ALPHA], w = (T)scal[S_OMEGA];
  T d0 = T(0), d1 = T(0);
  GRID_LOOP(c, N) {
    x[c] += a * y[c] + w * sh[c];
    const T rv = s[c] - w * t[c];
    r[c] = rv;
    d0 += rv * rv;
    d1 += rh[c] * rv;
  }
  double d[2] = {(double)d0, (double)d1};
  partials<2>(d, part);
}

// x += alpha y (early exit of BiCGStab when |s| is small); r = s
template <typename T>
__global__ void k_bi_half(int64_t N, const double* __restrict__ scal, T* __restrict__ x, const T* __restrict__ y,
                          T* __restrict__ r, const T* __restrict__ s) {
  pdl_enter();
  const T a = (T)scal[S_ALPHA];
  GRID_LOOP(c, N) {
    x[c] += a * y[c];
    r[c] = s[c];
  }
}

template <typename T>
__global__ void k_copy(int64_t N, const T* __restrict__ a, T* __restrict__ b) {
  pdl_enter(); GRID_LOOP(c, N) b[c] = a[c]; }
template <typename T>
__global__ void k_zero(int64_t N, T* __restrict__ a) {
  pdl_enter(); GRID_LOOP(c, N) a[c] = T(0); }

template <typename T>
__global__ void k_sum(int64_t N, const T* __restrict__ a, double* part) {
  pdl_enter();
  double d[1] = {0.0};
  GRID_LOOP(c, N) d[0] += (double)a[c];
  partials<1>(d, part);
}
__global__ void k_sub_mean(int64_t N, double* __restrict__ a, const double* __restrict__ scal) {
  pdl_enter();
  const double m = scal[S_MEAN];
  GRID_LOOP(c, N) a[c] -= m;
}
template <typename T>
__global__ void k_dot(int64_t N, const T* __restrict__ a, const T* __restrict__ b, double* part) {
  pdl_enter();
  T d0 = T(0);
  GRID_LOOP(c, N) d0 += a[c] * b[c];
  double d[1] = {(double)d0};
  partials<1>(d, part);
}
__global__ void k_dot64(int64_t N, const double* __restrict__ a, const double* __restrict__ b, double* part) {
  pdl_enter();
  double d[1] = {0.0};
  GRID_LOOP(c, N) d[0] += a[c] * b[c];
  partials<1>(d, part);
}
// r32 = (float)(r64 * s)
__global__ void k_down(int64_t N, const double* __restrict__ a, double s, float* __restrict__ b) {
  pdl_enter();
  GRID_LOOP(c, N) b[c] = (float)(a[c] * s);
}
// x64 += (double)x32 * s
__global__ void k_up_add(int64_t N, const float* __restrict__ a, double s, double* __restrict__ x) {
  pdl_enter();
  GRID_LOOP(c, N) x[c] += (double)a[c] * s;
}

// ComputeFullRHS (src/rhs.c:244-283) with the FD helpers of src/calculus.c;
// ComputeConstantRHS / ComputeSinusoidalRHS for the other --rhs-type values
// (cscale = 2 dx dy dz / det, the factor of both).
__global__ void k_rhs(GridDesc g, int rhs_type, RhsCoefs K, double cscale, const double* __restrict__ mom,
                      const double* __restrict__ scal, double* __restrict__ b) {
  pdl_enter();
  const int64_t N = g.N;
  const double* n = mom;
  const double* Gx = mom + N;
  const double* Gy = mom + 2 * N;
  const double* Gz = mom + 3 * N;
  GRID_LOOP(c, N) {
    if (rhs_type == CH_RHS_CONSTANT) {
      b[c] = scal[S_MEAN] * cscale;
      continue;
    }
    if (rhs_type == CH_RHS_SINUSOIDAL) {
      int i, j, k;
      ch_ijk(g, c, i, j, k);
      const double x = ((double)i + 0.5) * g.dx, y = ((double)j + 0.5) * g.dy, z = ((double)k + 0.5) * g.dz;
      const double val = cos(2 * CH_PI * x) * cos(2 * CH_PI * y) * cos(2 * CH_PI * z);
      b[c] = scal[S_MEAN] * val * cscale;
      continue;
    }
    b[c] = rhs_full_row(g, K, n, Gx, Gy, Gz, neighbours(g, c));
  }
}


// ------------------------------------------------------------------ multigrid
// Damped-Jacobi smoothing: y = x + w dinv (b - A x); x == nullptr means x = 0.
template <typename T>
__global__ void __launch_bounds__(256) k_smooth(GridDesc g, DevCoefs<T> C, const T* __restrict__ n,
                                                const T* __restrict__ dinv, const T* __restrict__ b,
                                                const T* __restrict__ x, T* __restrict__ y, T w) {
  pdl_enter();
  GRID_LOOP(c, g.N) {
    if (!x) {
      y[c] = w * dinv[c] * b[c];
    } else {
      const Nb nb = neighbours(g, c);
      y[c] = x[c] + w * dinv[c] * (b[c] - apply_row<T>(C, n, x, nb));
    }
  }
}

// Two damped-Jacobi sweeps from x = 0: the first iterate t = w dinv b is
// formed wherever the second sweep reads it, so it is never stored.
template <typename T>
__global__ void __launch_bounds__(256) k_smooth_zero2(GridDesc g, DevCoefs<T> C, const T* __restrict__ n,
                                                      const T* __restrict__ dinv, const T* __restrict__ b,
                                                      T* __restrict__ y, T w) {
  pdl_enter();
  auto t = [&](int64_t i) { return w * dinv[i] * b[i]; };
  GRID_LOOP(c, g.N) y[c] = t(c) + w * dinv[c] * (b[c] - apply_row_at<T>(C, n, t, neighbours(g, c)));
}

// r = b - A x without a norm (MG levels).
template <typename T>
__global__ void __launch_bounds__(256) k_resid(GridDesc g, DevCoefs<T> C, const T* __restrict__ n,
                                               const T* __restrict__ b, const T* __restrict__ x,
                                               T* __restrict__ r) {
  pdl_enter();
  GRID_LOOP(c, g.N) r[c] = b[c] - apply_row<T>(C, n, x, neighbours(g, c));
}

// Full weighting onto the coarse vertex grid (coarse node I = fine node 2I
// along each halved axis): 1D weights 1/4, 1/2, 1/4; axes that are not
// halved take the fine value.  Returns (R in) at coarse node c.
template <typename T>
__device__ __forceinline__ T restrict_node(const GridDesc& gf, const GridDesc& gc, int hx, int hy, int hz,
                                           const T* in, int64_t c) {
  int I, J, K;
  ch_ijk(gc, c, I, J, K);
  const int i0 = hx ? 2 * I : I, j0 = hy ? 2 * J : J, k0 = hz ? 2 * K : K;
  T acc = T(0);
  for (int dk = -hz; dk <= hz; ++dk) {
    const T wk = hz ? (dk == 0 ? T(0.5) : T(0.25)) : T(1);
    const int k = ch_wrap(k0 + dk, gf.Nz);
    for (int dj = -hy; dj <= hy; ++dj) {
      const T wj = hy ? (dj == 0 ? T(0.5) : T(0.25)) : T(1);
      const int j = ch_wrap(j0 + dj, gf.Ny);
      const int row = (k * gf.Ny + j) * gf.Nx;  // grids have < 2^31 nodes
      for (int di = -hx; di <= hx; ++di) {
        const T wi = hx ? (di == 0 ? T(0.5) : T(0.25)) : T(1);
        acc += wk * wj * wi * in[row + ch_wrap(i0 + di, gf.Nx)];
      }
    }
  }
  return acc;
}
// out = scale * R in.
template <typename T>
__global__ void k_restrict(GridDesc gf, GridDesc gc, int hx, int hy, int hz, const T* __restrict__ in,
                           T* __restrict__ out, T scale) {
  pdl_enter();
  GRID_LOOP(c, gc.N) out[c] = scale * restrict_node<T>(gf, gc, hx, hy, hz, in, c);
}

// Trilinear prolongation of ec to fine node c.
template <typename T>
__device__ __forceinline__ T prolong_node(const GridDesc& gf, const GridDesc& gc, int hx, int hy, int hz, const T* ec,
                                          int64_t c) {
  int i, j, k;
  ch_ijk(gf, c, i, j, k);
  int I0, I1, J0, J1, K0, K1;
  T wi1, wj1, wk1;
  if (hx) { I0 = i >> 1; I1 = (i & 1) ? ch_wrap(I0 + 1, gc.Nx) : I0; wi1 = (i & 1) ? T(0.5) : T(0); }
  else { I0 = I1 = i; wi1 = T(0); }
  if (hy) { J0 = j >> 1; J1 = (j & 1) ? ch_wrap(J0 + 1, gc.Ny) : J0; wj1 = (j & 1) ? T(0.5) : T(0); }
  else { J0 = J1 = j; wj1 = T(0); }
  if (hz) { K0 = k >> 1; K1 = (k & 1) ? ch_wrap(K0 + 1, gc.Nz) : K0; wk1 = (k & 1) ? T(0.5) : T(0); }
  else { K0 = K1 = k; wk1 = T(0); }
  const T wi0 = T(1) - wi1, wj0 = T(1) - wj1, wk0 = T(1) - wk1;
  auto at = [&](int I, int J, int K) { return ec[(K * gc.Ny + J) * gc.Nx + I]; };  // < 2^31 nodes
  return wk0 * (wj0 * (wi0 * at(I0, J0, K0) + wi1 * at(I1, J0, K0)) +
                wj1 * (wi0 * at(I0, J1, K0) + wi1 * at(I1, J1, K0))) +
         wk1 * (wj0 * (wi0 * at(I0, J0, K1) + wi1 * at(I1, J0, K1)) +
                wj1 * (wi0 * at(I0, J1, K1) + wi1 * at(I1, J1, K1)));
}
// xf += P ec.
template <typename T>
__global__ void k_prolong_add(GridDesc gf, GridDesc gc, int hx, int hy, int hz, const T* __restrict__ ec,
                              T* __restrict__ xf) {
  pdl_enter();
  GRID_LOOP(c, gf.N) xf[c] += prolong_node<T>(gf, gc, hx, hy, hz, ec, c);
}

// The lower part of a V(2,2) cycle in one CTA: levels q = 0 .. L-1 of the
// tail (level 0 of the tail has at most MG_TAIL_MAX nodes), every array in
// shared memory.  The node arithmetic is that of k_smooth_zero2, k_resid,
// k_restrict, k_coarse, k_prolong_add and k_smooth, so the result is the
// one of those kernels; the levels' launches become barriers.
constexpr int MG_TAIL_LEVELS = 8;
template <typename T>
struct TailLevels {
  GridDesc g[MG_TAIL_LEVELS];
  DevCoefs<T> C[MG_TAIL_LEVELS];
  const T* n[MG_TAIL_LEVELS];
  const T* dinv[MG_TAIL_LEVELS];
  int hx[MG_TAIL_LEVELS], hy[MG_TAIL_LEVELS], hz[MG_TAIL_LEVELS];  // halving from q to q + 1
  T sR[MG_TAIL_LEVELS];
  int off[MG_TAIL_LEVELS];  // level q's five arrays (n, dinv, b, x, t) start at element off[q]
  int L, sweeps;
};
// threads of the tail CTA (FP64 rows need more registers)
template <typename T>
constexpr int mg_tail_threads() { return sizeof(T) == 4 ? 1024 : 512; }
template <typename T>
__global__ void __launch_bounds__(mg_tail_threads<T>()) k_mg_tail(TailLevels<T> V, const T* __restrict__ b_in,
                                                                  T* __restrict__ x_out, T w) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smem_tail[];
  T* const base = reinterpret_cast<T*>(smem_tail);
  auto arr = [&](int q, int a) { return base + V.off[q] + (int64_t)a * V.g[q].N; };  // a: n dinv b x t
  for (int q = 0; q < V.L; ++q)
    for (int64_t c = threadIdx.x; c < V.g[q].N; c += blockDim.x) {
      arr(q, 0)[c] = V.n[q][c];
      arr(q, 1)[c] = V.dinv[q][c];
    }
  for (int64_t c = threadIdx.x; c < V.g[0].N; c += blockDim.x) arr(0, 2)[c] = b_in[c];
  __syncthreads();
  // down: two sweeps from zero, residual (into t), restriction
  for (int q = 0; q + 1 < V.L; ++q) {
    const GridDesc& g = V.g[q];
    const T *n = arr(q, 0), *dinv = arr(q, 1), *b = arr(q, 2);
    T *x = arr(q, 3), *r = arr(q, 4);
    auto t = [&](int64_t i) { return w * dinv[i] * b[i]; };
    for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x)
      x[c] = t(c) + w * dinv[c] * (b[c] - apply_row_at<T>(V.C[q], n, t, neighbours(g, c)));
    __syncthreads();
    for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x) r[c] = b[c] - apply_row<T>(V.C[q], n, x, neighbours(g, c));
    __syncthreads();
    T* b1 = arr(q + 1, 2);
    for (int64_t c = threadIdx.x; c < V.g[q + 1].N; c += blockDim.x)
      b1[c] = V.sR[q] * restrict_node<T>(g, V.g[q + 1], V.hx[q], V.hy[q], V.hz[q], r, c);
    __syncthreads();
  }
  // coarsest: sweeps from zero, x and t in turn
  const int qc = V.L - 1;
  {
    const GridDesc& g = V.g[qc];
    const T *n = arr(qc, 0), *dinv = arr(qc, 1), *b = arr(qc, 2);
    T *xa = arr(qc, 3), *xb = arr(qc, 4);
    for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x) xa[c] = w * dinv[c] * b[c];
    __syncthreads();
    for (int s = 1; s < V.sweeps; ++s) {
      for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x)
        xb[c] = xa[c] + w * dinv[c] * (b[c] - apply_row<T>(V.C[qc], n, xa, neighbours(g, c)));
      __syncthreads();
      T* tmp = xa; xa = xb; xb = tmp;
    }
    if (xa != arr(qc, 3)) {
      for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x) arr(qc, 3)[c] = xa[c];
      __syncthreads();
    }
  }
  // up: prolongation, two sweeps (x -> t -> x)
  for (int q = V.L - 2; q >= 0; --q) {
    const GridDesc& g = V.g[q];
    const T *n = arr(q, 0), *dinv = arr(q, 1), *b = arr(q, 2), *ec = arr(q + 1, 3);
    T *x = arr(q, 3), *t = arr(q, 4);
    for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x)
      x[c] += prolong_node<T>(g, V.g[q + 1], V.hx[q], V.hy[q], V.hz[q], ec, c);
    __syncthreads();
    for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x)
      t[c] = x[c] + w * dinv[c] * (b[c] - apply_row<T>(V.C[q], n, x, neighbours(g, c)));
    __syncthreads();
    for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x)
      x[c] = t[c] + w * dinv[c] * (b[c] - apply_row<T>(V.C[q], n, t, neighbours(g, c)));
    __syncthreads();
  }
  for (int64_t c = threadIdx.x; c < V.g[0].N; c += blockDim.x) x_out[c] = arr(0, 3)[c];
}

// Coarsest level: `sweeps` damped-Jacobi sweeps from zero in one block,
// iterates in shared memory (N <= 4096 nodes).
template <typename T>
__global__ void __launch_bounds__(1024) k_coarse(GridDesc g, DevCoefs<T> C, const T* __restrict__ n,
                                                 const T* __restrict__ dinv, const T* __restrict__ b,
                                                 T* __restrict__ x, int sweeps, T w) {
  pdl_enter();
  extern __shared__ unsigned char smem_raw[];
  T* xa = reinterpret_cast<T*>(smem_raw);
  T* xb = xa + g.N;
  for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x) xa[c] = w * dinv[c] * b[c];
  __syncthreads();
  for (int s = 1; s < sweeps; ++s) {
    for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x)
      xb[c] = xa[c] + w * dinv[c] * (b[c] - apply_row<T>(C, n, xa, neighbours(g, c)));
    __syncthreads();
    T* t = xa; xa = xb; xb = t;
  }
  for (int64_t c = threadIdx.x; c < g.N; c += blockDim.x) x[c] = xa[c];
}

// partials (r.z, r.r) after a multigrid preconditioner application
template <typename T>
__global__ void k_dot_rz_rr(int64_t N, const T* __restrict__ r, const T* __restrict__ z, double* part) {
  pdl_enter();
  T d0 = T(0), d1 = T(0);
  GRID_LOOP(c, N) {
    const T rv = r[c];
    d0 += rv * z[c];
    d1 += rv * rv;
  }
  double d[2] = {(double)d0, (double)d1};
  partials<2>(d, part);
}

// The last post-smoothing sweep of the finest level, with the preconditioned
// CG's partials (r.z, r.r) of r = b and z = y.
template <typename T>
__global__ void __launch_bounds__(256) k_smooth_dot(GridDesc g, DevCoefs<T> C, const T* __restrict__ n,
                                                    const T* __restrict__ dinv, const T* __restrict__ b,
                                                    const T* __restrict__ x, T* __restrict__ y, T w, double* part) {
  pdl_enter();
  T d0 = T(0), d1 = T(0);
  GRID_LOOP(c, g.N) {
    const Nb nb = neighbours(g, c);
    const T rv = b[c];
    const T z = x[c] + w * dinv[c] * (rv - apply_row<T>(C, n, x, nb));
    y[c] = z;
    d0 += rv * z;
    d1 += rv * rv;
  }
  double d[2] = {(double)d0, (double)d1};
  partials<2>(d, part);
}

// ------------------------------------------------------------------ host side
static int grid_n(int64_t n, int sms) {
  int64_t need = (n + 255) / 256;
  int64_t cap = (int64_t)sms * 4;
  return (int)(need < cap ? (need < 1 ? 1 : need) : cap);
}

ch_status PotentialSolver::init(const ch_params& p, const GridDesc& g, int sms) {
  p_ = p;
  g_ = g;
  c_ = op_coefs(p, g);
  sms_ = sms;
  N_ = g.N;
  nb_ = grid_n(N_, sms);
  const size_t b64 = sizeof(double) * N_;
  double** v64[] = {&r_, &z_, &pd_, &q_, &rh_, &s_, &t_, &sh_, &dinv_};
  for (double** v : v64) CH_CUDA_OK(cudaMalloc(v, b64));
  if (p.precision == CH_MIXED) {
    const size_t b32 = sizeof(float) * N_;
    float** v32[] = {&n32_, &b32_, &x32_, &r32_, &z32_, &p32_, &q32_, &rh32_, &s32_, &t32_, &sh32_, &dinv32_};
    for (float** v : v32) CH_CUDA_OK(cudaMalloc(v, b32));
  }
  CH_CUDA_OK(cudaMalloc(&part_, sizeof(double) * 4 * nb_));
  CH_CUDA_OK(cudaMalloc(&scal_, sizeof(double) * S_NSLOT));
  CH_CUDA_OK(cudaMemset(scal_, 0, sizeof(double) * S_NSLOT));
  CH_CUDA_OK(cudaMallocHost(&hscal_, sizeof(double) * S_NSLOT));
  CH_CUDA_OK(cudaMallocHost(&hring_, sizeof(double) * 4));
  for (auto& e : evs_) CH_CUDA_OK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return CH_OK;
}

void PotentialSolver::release() {
  for (auto& e : graphs_) cudaGraphExecDestroy(e.exec);
  graphs_.clear();
  for (auto& e : evs_)
    if (e) cudaEventDestroy(e);
  if (hring_) cudaFreeHost(hring_);
  hring_ = nullptr;
  mg_release<float>(mg32_);
  mg_release<double>(mg64_);
  void* all[] = {r_, z_, pd_, q_, rh_, s_, t_, sh_, dinv_, n32_, b32_, x32_, r32_, z32_, p32_, q32_, rh32_,
                 s32_, t32_, sh32_, dinv32_, part_, scal_};
  for (void* v : all)
    if (v) cudaFree(v);
  if (hscal_) cudaFreeHost(hscal_);
  r_ = z_ = pd_ = q_ = rh_ = s_ = t_ = sh_ = dinv_ = nullptr;
  n32_ = b32_ = x32_ = r32_ = z32_ = p32_ = q32_ = rh32_ = s32_ = t32_ = sh32_ = dinv32_ = nullptr;
  part_ = scal_ = hscal_ = nullptr;
}


// ------------------------------------------------------------------ multigrid (host)
static constexpr int MG_NU = 2;            // pre- and post-smoothing sweeps (even)
static constexpr double MG_OMEGA = 0.8;    // Jacobi damping
// Jacobi sweeps of the coarsest level: enough to reduce its smoothest mode
// well below the V-cycle's own error (4 per node of its longest edge; 16 for
// the 4^3 level of a 2^k grid, where 16 and 64 sweeps give the same Krylov
// iteration counts).
static int mg_coarse_sweeps(const GridDesc& g) {
  const int e = g.Nx > g.Ny ? (g.Nx > g.Nz ? g.Nx : g.Nz) : (g.Ny > g.Nz ? g.Ny : g.Nz);
  const int s = 4 * e;
  return s < 16 ? 16 : (s > 64 ? 64 : s);
}
static constexpr int64_t MG_COARSE_MAX = 4096;
static constexpr int64_t MG_TAIL_MAX = 512;          // top level of the one-CTA tail
static constexpr size_t MG_TAIL_SMEM = 200 * 1024;   // its shared memory at most

template <typename T>
ch_status PotentialSolver::mg_build(MGHier<T>& h) {
  if (h.built) return CH_OK;
  h.g[0] = g_;
  int L = 1;
  while (L < CH_MG_MAX_LEVELS) {
    const GridDesc& f = h.g[L - 1];
    const int hx = (f.Nx % 2 == 0 && f.Nx / 2 >= 4), hy = (f.Ny % 2 == 0 && f.Ny / 2 >= 4),
              hz = (f.Nz % 2 == 0 && f.Nz / 2 >= 4);
    if (!(hx || hy || hz) || f.N <= 64) break;
    GridDesc c = f;
    c.Nx = hx ? f.Nx / 2 : f.Nx; c.Ny = hy ? f.Ny / 2 : f.Ny; c.Nz = hz ? f.Nz / 2 : f.Nz;
    c.dx = hx ? 2 * f.dx : f.dx; c.dy = hy ? 2 * f.dy : f.dy; c.dz = hz ? 2 * f.dz : f.dz;
    ch_grid_finish(c);
    h.hx[L - 1] = hx; h.hy[L - 1] = hy; h.hz[L - 1] = hz;
    // the full operator is finite-difference scaled (averaged residuals);
    // the Laplacian of src/lhs.c:205-207 is finite-volume scaled
    h.sR[L - 1] = p_.lhs_type == CH_LHS_LAPLACIAN ? (c.dx * c.dy * c.dz) / (f.dx * f.dy * f.dz) : 1.0;
    h.g[L] = c;
    ++L;
  }
  if (h.g[L - 1].N > MG_COARSE_MAX)
    return ch_fail(CH_ERR_UNSUPPORTED, "multigrid: coarsest grid %dx%dx%d exceeds %lld nodes; use -ch_pc jacobi",
                   h.g[L - 1].Nx, h.g[L - 1].Ny, h.g[L - 1].Nz, (long long)MG_COARSE_MAX);
  h.L = L;
  for (int l = 0; l < L; ++l) {
    const size_t b = sizeof(T) * h.g[l].N;
    h.C[l] = dev_coefs<T>(op_coefs(p_, h.g[l]));
    h.n[l] = nullptr;
    if (l > 0) CH_CUDA_OK(cudaMalloc(&h.n[l], b));
    CH_CUDA_OK(cudaMalloc(&h.dinv[l], b));
    CH_CUDA_OK(cudaMalloc(&h.r[l], b));
    CH_CUDA_OK(cudaMalloc(&h.t[l], b));
    h.x[l] = h.b[l] = nullptr;
    if (l > 0) {
      CH_CUDA_OK(cudaMalloc(&h.x[l], b));
      CH_CUDA_OK(cudaMalloc(&h.b[l], b));
    }
  }
  // (per kernel, not per hierarchy: the largest coarse grid of any solver)
  CH_CUDA_OK(cudaFuncSetAttribute(k_coarse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(2 * sizeof(T) * MG_COARSE_MAX)));
  // the one-CTA tail: from the first level of at most MG_TAIL_MAX nodes,
  // when its levels' five arrays fit in shared memory
  h.tail = -1;
  h.tail_smem = 0;
  for (int l = 0; l + 1 < L; ++l) {
    if (h.g[l].N > MG_TAIL_MAX) continue;
    size_t bytes = 0;
    for (int q = l; q < L; ++q) bytes += 5 * sizeof(T) * (size_t)h.g[q].N;
    if (L - l <= MG_TAIL_LEVELS && bytes <= MG_TAIL_SMEM) {
      // the attribute belongs to the kernel, not to this hierarchy: the fixed
      // maximum serves every solver on the device
      CH_CUDA_OK(cudaFuncSetAttribute(k_mg_tail<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)MG_TAIL_SMEM));
      h.tail = l;
      h.tail_smem = bytes;
    }
    break;
  }
  h.built = true;
  return CH_OK;
}

template <typename T>
void PotentialSolver::mg_release(MGHier<T>& h) {
  for (int l = 0; l < h.L; ++l) {
    T* v[] = {l > 0 ? h.n[l] : nullptr, h.dinv[l], h.r[l], h.t[l], l > 0 ? h.x[l] : nullptr,
              l > 0 ? h.b[l] : nullptr};
    for (T* q : v)
      if (q) cudaFree(q);
  }
  h.L = 0;
  h.built = false;
}

// New density: restrict it down the hierarchy and rebuild the diagonals.
template <typename T>
void PotentialSolver::mg_update(MGHier<T>& h, const T* n_fine, cudaStream_t s) {
  h.n[0] = const_cast<T*>(n_fine);
  for (int l = 0; l < h.L; ++l) {
    if (l > 0)
      launch(k_restrict<T>, grid_n(h.g[l].N, sms_), 256, 0, s, h.g[l - 1], h.g[l], h.hx[l - 1], h.hy[l - 1], h.hz[l - 1],
                                                          h.n[l - 1], h.n[l], T(1));
    launch(k_jacobi<T>, grid_n(h.g[l].N, sms_), 256, 0, s, h.g[l], h.C[l], h.n[l], h.dinv[l], 1);
  }
}

// One V(2,2) cycle from a zero guess: x ~= A_l^{-1} b.  With part (finest
// level only) the partials (b.x, b.b) of the result are written to part by
// the last sweep, over the Krylov grid nb_.
template <typename T>
void PotentialSolver::mg_vcycle(MGHier<T>& h, int l, const T* b, T* x, cudaStream_t s, double* part) {
  const GridDesc& g = h.g[l];
  const int nb = grid_n(g.N, sms_);
  const T w = (T)MG_OMEGA;
  if (l == h.L - 1) {
    const size_t sh = 2 * sizeof(T) * g.N;
    launch(k_coarse<T>, 1, 1024, sh, s, g, h.C[l], h.n[l], h.dinv[l], b, x, mg_coarse_sweeps(g), w);
    if (part) launch(k_dot_rz_rr<T>, nb_, 256, 0, s, g.N, b, x, part);
    return;
  }
  if (l == h.tail) {
    TailLevels<T> V;
    V.L = h.L - l;
    V.sweeps = mg_coarse_sweeps(h.g[h.L - 1]);
    int off = 0;
    for (int q = 0; q < V.L; ++q) {
      V.g[q] = h.g[l + q];
      V.C[q] = h.C[l + q];
      V.n[q] = h.n[l + q];
      V.dinv[q] = h.dinv[l + q];
      V.hx[q] = h.hx[l + q]; V.hy[q] = h.hy[l + q]; V.hz[q] = h.hz[l + q];
      V.sR[q] = (T)h.sR[l + q];
      V.off[q] = off;
      off += 5 * (int)h.g[l + q].N;
    }
    launch(k_mg_tail<T>, 1, mg_tail_threads<T>(), h.tail_smem, s, V, b, x, w);
    if (part) launch(k_dot_rz_rr<T>, nb_, 256, 0, s, g.N, b, x, part);
    return;
  }
  // pre-smoothing (MG_NU = 2 sweeps from zero, in one pass)
  static_assert(MG_NU == 2, "the pre-smoothing pass fuses exactly two sweeps");
  launch(k_smooth_zero2<T>, nb, 256, 0, s, g, h.C[l], h.n[l], h.dinv[l], b, x, w);
  // residual, restriction, coarse correction, prolongation
  launch(k_resid<T>, nb, 256, 0, s, g, h.C[l], h.n[l], b, x, h.r[l]);
  launch(k_restrict<T>, grid_n(h.g[l + 1].N, sms_), 256, 0, s, g, h.g[l + 1], h.hx[l], h.hy[l], h.hz[l], h.r[l],
                                                          h.b[l + 1], (T)h.sR[l]);
  mg_vcycle<T>(h, l + 1, h.b[l + 1], h.x[l + 1], s);
  launch(k_prolong_add<T>, nb, 256, 0, s, g, h.g[l + 1], h.hx[l], h.hy[l], h.hz[l], h.x[l + 1], x);
  // post-smoothing: x -> t -> x
  for (int k = 0; k < MG_NU; ++k) {
    T* src = (k % 2 == 0) ? x : h.t[l];
    T* dst = (k % 2 == 0) ? h.t[l] : x;
    if (part && k == MG_NU - 1)
      launch(k_smooth_dot<T>, nb_, 256, 0, s, g, h.C[l], h.n[l], h.dinv[l], b, src, dst, w, part);
    else
      launch(k_smooth<T>, nb, 256, 0, s, g, h.C[l], h.n[l], h.dinv[l], b, src, dst, w);
  }
}

double PotentialSolver::dot64(const double* a, const double* b, cudaStream_t s) {
  launch(k_dot64, nb_, 256, 0, s, N_, a, b, part_);
  launch(k_scalar, 1, 256, 0, s, part_, nb_, 1, OP_RR, scal_, 0.0);
  cudaMemcpyAsync(hscal_, scal_, sizeof(double) * S_NSLOT, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  return hscal_[S_RR];
}

void PotentialSolver::remove_mean64(double* v, cudaStream_t s) {
  launch(k_sum<double>, nb_, 256, 0, s, N_, v, part_);
  launch(k_scalar, 1, 256, 0, s, part_, nb_, 1, OP_MEAN, scal_, 1.0 / (double)N_);
  launch(k_sub_mean, nb_, 256, 0, s, N_, v, scal_);
}

void PotentialSolver::build_rhs(const double* mom, double* b, cudaStream_t s) {
  const double Kx = p_.kappa_e[0], Ky = p_.kappa_e[1], Kz = p_.kappa_e[2];
  const double det = 1 + Kx * Kx + Ky * Ky + Kz * Kz;
  const double R00 = 1 + Kx * Kx, R01 = Ky * Kx - Kz, R02 = Kz * Kx + Ky;
  const double R10 = Kx * Ky + Kz, R11 = 1 + Ky * Ky, R12 = Kz * Ky - Kx;
  const double R20 = Kx * Kz - Ky, R21 = Ky * Kz + Kx, R22 = 1 + Kz * Kz;
  if (p_.rhs_type != CH_RHS_FULL) {
    // mean density (VecMean, src/rhs.c:34,93)
    launch(k_sum<double>, nb_, 256, 0, s, N_, mom, part_);
    launch(k_scalar, 1, 256, 0, s, part_, nb_, 1, OP_MEAN, scal_, 1.0 / (double)N_);
  }
  const double R[9] = {R00, R01, R02, R10, R11, R12, R20, R21, R22};
  const RhsCoefs K = rhs_coefs(R, det, p_.E0, p_.cth, p_.cG, (p_.faithful & CH_FAITHFUL_D8) != 0, g_.dx, g_.dy, g_.dz);
  launch(k_rhs, nb_, 256, 0, s, g_, p_.rhs_type, K, 2.0 * g_.dx * g_.dy * g_.dz / det, mom, scal_, b);
  if (p_.rhs_type != CH_RHS_CONSTANT) remove_mean64(b, s);  // MatNullSpaceRemove (src/rhs.c:294-296)
}

void PotentialSolver::apply64(const double* n, const double* x, double* y, cudaStream_t s) {
  launch(k_apply<double>, nb_, 256, 0, s, g_, dev_coefs<double>(c_), n, x, y, nullptr, nullptr);
}

// Preconditioned Krylov solve of A x = b in precision T (x holds the start).
// Converged when ||r||_2 <= rtol ||b||_2 (recurrence residual).
template <typename T>
ch_status PotentialSolver::krylov(const GridDesc& g, const T* n, const T* b, T* x, double rtol, int maxit,
                                  bool zero_guess, int* its, double* rnorm_out, MGHier<T>* mg, cudaStream_t s,
                                  double bnorm_known) {
  const DevCoefs<T> C = dev_coefs<T>(c_);
  const int64_t N = g.N;
  const bool f64 = sizeof(T) == 8;
  T* r = f64 ? (T*)r_ : (T*)r32_;
  T* z = f64 ? (T*)z_ : (T*)z32_;
  T* pp = f64 ? (T*)pd_ : (T*)p32_;
  T* q = f64 ? (T*)q_ : (T*)q32_;
  T* rh = f64 ? (T*)rh_ : (T*)rh32_;
  T* sv = f64 ? (T*)s_ : (T*)s32_;
  T* tv = f64 ? (T*)t_ : (T*)t32_;
  T* sh = f64 ? (T*)sh_ : (T*)sh32_;
  T* dinv = f64 ? (T*)dinv_ : (T*)dinv32_;
  const int nb = nb_;
  if (!mg) launch(k_jacobi<T>, nb, 256, 0, s, g, C, n, dinv, p_.pc_type == CH_PC_JACOBI);
  // z = M r with M = Jacobi (fused) or one multigrid V-cycle
  auto precond = [&](const T* rr_, T* zz_) {
    if (mg) {
      mg_vcycle<T>(*mg, 0, rr_, zz_, s, part_);  // with the partials (r.z, r.r)
    } else {
      launch(k_prec_dot<T>, nb, 256, 0, s, N, dinv, rr_, zz_, part_);
    }
  };
  if (zero_guess) {
    launch(k_zero<T>, nb, 256, 0, s, N, x);
    launch(k_copy<T>, nb, 256, 0, s, N, b, r);
  } else {
    launch(k_residual<T>, nb, 256, 0, s, g, C, n, b, x, r, part_);
  }
  precond(r, z);
  launch(k_scalar, 1, 256, 0, s, part_, nb, 2, OP_SET_RZ_RR, scal_, 0.0);
  // ||b||: given by the caller (no host round trip; the first iterations
  // then run even when the start is already converged), or measured
  double bnorm = bnorm_known, rr = 0.0;
  if (!(bnorm_known >= 0.0)) {
    launch(k_dot<T>, nb, 256, 0, s, N, b, b, part_);
    launch(k_scalar, 1, 256, 0, s, part_, nb, 1, OP_TMP, scal_, 0.0);
    CH_CUDA_OK(cudaMemcpyAsync(hscal_, scal_, sizeof(double) * S_NSLOT, cudaMemcpyDeviceToHost, s));
    CH_CUDA_OK(cudaStreamSynchronize(s));
    bnorm = sqrt(hscal_[S_TMP]);
    rr = hscal_[S_RR];
  }
  const double tol = rtol * bnorm;
  int it = 0;
  if (bnorm == 0.0 || (!(bnorm_known >= 0.0) && sqrt(rr) <= tol)) {
    *its = 0;
    *rnorm_out = sqrt(rr);
    return CH_OK;
  }
  // One iteration, enqueued on s directly or under graph capture.  Scalars
  // stay on the device, so an iteration has no host dependency.
  auto cg_body = [&]() {
    launch(k_apply<T>, nb, 256, 0, s, g, C, n, pp, q, pp, part_);
    launch(k_scalar, 1, 256, 0, s, part_, nb, 1, OP_CG_ALPHA, scal_, 0.0);
    if (mg) {
      launch(k_cg_xr_plain<T>, nb, 256, 0, s, N, scal_, x, r, pp, q);
      precond(r, z);
    } else {
      launch(k_cg_xr<T>, nb, 256, 0, s, N, scal_, x, r, pp, q, dinv, z, part_);
    }
    launch(k_scalar, 1, 256, 0, s, part_, nb, 2, OP_CG_BETA, scal_, 0.0);
    launch(k_cg_p<T>, nb, 256, 0, s, N, scal_, z, pp, 0);
  };
  // BiCGStab, right preconditioned (van der Vorst 1992); p = v = 0 at the
  // start makes the first p = r whatever beta and omega hold.
  auto bi_body = [&]() {
    launch(k_bi_p<T>, nb, 256, 0, s, N, scal_, r, pp, q, mg ? (const T*)nullptr : dinv, z, 0);  // z = y = M p
    if (mg) mg_vcycle<T>(*mg, 0, pp, z, s);
    launch(k_apply<T>, nb, 256, 0, s, g, C, n, z, q, rh, part_);  // v = A y; rh.v
    launch(k_scalar, 1, 256, 0, s, part_, nb, 1, OP_BI_ALPHA, scal_, 0.0);
    launch(k_bi_s<T>, nb, 256, 0, s, N, scal_, r, q, mg ? (const T*)nullptr : dinv, sv, sh, part_);
    if (mg) mg_vcycle<T>(*mg, 0, sv, sh, s);
    launch(k_apply_dot2<T>, nb, 256, 0, s, g, C, n, sh, tv, sv, part_);
    launch(k_scalar, 1, 256, 0, s, part_, nb, 2, OP_BI_OMEGA, scal_, 0.0);
    launch(k_bi_xr<T>, nb, 256, 0, s, N, scal_, x, z, sh, r, sv, tv, rh, part_);
    launch(k_scalar, 1, 256, 0, s, part_, nb, 2, OP_BI_BETA, scal_, 0.0);
  };
  const bool cg = p_.ksp_type == CH_KSP_CG;
  if (cg) {
    launch(k_cg_p<T>, nb, 256, 0, s, N, scal_, z, pp, 1);
  } else {
    launch(k_copy<T>, nb, 256, 0, s, N, r, rh);
    launch(k_zero<T>, nb, 256, 0, s, N, pp);
    launch(k_zero<T>, nb, 256, 0, s, N, q);  // v
    launch(k_scalar, 1, 256, 0, s, part_, nb, 2, OP_SET_BICG, scal_, 0.0);
  }
  // the iteration as one CUDA graph (captured once per buffer set)
  GraphKey key{(int)sizeof(T), (int)p_.ksp_type, (const void*)mg, (const void*)n, (const void*)b, (const void*)x};
  GraphEntry* ge = nullptr;
  for (auto& e : graphs_)
    if (e.k == key) ge = &e;
  if (!ge) {
    cudaGraph_t graph;
    const unsigned long long before = ::ch::launches_now();
    CH_CUDA_OK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    if (cg) cg_body(); else bi_body();
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess) return ch_cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
    const long long nodes = (long long)(::ch::launches_now() - before);
    ::ch::note_launch_n(-nodes);  // captured, not yet launched
    GraphEntry e;
    e.k = key;
    e.nodes = nodes;
    ce = cudaGraphInstantiate(&e.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return ch_cuda_fail(ce, "cudaGraphInstantiate", __FILE__, __LINE__);
    graphs_.push_back(e);
    ge = &graphs_.back();
  }
  // Launch iterations back to back; test iteration k-1's residual while
  // iteration k runs (so a converged solve runs one extra iteration).
  const int RING = 4;
  bool converged = false;
  while (it < maxit) {
    CH_CUDA_OK(cudaGraphLaunch(ge->exec, s));
    ::ch::note_launch_n(ge->nodes);
    CH_CUDA_OK(cudaMemcpyAsync(hring_ + it % RING, scal_ + S_RR, sizeof(double), cudaMemcpyDeviceToHost, s));
    CH_CUDA_OK(cudaEventRecord(evs_[it % RING], s));
    ++it;
    if (it >= 2) {
      CH_CUDA_OK(cudaEventSynchronize(evs_[(it - 2) % RING]));
      if (!(sqrt(hring_[(it - 2) % RING]) > tol)) { converged = true; break; }
    }
  }
  CH_CUDA_OK(cudaStreamSynchronize(s));
  rr = hring_[(it - 1) % RING];
  (void)converged;
  *its = it;
  *rnorm_out = sqrt(rr);
  return CH_OK;
}

ch_status PotentialSolver::solve(const double* n, const double* b, double* phi, SolveStats* st, cudaStream_t s) {
  st->iterations = 0;
  st->refinements = 0;
  ch_status rc = (p_.precision == CH_MIXED && p_.lhs_type != CH_LHS_IDENTITY) ? solve_mixed(n, b, phi, st, s)
                                                                             : solve_fp64(n, b, phi, st, s);
  return rc;
}

ch_status PotentialSolver::solve_fp64(const double* n, const double* b, double* phi, SolveStats* st,
                                      cudaStream_t s) {
  const bool singular = p_.lhs_type != CH_LHS_IDENTITY;
  if (singular) remove_mean64(phi, s);
  int its = 0;
  double rn = 0.0;
  MGHier<double>* mg = nullptr;
  if (p_.pc_type == CH_PC_MG) {
    ch_status rm = mg_build<double>(mg64_);
    if (rm) return rm;
    mg_update<double>(mg64_, n, s);
    mg = &mg64_;
  }
  ch_status rc = krylov<double>(g_, n, b, phi, p_.ksp_rtol, p_.ksp_max_it, false, &its, &rn, mg, s);
  if (rc) return rc;
  if (singular) remove_mean64(phi, s);
  // true residual
  launch(k_residual<double>, nb_, 256, 0, s, g_, dev_coefs<double>(c_), n, b, phi, r_, part_);
  launch(k_scalar, 1, 256, 0, s, part_, nb_, 1, OP_RR, scal_, 0.0);
  CH_CUDA_OK(cudaMemcpyAsync(hscal_, scal_, sizeof(double) * S_NSLOT, cudaMemcpyDeviceToHost, s));
  CH_CUDA_OK(cudaStreamSynchronize(s));
  st->iterations = its;
  st->rnorm = sqrt(hscal_[S_RR]);
  st->bnorm = sqrt(dot64(b, b, s));
  const double tol = fmax(p_.ksp_rtol * st->bnorm, p_.ksp_atol);
  if (st->rnorm > tol * 1.01 && st->rnorm > 0.0) return CH_ERR_NOT_CONVERGED;
  return CH_OK;
}

// FP64 iterative refinement around FP32 Krylov solves of the correction.
ch_status PotentialSolver::solve_mixed(const double* n, const double* b, double* phi, SolveStats* st,
                                       cudaStream_t s) {
  const DevCoefs<double> C64 = dev_coefs<double>(c_);
  launch(k_down, nb_, 256, 0, s, N_, n, 1.0, n32_);
  MGHier<float>* mg = nullptr;
  if (p_.pc_type == CH_PC_MG) {
    ch_status rm = mg_build<float>(mg32_);
    if (rm) return rm;
    mg_update<float>(mg32_, n32_, s);
    mg = &mg32_;
  }
  remove_mean64(phi, s);
  const double bnorm = sqrt(dot64(b, b, s));
  st->bnorm = bnorm;
  const double tol = fmax(p_.ksp_rtol * bnorm, p_.ksp_atol);
  const double inner_rtol = 1e-4;
  int total = 0, ref = 0;
  double rn = 0.0;
  for (; ref < 50; ++ref) {
    launch(k_residual<double>, nb_, 256, 0, s, g_, C64, n, b, phi, r_, part_);
    launch(k_scalar, 1, 256, 0, s, part_, nb_, 1, OP_RR, scal_, 0.0);
    CH_CUDA_OK(cudaMemcpyAsync(hscal_ + S_RR, scal_ + S_RR, sizeof(double), cudaMemcpyDeviceToHost, s));
    CH_CUDA_OK(cudaStreamSynchronize(s));
    rn = sqrt(hscal_[S_RR]);
    if (rn <= tol || rn == 0.0) break;
    const double sc = 1.0 / rn;
    launch(k_down, nb_, 256, 0, s, N_, r_, sc, b32_);
    int its = 0;
    double rin = 0.0;
    // b32 = r / ||r|| has unit norm up to its FP32 rounding
    ch_status rc = krylov<float>(g_, n32_, b32_, x32_, inner_rtol, p_.ksp_max_it, true, &its, &rin, mg, s, 1.0);
    if (rc) return rc;
    total += its;
    launch(k_up_add, nb_, 256, 0, s, N_, x32_, rn, phi);
    remove_mean64(phi, s);
  }
  st->iterations = total;
  st->refinements = ref;
  st->rnorm = rn;
  if (rn > tol * 1.01 && rn > 0.0) return CH_ERR_NOT_CONVERGED;
  return CH_OK;
}

}  // namespace ch
