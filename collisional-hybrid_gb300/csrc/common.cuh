// common.cuh -- shared device definitions of the hybrid-PIC hot path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "chybrid.h"

#define CH_PI 3.14159265358979323846

// Philox counter word 2 = purpose << 24 | block (same layout as the CPU oracle).
#define CH_PURPOSE_COLLIDE 1u
#define CH_PURPOSE_LOAD 2u
#define CH_STEP_LOADER 0xFFFFFFFFu

// Fixed-point scales of the order-independent (deterministic) reductions.
#define CH_SBAR_SCALE 16777216.0          // 2^24, sum of mean relative speeds
#define CH_EXPECT_SCALE 4294967296.0      // 2^32, sum of collision probabilities

// Packed cell of the mixed form: i | j << 11 | k << 22.
#define CH_PACK_BX 11
#define CH_PACK_BY 11
#define CH_MAX_NX 2048
#define CH_MAX_NY 2048
#define CH_MAX_NZ 1024

struct GridDesc {
  int Nx, Ny, Nz;
  int64_t N;
  double x0, y0, z0;
  double Lx, Ly, Lz;
  double dx, dy, dz;
  // exact division of node indices by Nx and Nx*Ny (see ch_ijk)
  uint32_t mx, sx1, sx2, mxy, sxy1, sxy2;
};

// Multiplier and shifts for the exact unsigned division n / d of any 32-bit
// n by a constant d (Granlund & Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994, Fig. 4.1): l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1, t = mulhi(m, n),
// n / d = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0).
__host__ inline void ch_magic(uint32_t d, uint32_t* m, uint32_t* s1, uint32_t* s2) {
  uint32_t l = 0;
  while (l < 32 && (1ull << l) < d) ++l;
  *m = (uint32_t)((((1ull << l) - d) << 32) / d + 1);
  *s1 = l < 1 ? l : 1;
  *s2 = l > 0 ? l - 1 : 0;
}
__device__ __forceinline__ uint32_t ch_divu(uint32_t n, uint32_t m, uint32_t s1, uint32_t s2) {
  const uint32_t t = __umulhi(m, n);
  return (t + ((n - t) >> s1)) >> s2;
}

// Node count and division constants of a grid whose Nx, Ny, Nz are set.
__host__ inline void ch_grid_finish(GridDesc& g) {
  g.N = (int64_t)g.Nx * g.Ny * g.Nz;
  ch_magic((uint32_t)g.Nx, &g.mx, &g.sx1, &g.sx2);
  ch_magic((uint32_t)g.Nx * (uint32_t)g.Ny, &g.mxy, &g.sxy1, &g.sxy2);
}

// (i, j, k) of natural index c (N < 2^32).
__device__ __forceinline__ void ch_ijk(const GridDesc& g, int64_t c, int& i, int& j, int& k) {
  const uint32_t u = (uint32_t)c;
  const uint32_t q = ch_divu(u, g.mx, g.sx1, g.sx2);
  const uint32_t r = ch_divu(u, g.mxy, g.sxy1, g.sxy2);
  i = (int)(u - q * (uint32_t)g.Nx);
  k = (int)r;
  j = (int)(q - r * (uint32_t)g.Ny);
}

// i mod n in [0, n); one compare for the usual |i| < 2n.
__host__ __device__ inline int ch_wrap(int i, int n) {
  if (i >= 0 && i < n) return i;
  if (i < 0 && i >= -n) return i + n;
  if (i >= n && i < 2 * n) return i - n;
  i %= n;
  return i < 0 ? i + n : i;
}

__host__ __device__ inline int64_t ch_nid(const GridDesc& g, int i, int j, int k) {
  return ((int64_t)ch_wrap(k, g.Nz) * g.Ny + ch_wrap(j, g.Ny)) * g.Nx + ch_wrap(i, g.Nx);
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper.
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 ch_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                        uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return U4{c0, c1, c2, c3};
}

// (r + 1/2) 2^-32: in (0, 1), exact in FP64.
__device__ __forceinline__ double ch_unit(uint32_t r) { return ((double)r + 0.5) * 2.3283064365386962890625e-10; }
// 24-bit FP32 variant: ((r >> 8) + 1/2) 2^-24, in (0, 1).
__device__ __forceinline__ float ch_unitf(uint32_t r) { return ((float)(r >> 8) + 0.5f) * 5.9604644775390625e-8f; }

// Run-wide constants of one particle pass.
struct StepConsts {
  GridDesc g;
  double tscale;        // (q/m) dt/2
  double t[3], s[3];    // Boris rotation vectors
  double E0[3];
  int push_E0;
  uint32_t faithful;
  double dt;
  // collisions
  int collide;
  double pscale;        // Nc / S
  double vnT, vn0[3], mi, mn, viTr, m1;
  int nn_profile;
  double nn_center, nn_sigma, nn_floor;
  uint32_t seed_lo, seed_hi, run, step;
  // deposit
  double dep_scale;     // fixed-point scale 2^s
  // FP32 copies of the constants above (ch_consts_finish), rounded once on
  // the host: the FP32 kernels read them as they are, so no FP64 arithmetic
  // or conversion (a slow pipe on this part) runs inside their loops
  struct {
    float dtx, dty, dtz;        // dt / dx: cells per unit velocity
    float t[3], s[3], pE0[3];   // pE0 = E0 tscale
    float vnT, vn0[3], mi, mn, viTr, m1;
    float nn_center, nn_sigma, nn_floor, dep_scale;
    float wi, wn;   // mi / (mi + mn), mn / (mi + mn): centre-of-mass weights
    float vlim2;    // (10 viTr)^2: the square of the refusal speed
  } f;
};

// Fills StepConsts::f from the FP64 fields; called after every change of them.
inline void ch_consts_finish(StepConsts& k) {
  k.f.dtx = (float)(k.dt / k.g.dx);
  k.f.dty = (float)(k.dt / k.g.dy);
  k.f.dtz = (float)(k.dt / k.g.dz);
  for (int d = 0; d < 3; ++d) {
    k.f.t[d] = (float)k.t[d];
    k.f.s[d] = (float)k.s[d];
    k.f.pE0[d] = (float)(k.E0[d] * k.tscale);
    k.f.vn0[d] = (float)k.vn0[d];
  }
  k.f.vnT = (float)k.vnT;
  k.f.mi = (float)k.mi;
  k.f.mn = (float)k.mn;
  k.f.viTr = (float)k.viTr;
  k.f.m1 = (float)k.m1;
  k.f.nn_center = (float)k.nn_center;
  k.f.nn_sigma = (float)k.nn_sigma;
  k.f.nn_floor = (float)k.nn_floor;
  k.f.dep_scale = (float)k.dep_scale;
  const double M = k.mi + k.mn;
  k.f.wi = M > 0.0 ? (float)(k.mi / M) : 0.0f;
  k.f.wn = M > 0.0 ? (float)(k.mn / M) : 0.0f;
  k.f.vlim2 = (float)(100.0 * k.viTr * k.viTr);
}

// The constant in the kernel's precision: the FP64 field, or its FP32 copy.
template <typename R>
__host__ __device__ __forceinline__ R ch_pick(double d, float f);
template <>
__host__ __device__ __forceinline__ double ch_pick<double>(double d, float) { return d; }
template <>
__host__ __device__ __forceinline__ float ch_pick<float>(double, float f) { return f; }

// Device-side counters; every sum is integer so the result does not depend
// on the order in which blocks finish.
struct DevCounters {
  unsigned long long collisions;
  unsigned long long refused;
  long long sbar_fx;
  long long expected_fx;
  int range_error;
  int pad;
};

#define CH_CUDA_OK(expr)                         \
  do {                                           \
    cudaError_t e_ = (expr);                     \
    if (e_ != cudaSuccess) return ch_cuda_fail(e_, #expr, __FILE__, __LINE__); \
  } while (0)

ch_status ch_cuda_fail(cudaError_t e, const char* what, const char* file, int line);

namespace ch {
// Counts kernel launches made by this library (reported by ch_get_profile);
// a CUDA graph launch counts the kernels it holds.
void note_launch();
void note_launch_n(long long n);
unsigned long long launches_now();
}
ch_status ch_fail(ch_status code, const char* fmt, ...);
