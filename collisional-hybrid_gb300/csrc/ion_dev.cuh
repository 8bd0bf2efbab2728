// ion_dev.cuh -- device helpers of the ion kernels shared by the pass, the
// ensemble and the adjoint: the fixed-point CIC deposit and the periodic wrap.
#pragma once

#include "common.cuh"

namespace ch {

__device__ __forceinline__ void red_add(unsigned long long* a, long long v) {
  atomicAdd(a, (unsigned long long)v);
}

template <typename R>
__device__ __forceinline__ long long to_fx(R v, R scale) {
  return __double2ll_rn((double)(v * scale));
}
template <>
__device__ __forceinline__ long long to_fx<float>(float v, float scale) {
  return __float2ll_rn(v * scale);
}

// Deposit one ion's CIC weights: nodes (i..i+1, j..j+1, k..k+1), weights in
// the order of src/particles.c:204-211.
template <typename R>
__device__ __forceinline__ void deposit_cic(const GridDesc& g, unsigned long long* __restrict__ acc, int i, int j,
                                            int k, R wxh, R wyh, R wzh, R vx, R vy, R vz, R scale) {
  const R wxl = R(1) - wxh, wyl = R(1) - wyh, wzl = R(1) - wzh;
  const int i1 = (i + 1 == g.Nx) ? 0 : i + 1;
  const int j1 = (j + 1 == g.Ny) ? 0 : j + 1;
  const int k1 = (k + 1 == g.Nz) ? 0 : k + 1;
  const int64_t N = g.N;
  const int64_t rz0 = (int64_t)k * g.Ny, rz1 = (int64_t)k1 * g.Ny;
  const int64_t c[8] = {(rz1 + j1) * g.Nx + i1, (rz0 + j1) * g.Nx + i1, (rz1 + j) * g.Nx + i1,
                        (rz0 + j) * g.Nx + i1,  (rz1 + j1) * g.Nx + i,  (rz0 + j1) * g.Nx + i,
                        (rz1 + j) * g.Nx + i,   (rz0 + j) * g.Nx + i};
  const R w[8] = {wzh * wyh * wxh, wzl * wyh * wxh, wzh * wyl * wxh, wzl * wyl * wxh,
                  wzh * wyh * wxl, wzl * wyh * wxl, wzh * wyl * wxl, wzl * wyl * wxl};
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    red_add(acc + c[q], to_fx<R>(w[q], scale));
    red_add(acc + N + c[q], to_fx<R>(vx * w[q], scale));
    red_add(acc + 2 * N + c[q], to_fx<R>(vy * w[q], scale));
    red_add(acc + 3 * N + c[q], to_fx<R>(vz * w[q], scale));
  }
}

// Deposit of one ion per lane with the contributions of lanes that share a
// cell summed across the warp before the global atomics: in cell-sorted
// order the ions of a cell sit in consecutive lanes, so a run of lanes
// issues 32 atomics instead of 32 per ion.  Runs start at a lane whose cell
// differs from its left neighbour's, so a cell that recurs later in the warp
// (an ion displaced since the sort) forms a run of its own.  Every
// contribution is rounded to fixed point before any sum, so the result is
// that of deposit_cic bit for bit.  All 32 lanes of the warp must call it;
// lanes without an ion pass active = false.
__device__ __forceinline__ void deposit_cic_warp(const GridDesc& g, unsigned long long* __restrict__ acc, bool active,
                                                 int i, int j, int k, double wxh, double wyh, double wzh, double vx,
                                                 double vy, double vz, double scale) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t key = active ? ((int64_t)k * g.Ny + j) * g.Nx + i : -1;
  const int64_t left = __shfl_up_sync(full, key, 1);
  const bool head = active && (lane == 0 || left != key);
  const unsigned heads = __ballot_sync(full, head);
  const unsigned upto = lane == 31 ? full : ((1u << (lane + 1)) - 1u);
  const int seg = (heads & upto) ? 31 - __clz(heads & upto) : -1;  // the run this lane belongs to
  int take_mask = 0;  // bit b: the lane 2^b to the right is in the same run
#pragma unroll
  for (int b = 0; b < 5; ++b) {
    const int off = 1 << b;
    const int oseg = __shfl_down_sync(full, seg, off);
    if (lane + off < 32 && oseg == seg) take_mask |= 1 << b;
  }
  const double wxl = 1.0 - wxh, wyl = 1.0 - wyh, wzl = 1.0 - wzh;
  const double w[8] = {wzh * wyh * wxh, wzl * wyh * wxh, wzh * wyl * wxh, wzl * wyl * wxh,
                       wzh * wyh * wxl, wzl * wyh * wxl, wzh * wyl * wxl, wzl * wyl * wxl};
  const int i1 = (i + 1 == g.Nx) ? 0 : i + 1;
  const int j1 = (j + 1 == g.Ny) ? 0 : j + 1;
  const int k1 = (k + 1 == g.Nz) ? 0 : k + 1;
  const int64_t N = g.N;
  const int64_t rz0 = (int64_t)k * g.Ny, rz1 = (int64_t)k1 * g.Ny;
  const int64_t c[8] = {(rz1 + j1) * g.Nx + i1, (rz0 + j1) * g.Nx + i1, (rz1 + j) * g.Nx + i1,
                        (rz0 + j) * g.Nx + i1,  (rz1 + j1) * g.Nx + i,  (rz0 + j1) * g.Nx + i,
                        (rz1 + j) * g.Nx + i,   (rz0 + j) * g.Nx + i};
  const double vm[4] = {1.0, vx, vy, vz};
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    long long a[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = active ? to_fx<double>(m == 0 ? w[q] : vm[m] * w[q], scale) : 0ll;
#pragma unroll
    for (int b = 0; b < 5; ++b) {
      const int off = 1 << b;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const long long o = __shfl_down_sync(full, a[q], off);
        if (take_mask & (1 << b)) a[q] += o;
      }
    }
    if (head) {
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (a[q] != 0) red_add(acc + m * N + c[q], a[q]);
    }
  }
}

// Periodic wrap of an absolute coordinate into [x0, x0 + L).
__device__ __forceinline__ double wrap_pos(double x, double x0, double L) {
  double u = x - x0;
  if (u < 0.0 || u >= L) u -= L * floor(u / L);
  if (u >= L) u -= L;
  if (u < 0.0) u = 0.0;
  return x0 + u;
}

}  // namespace ch
