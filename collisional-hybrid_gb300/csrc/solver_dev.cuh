// solver_dev.cuh -- device helpers of the matrix-free 19-point operator,
// shared by the single-run solver and the batched ensemble.
#pragma once

#include "solver.cuh"

namespace ch {

// ------------------------------------------------------------------ device helpers
// Node indices of the 19-point stencil around a node.  Every grid has fewer
// than 2^31 nodes, so the indices are 32-bit: each is the centre plus a sum
// of per-axis steps, the periodic wrap folded into the step.
struct Nb {
  int c, e, w, n, s, u, d;       // centre and faces (x+, x-, y+, y-, z+, z-)
  int en, es, wn, ws, eu, ed, wu, wd, nu, nd, su, sd;  // 12 edges
};

__device__ __forceinline__ Nb neighbours(const GridDesc& g, int64_t c64) {
  int i, j, k;
  ch_ijk(g, c64, i, j, k);
  const int X = g.Nx, XY = g.Nx * g.Ny;
  const int xp = i + 1 == g.Nx ? 1 - X : 1, xm = i == 0 ? X - 1 : -1;
  const int yp = j + 1 == g.Ny ? X - XY : X, ym = j == 0 ? XY - X : -X;
  const int zp = k + 1 == g.Nz ? XY - (int)g.N : XY, zm = k == 0 ? (int)g.N - XY : -XY;
  Nb b;
  b.c = (int)c64;
  b.e = b.c + xp; b.w = b.c + xm;
  b.n = b.c + yp; b.s = b.c + ym;
  b.u = b.c + zp; b.d = b.c + zm;
  b.en = b.e + yp; b.es = b.e + ym; b.wn = b.w + yp; b.ws = b.w + ym;
  b.eu = b.e + zp; b.ed = b.e + zm; b.wu = b.w + zp; b.wd = b.w + zm;
  b.nu = b.n + zp; b.nd = b.n + zm; b.su = b.s + zp; b.sd = b.s + zm;
  return b;
}

template <typename T>
DevCoefs<T> dev_coefs(const OpCoefs& c) {
  DevCoefs<T> d;
  d.sxx = (T)c.sxx; d.syy = (T)c.syy; d.szz = (T)c.szz;
  d.sxy = (T)c.sxy; d.sxz = (T)c.sxz; d.syz = (T)c.syz;
  d.syx = (T)c.syx; d.szx = (T)c.szx; d.szy = (T)c.szy;
  d.type = c.type;
  d.cross = (c.sxy != 0 || c.sxz != 0 || c.syz != 0 || c.syx != 0 || c.szx != 0 || c.szy != 0);
  return d;
}

// One row of A(n) x.  Values follow src/lhs.c:488-511 (f[...] assignments)
// and src/lhs.c:7-106 (stencil order).  xat(i) gives x at node i (an array
// read, or a value formed on the fly).
template <typename T, typename X>
__device__ __forceinline__ T apply_row_at(const DevCoefs<T>& C, const T* n, X xat, const Nb& b) {
  if (C.type == CH_LHS_IDENTITY) return xat(b.c);
  const T xc = xat(b.c), xe = xat(b.e), xw = xat(b.w), xn = xat(b.n), xs = xat(b.s), xu = xat(b.u), xd = xat(b.d);
  if (C.type == CH_LHS_LAPLACIAN)
    return C.sxx * (xe + xw) + C.syy * (xn + xs) + C.szz * (xu + xd) - T(2) * (C.sxx + C.syy + C.szz) * xc;
  const T nijk = n[b.c], npjk = n[b.e], nmjk = n[b.w], nipk = n[b.n], nimk = n[b.s], nijp = n[b.u], nijm = n[b.d];
  // star terms: sum of f_face (x_face - x_c) over the six faces reproduces
  // the diagonal value -(sum of the star values) exactly in exact arithmetic
  T acc = C.sxx * ((npjk + nijk) * (xe - xc) + (nijk + nmjk) * (xw - xc)) +
          C.syy * ((nipk + nijk) * (xn - xc) + (nijk + nimk) * (xs - xc)) +
          C.szz * ((nijp + nijk) * (xu - xc) + (nijk + nijm) * (xd - xc));
  if (C.cross) {
    const T sxy = C.sxy, sxz = C.sxz, syz = C.syz, syx = C.syx, szx = C.szx, szy = C.szy;
    // cross parts of the six star values
    acc += (syx * (nipk - nimk) + szx * (nijp - nijm)) * (xe - xw);
    acc += (sxy * (npjk - nmjk) + szy * (nijp - nijm)) * (xn - xs);
    acc += (sxz * (npjk - nmjk) + syz * (nipk - nimk)) * (xu - xd);
    // x-y corners
    acc += (sxy * (npjk + nijk) + syx * (nipk + nijk)) * xat(b.en);
    acc += (-sxy * (npjk + nijk) - syx * (nijk + nimk)) * xat(b.es);
    acc += (-sxy * (nijk + nmjk) - syx * (nipk + nijk)) * xat(b.wn);
    acc += (sxy * (nijk + nmjk) + syx * (nijk + nimk)) * xat(b.ws);
    // x-z corners
    acc += (sxz * (npjk + nijk) + szx * (nijp + nijk)) * xat(b.eu);
    acc += (-sxz * (npjk + nijk) - szx * (nijk + nijm)) * xat(b.ed);
    acc += (-sxz * (nijk + nmjk) - szx * (nijp + nijk)) * xat(b.wu);
    acc += (sxz * (nijk + nmjk) + szx * (nijk + nijm)) * xat(b.wd);
    // y-z corners
    acc += (syz * (nipk + nijk) + szy * (nijp + nijk)) * xat(b.nu);
    acc += (-syz * (nipk + nijk) - szy * (nijk + nijm)) * xat(b.nd);
    acc += (-syz * (nijk + nimk) - szy * (nijp + nijk)) * xat(b.su);
    acc += (syz * (nijk + nimk) + szy * (nijk + nijm)) * xat(b.sd);
  }
  return acc;
}
template <typename T>
__device__ __forceinline__ T apply_row(const DevCoefs<T>& C, const T* n, const T* x, const Nb& b) {
  return apply_row_at<T>(C, n, [x](int64_t i) { return x[i]; }, b);
}

template <typename T>
__device__ __forceinline__ T diag_row(const DevCoefs<T>& C, const T* n, const Nb& b) {
  if (C.type == CH_LHS_IDENTITY) return T(1);
  if (C.type == CH_LHS_LAPLACIAN) return -T(2) * (C.sxx + C.syy + C.szz);
  const T nijk = n[b.c];
  return -(C.sxx * (n[b.e] + T(2) * nijk + n[b.w]) + C.syy * (n[b.n] + T(2) * nijk + n[b.s]) +
           C.szz * (n[b.u] + T(2) * nijk + n[b.d]));
}

// ComputeFullRHS at one node (src/rhs.c:133-303, src/calculus.c:21-520):
// b = (1/det)[(R E0).grad n + c_th sum R_ab d_a d_b n + det c_G div Gamma].
// The differences of n and Gamma are formed as the reference forms them;
// every constant factor (1/(2 dx), 1/dx^2, 1/det, R, E0, c_th, c_G) is folded
// on the host into one coefficient per difference (rhs_coefs), so the row is
// a dozen FP64 products and no divisions.  d8 selects the as-written d2Fdyz
// (x-z stencil, src/calculus.c:464).
struct RhsCoefs {
  double ex, ey, ez;     // (R E0)_a / (2 d_a det)
  double pxx, pyy, pzz;  // c_th R_aa / (d_a^2 det)
  double pxy, pxz, pyz;  // c_th (R_ab + R_ba) / (4 d_a d_b det)
  double gx, gy, gz;     // c_G / (2 d_a)
  int d8;
};
inline RhsCoefs rhs_coefs(const double R[9], double det, const double E0[3], double cth, double cG, bool d8,
                          double dx, double dy, double dz) {
  RhsCoefs K;
  const double a[3] = {R[0] * E0[0] + R[1] * E0[1] + R[2] * E0[2], R[3] * E0[0] + R[4] * E0[1] + R[5] * E0[2],
                       R[6] * E0[0] + R[7] * E0[1] + R[8] * E0[2]};
  K.ex = a[0] / (2.0 * dx * det);
  K.ey = a[1] / (2.0 * dy * det);
  K.ez = a[2] / (2.0 * dz * det);
  K.pxx = cth * R[0] / (dx * dx * det);
  K.pyy = cth * R[4] / (dy * dy * det);
  K.pzz = cth * R[8] / (dz * dz * det);
  K.pxy = cth * (R[1] + R[3]) / (4.0 * dx * dy * det);
  K.pxz = cth * (R[2] + R[6]) / (4.0 * dx * dz * det);
  K.pyz = cth * (R[5] + R[7]) / (4.0 * dy * dz * det);
  K.gx = cG / (2.0 * dx);
  K.gy = cG / (2.0 * dy);
  K.gz = cG / (2.0 * dz);
  K.d8 = d8 ? 1 : 0;
  return K;
}
__device__ __forceinline__ double rhs_full_row(const GridDesc& g, const RhsCoefs& K, const double* n, const double* Gx,
                                               const double* Gy, const double* Gz, const Nb& q) {
  (void)g;
  const double dnx = n[q.e] - n[q.w], dny = n[q.n] - n[q.s], dnz = n[q.u] - n[q.d];
  const double lxx = n[q.e] - 2.0 * n[q.c] + n[q.w];
  const double lyy = n[q.n] - 2.0 * n[q.c] + n[q.s];
  const double lzz = n[q.u] - 2.0 * n[q.c] + n[q.d];
  const double lxy = n[q.en] - n[q.wn] - n[q.es] + n[q.ws];
  const double lxz = n[q.eu] - n[q.wu] - n[q.ed] + n[q.wd];
  const double lyz = K.d8 ? lxz : (n[q.nu] - n[q.su] - n[q.nd] + n[q.sd]);
  return K.ex * dnx + K.ey * dny + K.ez * dnz + K.pxx * lxx + K.pyy * lyy + K.pzz * lzz + K.pxy * lxy +
         K.pxz * lxz + K.pyz * lyz + K.gx * (Gx[q.e] - Gx[q.w]) + K.gy * (Gy[q.n] - Gy[q.s]) +
         K.gz * (Gz[q.u] - Gz[q.d]);
}

// Block partial sums of K doubles (fixed order).
template <int K>
__device__ __forceinline__ void partials(double (&v)[K], double* __restrict__ part) {
  __shared__ double sm[K][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sm[q][wid] = x;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      double x = lane < nw ? sm[q][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) part[(size_t)blockIdx.x * K + q] = x;
    }
  }
}


}  // namespace ch
