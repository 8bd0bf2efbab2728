// solver_dev.cuh -- device helpers of the matrix-free 19-point operator,
// shared by the single-run solver and the batched ensemble.
#pragma once

#include "solver.cuh"

namespace ch {

// ------------------------------------------------------------------ device helpers
struct Nb {
  int64_t c, e, w, n, s, u, d;       // centre and faces (x+, x-, y+, y-, z+, z-)
  int64_t en, es, wn, ws, eu, ed, wu, wd, nu, nd, su, sd;  // 12 edges
};

__device__ __forceinline__ Nb neighbours(const GridDesc& g, int64_t c) {
  int i, j, k;
  ch_ijk(g, c, i, j, k);
  const int ip = i + 1 == g.Nx ? 0 : i + 1, im = i == 0 ? g.Nx - 1 : i - 1;
  const int jp = j + 1 == g.Ny ? 0 : j + 1, jm = j == 0 ? g.Ny - 1 : j - 1;
  const int kp = k + 1 == g.Nz ? 0 : k + 1, km = k == 0 ? g.Nz - 1 : k - 1;
  const int64_t X = g.Nx, XY = (int64_t)g.Nx * g.Ny;
  const int64_t r0 = k * XY, rp = kp * XY, rm = km * XY;
  const int64_t y0 = j * X, yp = jp * X, ym = jm * X;
  Nb b;
  b.c = r0 + y0 + i;
  b.e = r0 + y0 + ip; b.w = r0 + y0 + im;
  b.n = r0 + yp + i;  b.s = r0 + ym + i;
  b.u = rp + y0 + i;  b.d = rm + y0 + i;
  b.en = r0 + yp + ip; b.es = r0 + ym + ip; b.wn = r0 + yp + im; b.ws = r0 + ym + im;
  b.eu = rp + y0 + ip; b.ed = rm + y0 + ip; b.wu = rp + y0 + im; b.wd = rm + y0 + im;
  b.nu = rp + yp + i;  b.nd = rm + yp + i;  b.su = rp + ym + i;  b.sd = rm + ym + i;
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
// and src/lhs.c:7-106 (stencil order).
template <typename T>
__device__ __forceinline__ T apply_row(const DevCoefs<T>& C, const T* n, const T* x, const Nb& b) {
  if (C.type == CH_LHS_IDENTITY) return x[b.c];
  const T xc = x[b.c];
  if (C.type == CH_LHS_LAPLACIAN)
    return C.sxx * (x[b.e] + x[b.w]) + C.syy * (x[b.n] + x[b.s]) + C.szz * (x[b.u] + x[b.d]) -
           T(2) * (C.sxx + C.syy + C.szz) * xc;
  const T nijk = n[b.c], npjk = n[b.e], nmjk = n[b.w], nipk = n[b.n], nimk = n[b.s], nijp = n[b.u], nijm = n[b.d];
  // star terms: sum of f_face (x_face - x_c) over the six faces reproduces
  // the diagonal value -(sum of the star values) exactly in exact arithmetic
  T acc = C.sxx * ((npjk + nijk) * (x[b.e] - xc) + (nijk + nmjk) * (x[b.w] - xc)) +
          C.syy * ((nipk + nijk) * (x[b.n] - xc) + (nijk + nimk) * (x[b.s] - xc)) +
          C.szz * ((nijp + nijk) * (x[b.u] - xc) + (nijk + nijm) * (x[b.d] - xc));
  if (C.cross) {
    const T sxy = C.sxy, sxz = C.sxz, syz = C.syz, syx = C.syx, szx = C.szx, szy = C.szy;
    // cross parts of the six star values
    acc += (syx * (nipk - nimk) + szx * (nijp - nijm)) * (x[b.e] - x[b.w]);
    acc += (sxy * (npjk - nmjk) + szy * (nijp - nijm)) * (x[b.n] - x[b.s]);
    acc += (sxz * (npjk - nmjk) + syz * (nipk - nimk)) * (x[b.u] - x[b.d]);
    // x-y corners
    acc += (sxy * (npjk + nijk) + syx * (nipk + nijk)) * x[b.en];
    acc += (-sxy * (npjk + nijk) - syx * (nijk + nimk)) * x[b.es];
    acc += (-sxy * (nijk + nmjk) - syx * (nipk + nijk)) * x[b.wn];
    acc += (sxy * (nijk + nmjk) + syx * (nijk + nimk)) * x[b.ws];
    // x-z corners
    acc += (sxz * (npjk + nijk) + szx * (nijp + nijk)) * x[b.eu];
    acc += (-sxz * (npjk + nijk) - szx * (nijk + nijm)) * x[b.ed];
    acc += (-sxz * (nijk + nmjk) - szx * (nijp + nijk)) * x[b.wu];
    acc += (sxz * (nijk + nmjk) + szx * (nijk + nijm)) * x[b.wd];
    // y-z corners
    acc += (syz * (nipk + nijk) + szy * (nijp + nijk)) * x[b.nu];
    acc += (-syz * (nipk + nijk) - szy * (nijk + nijm)) * x[b.nd];
    acc += (-syz * (nijk + nimk) - szy * (nijp + nijk)) * x[b.su];
    acc += (syz * (nijk + nimk) + szy * (nijk + nijm)) * x[b.sd];
  }
  return acc;
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
// d8 selects the as-written d2Fdyz (x-z stencil, src/calculus.c:464).
struct RhsCoefs {
  double R[9];
  double det;
  double E0[3];
  double cth, cG;
  int d8;
};
__device__ __forceinline__ double rhs_full_row(const GridDesc& g, const RhsCoefs& K, const double* n, const double* Gx,
                                               const double* Gy, const double* Gz, const Nb& q) {
  const double dx = g.dx, dy = g.dy, dz = g.dz;
  const double dndx = (n[q.e] - n[q.w]) / (2.0 * dx);
  const double dndy = (n[q.n] - n[q.s]) / (2.0 * dy);
  const double dndz = (n[q.u] - n[q.d]) / (2.0 * dz);
  const double dGxdx = (Gx[q.e] - Gx[q.w]) / (2.0 * dx);
  const double dGydy = (Gy[q.n] - Gy[q.s]) / (2.0 * dy);
  const double dGzdz = (Gz[q.u] - Gz[q.d]) / (2.0 * dz);
  const double d2ndxx = (n[q.e] - 2.0 * n[q.c] + n[q.w]) / (dx * dx);
  const double d2ndyy = (n[q.n] - 2.0 * n[q.c] + n[q.s]) / (dy * dy);
  const double d2ndzz = (n[q.u] - 2.0 * n[q.c] + n[q.d]) / (dz * dz);
  const double d2ndxy = (n[q.en] - n[q.wn] - n[q.es] + n[q.ws]) / (4.0 * dx * dy);
  const double d2ndxz = (n[q.eu] - n[q.wu] - n[q.ed] + n[q.wd]) / (4.0 * dx * dz);
  const double vyz = K.d8 ? (n[q.eu] - n[q.wu] - n[q.ed] + n[q.wd]) : (n[q.nu] - n[q.su] - n[q.nd] + n[q.sd]);
  const double d2ndyz = vyz / (4.0 * dy * dz);
  const double* R = K.R;
  const double Eterm = (R[0] * K.E0[0] + R[1] * K.E0[1] + R[2] * K.E0[2]) * dndx +
                       (R[3] * K.E0[0] + R[4] * K.E0[1] + R[5] * K.E0[2]) * dndy +
                       (R[6] * K.E0[0] + R[7] * K.E0[1] + R[8] * K.E0[2]) * dndz;
  const double Pterm = K.cth * (R[0] * d2ndxx + R[1] * d2ndxy + R[2] * d2ndxz + R[3] * d2ndxy + R[4] * d2ndyy +
                                R[5] * d2ndyz + R[6] * d2ndxz + R[7] * d2ndyz + R[8] * d2ndzz);
  const double Gterm = K.det * K.cG * (dGxdx + dGydy + dGzdz);
  return (1.0 / K.det) * (Eterm + Pterm + Gterm);
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
