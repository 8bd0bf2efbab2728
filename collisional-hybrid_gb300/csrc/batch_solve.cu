// batch_solve.cu -- the potential solves of an ensemble in one launch.
//
// Each run of the ensemble is solved by one thread-block cluster: its CTAs
// split the run's nodes into contiguous ranges, synchronise with the
// hardware cluster barrier (release/acquire at cluster scope, so global
// writes before a barrier are visible to every CTA of the cluster after it)
// and form dot products from per-CTA partials read through distributed
// shared memory in rank order, so every CTA holds bitwise the same scalars
// and takes the same branches.  Runs of different sizes finish
// independently; nothing waits on another cluster.
//
// The algorithm is the mixed form of the single-run solver: the full RHS
// (src/rhs.c:133-303) with its mean removed, FP64 iterative refinement of phi
// around an FP32 CG preconditioned by one geometric-multigrid V(2,2) cycle,
// and at the end the node field -grad(phi) (q/m) dt/2 of the next push.
//
// Loads of data written inside the kernel are plain loads (never the
// read-only path), because other CTAs of the cluster write them.
#include <cooperative_groups.h>

#include <atomic>

#include "batch.cuh"

namespace cg = cooperative_groups;

namespace ch {

namespace {

constexpr float B_OMEGA = 0.8f;      // damped-Jacobi weight of the smoother
constexpr int B_COARSE_SWEEPS_MAX = 64;  // Jacobi sweeps of the coarsest level: 4 per node of its longest edge
constexpr double B_INNER_RTOL = 1e-4;
constexpr int B_MAX_REFINE = 50;
constexpr int B_MAX_INNER = 200;     // inner iterations per refinement (rtol 1e-4 takes ~10)

struct ClusterRed {
  double part[2][4];  // this CTA's partials, two alternating sets
  double warp[8][4];
  double out[4];
};

struct SolveShared {
  ClusterRed red;
  float xa[BATCH_COARSE_MAX];
  float xb[BATCH_COARSE_MAX];
};

// Cluster-wide sums of K doubles (K <= 4): block sum in a fixed order, then
// the CTAs' partials added in rank order.  One cluster barrier.
template <int K>
__device__ __forceinline__ void csum(cg::cluster_group& cl, SolveShared& sh, int& set, double (&v)[K]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh.red.warp[wid][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double x = 0.0;
    for (int w = 0; w < nw; ++w) x += sh.red.warp[w][threadIdx.x];
    sh.red.part[set][threadIdx.x] = x;
  }
  cl.sync();
  if (threadIdx.x < K) {
    double x = 0.0;
    const int C = (int)cl.num_blocks();
    for (int rk = 0; rk < C; ++rk) x += cl.map_shared_rank(&sh.red.part[set][0], rk)[threadIdx.x];
    sh.red.out[threadIdx.x] = x;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < K; ++q) v[q] = sh.red.out[q];
  set ^= 1;
}

__device__ __forceinline__ void own_range(int64_t N, int rank, int C, int64_t* lo, int64_t* hi) {
  *lo = N * rank / C;
  *hi = N * (rank + 1) / C;
}

#define OWN(c, N)                                  \
  int64_t lo_##c, hi_##c;                          \
  own_range((N), rank, C, &lo_##c, &hi_##c);       \
  for (int64_t c = lo_##c + threadIdx.x; c < hi_##c; c += blockDim.x)

// Full weighting (see k_restrict) of fine vector `in` at coarse node c.
__device__ __forceinline__ float restrict_at(const GridDesc& gf, const GridDesc& gc, int hx, int hy, int hz,
                                             const float* in, int64_t c) {
  int I, J, K;
  ch_ijk(gc, c, I, J, K);
  const int i0 = hx ? 2 * I : I, j0 = hy ? 2 * J : J, k0 = hz ? 2 * K : K;
  float acc = 0.0f;
  for (int dk = -hz; dk <= hz; ++dk) {
    const float wk = hz ? (dk == 0 ? 0.5f : 0.25f) : 1.0f;
    const int k = ch_wrap(k0 + dk, gf.Nz);
    for (int dj = -hy; dj <= hy; ++dj) {
      const float wj = hy ? (dj == 0 ? 0.5f : 0.25f) : 1.0f;
      const int j = ch_wrap(j0 + dj, gf.Ny);
      const int64_t row = ((int64_t)k * gf.Ny + j) * gf.Nx;
      for (int di = -hx; di <= hx; ++di) {
        const float wi = hx ? (di == 0 ? 0.5f : 0.25f) : 1.0f;
        acc += wk * wj * wi * in[row + ch_wrap(i0 + di, gf.Nx)];
      }
    }
  }
  return acc;
}

// Trilinear prolongation (see k_prolong_add) of coarse `ec` at fine node c.
__device__ __forceinline__ float prolong_at(const GridDesc& gf, const GridDesc& gc, int hx, int hy, int hz,
                                            const float* ec, int64_t c) {
  int i, j, k;
  ch_ijk(gf, c, i, j, k);
  int I0, I1, J0, J1, K0, K1;
  float wi1, wj1, wk1;
  if (hx) { I0 = i >> 1; I1 = (i & 1) ? ch_wrap(I0 + 1, gc.Nx) : I0; wi1 = (i & 1) ? 0.5f : 0.0f; }
  else { I0 = I1 = i; wi1 = 0.0f; }
  if (hy) { J0 = j >> 1; J1 = (j & 1) ? ch_wrap(J0 + 1, gc.Ny) : J0; wj1 = (j & 1) ? 0.5f : 0.0f; }
  else { J0 = J1 = j; wj1 = 0.0f; }
  if (hz) { K0 = k >> 1; K1 = (k & 1) ? ch_wrap(K0 + 1, gc.Nz) : K0; wk1 = (k & 1) ? 0.5f : 0.0f; }
  else { K0 = K1 = k; wk1 = 0.0f; }
  const float wi0 = 1.0f - wi1, wj0 = 1.0f - wj1, wk0 = 1.0f - wk1;
  auto at = [&](int I, int J, int K) { return ec[((int64_t)K * gc.Ny + J) * gc.Nx + I]; };
  return wk0 * (wj0 * (wi0 * at(I0, J0, K0) + wi1 * at(I1, J0, K0)) +
                wj1 * (wi0 * at(I0, J1, K0) + wi1 * at(I1, J1, K0))) +
         wk1 * (wj0 * (wi0 * at(I0, J0, K1) + wi1 * at(I1, J0, K1)) +
                wj1 * (wi0 * at(I0, J1, K1) + wi1 * at(I1, J1, K1)));
}

}  // namespace

__global__ void __launch_bounds__(256) k_batch_solve(const BSolveRun* runs) {
  __shared__ SolveShared sh;
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const BSolveRun& R = runs[blockIdx.x / C];
  const GridDesc& g = R.g;
  const int64_t N = g.N;
  const int L = R.L;
  int set = 0;
  int flags = 0;
  const float w = B_OMEGA;

  // ---- RHS (FP64) with its mean removed; FP32 density of level 0
  const double* n64 = R.mom;
  double bnorm = 0.0;
  {
    double s[1] = {0.0};
    float* n32 = R.lv[0].n;
    OWN(c, N) {
      const double b = rhs_full_row(g, R.K, n64, n64 + N, n64 + 2 * N, n64 + 3 * N, neighbours(g, c));
      R.b64[c] = b;
      s[0] += b;
      const double nv = n64[c];
      if (!(nv >= 0.0)) flags |= 1;  // negative (wrapped) or non-finite density
      n32[c] = (float)nv;
    }
    csum<1>(cl, sh, set, s);
    const double mean = s[0] / (double)N;
    double bb[1] = {0.0};
    OWN(c2, N) {
      const double b = R.b64[c2] - mean;
      R.b64[c2] = b;
      bb[0] += b * b;
    }
    csum<1>(cl, sh, set, bb);  // also orders the n32 writes before the restriction
    bnorm = sqrt(bb[0]);
  }
  // ---- density hierarchy and Jacobi diagonals
  OWN(c, N) {
    const float d = diag_row<float>(R.lv[0].C, R.lv[0].n, neighbours(g, c));
    R.lv[0].dinv[c] = d != 0.0f ? 1.0f / d : 1.0f;
  }
  for (int l = 1; l < L; ++l) {
    const BLevel& F = R.lv[l - 1];
    const BLevel& Q = R.lv[l];
    OWN(c, Q.g.N) Q.n[c] = restrict_at(F.g, Q.g, F.hx, F.hy, F.hz, F.n, c);
    cl.sync();
    OWN(c2, Q.g.N) {
      const float d = diag_row<float>(Q.C, Q.n, neighbours(Q.g, c2));
      Q.dinv[c2] = d != 0.0f ? 1.0f / d : 1.0f;
    }
  }
  // ---- warm start: phi with its mean removed
  {
    double s[1] = {0.0};
    OWN(c, N) s[0] += R.phi[c];
    csum<1>(cl, sh, set, s);
    const double mean = s[0] / (double)N;
    OWN(c2, N) R.phi[c2] -= mean;
    cl.sync();  // phi and every level's diagonal are complete
  }

  // One V(2,2) cycle from zero: x0 ~= A^{-1} b0 on level 0.
  auto vcycle = [&](const float* b0, float* x0) {
    for (int l = 0; l < L - 1; ++l) {
      const BLevel& V = R.lv[l];
      const float* b = l ? V.b : b0;
      float* x = l ? V.x : x0;
      OWN(c, V.g.N) V.t[c] = w * V.dinv[c] * b[c];
      cl.sync();
      OWN(c2, V.g.N) x[c2] = V.t[c2] + w * V.dinv[c2] * (b[c2] - apply_row<float>(V.C, V.n, V.t, neighbours(V.g, c2)));
      cl.sync();
      OWN(c3, V.g.N) V.r[c3] = b[c3] - apply_row<float>(V.C, V.n, x, neighbours(V.g, c3));
      cl.sync();
      const BLevel& Q = R.lv[l + 1];
      OWN(c4, Q.g.N) Q.b[c4] = V.sR * restrict_at(V.g, Q.g, V.hx, V.hy, V.hz, V.r, c4);
      cl.sync();
    }
    {
      // coarsest level: every CTA runs the same sweeps in its shared memory
      // and writes its own range
      const BLevel& V = R.lv[L - 1];
      const float* b = L > 1 ? V.b : b0;
      float* x = L > 1 ? V.x : x0;
      const int Nc = (int)V.g.N;
      float* xa = sh.xa;
      float* xb = sh.xb;
      for (int c = threadIdx.x; c < Nc; c += blockDim.x) xa[c] = w * V.dinv[c] * b[c];
      __syncthreads();
      const int emax = max(V.g.Nx, max(V.g.Ny, V.g.Nz));
      const int sweeps = min(B_COARSE_SWEEPS_MAX, max(16, 4 * emax));
      for (int sw = 1; sw < sweeps; ++sw) {
        for (int c = threadIdx.x; c < Nc; c += blockDim.x)
          xb[c] = xa[c] + w * V.dinv[c] * (b[c] - apply_row<float>(V.C, V.n, xa, neighbours(V.g, c)));
        __syncthreads();
        float* t = xa; xa = xb; xb = t;
      }
      OWN(c, (int64_t)Nc) x[c] = xa[c];
      cl.sync();
    }
    for (int l = L - 2; l >= 0; --l) {
      const BLevel& V = R.lv[l];
      const BLevel& Q = R.lv[l + 1];
      const float* b = l ? V.b : b0;
      float* x = l ? V.x : x0;
      OWN(c, V.g.N) x[c] += prolong_at(V.g, Q.g, V.hx, V.hy, V.hz, Q.x, c);
      cl.sync();
      OWN(c2, V.g.N) V.t[c2] = x[c2] + w * V.dinv[c2] * (b[c2] - apply_row<float>(V.C, V.n, x, neighbours(V.g, c2)));
      cl.sync();
      OWN(c3, V.g.N) x[c3] = V.t[c3] + w * V.dinv[c3] * (b[c3] - apply_row<float>(V.C, V.n, V.t, neighbours(V.g, c3)));
      cl.sync();
    }
  };

  // ---- FP64 iterative refinement around FP32 MG-PCG
  const double tol = fmax(R.rtol * bnorm, R.atol);
  const BLevel& V0 = R.lv[0];
  int total = 0, ref = 0;
  double rn = 0.0;
  for (; ref < B_MAX_REFINE; ++ref) {
    double rr[1] = {0.0};
    OWN(c, N) {
      const double r = R.b64[c] - apply_row<double>(R.C64, n64, R.phi, neighbours(g, c));
      R.r64[c] = r;
      rr[0] += r * r;
    }
    csum<1>(cl, sh, set, rr);
    rn = sqrt(rr[0]);
    if (!(rn > tol) || rn == 0.0) break;
    const double sc = 1.0 / rn;
    OWN(c2, N) {
      const float b = (float)(R.r64[c2] * sc);
      R.b32[c2] = b;
      R.r32[c2] = b;
      R.x32[c2] = 0.0f;
    }
    cl.sync();
    // z = M r, rz = (r, z), bb = (b, b)
    vcycle(R.r32, R.z32);
    double d2[2] = {0.0, 0.0};
    OWN(c3, N) {
      const double r = R.r32[c3];
      d2[0] += r * (double)R.z32[c3];
      d2[1] += r * r;
    }
    csum<2>(cl, sh, set, d2);
    double rz = d2[0];
    const double itol = B_INNER_RTOL * sqrt(d2[1]);
    int its = 0;
    if (sqrt(d2[1]) > itol) {
      OWN(c4, N) R.p32[c4] = R.z32[c4];
      cl.sync();
      const int maxit = R.maxit < B_MAX_INNER ? R.maxit : B_MAX_INNER;
      for (; its < maxit;) {
        double pq[1] = {0.0};
        OWN(c5, N) {
          const float q = apply_row<float>(V0.C, V0.n, R.p32, neighbours(g, c5));
          R.q32[c5] = q;
          pq[0] += (double)R.p32[c5] * (double)q;
        }
        csum<1>(cl, sh, set, pq);
        const float alpha = pq[0] != 0.0 ? (float)(rz / pq[0]) : 0.0f;
        double r2[1] = {0.0};
        OWN(c6, N) {
          R.x32[c6] += alpha * R.p32[c6];
          const float r = R.r32[c6] - alpha * R.q32[c6];
          R.r32[c6] = r;
          r2[0] += (double)r * (double)r;
        }
        csum<1>(cl, sh, set, r2);
        ++its;
        if (!(sqrt(r2[0]) > itol)) break;
        vcycle(R.r32, R.z32);
        double rzn[1] = {0.0};
        OWN(c7, N) rzn[0] += (double)R.r32[c7] * (double)R.z32[c7];
        csum<1>(cl, sh, set, rzn);
        const float beta = rz != 0.0 ? (float)(rzn[0] / rz) : 0.0f;
        rz = rzn[0];
        OWN(c8, N) R.p32[c8] = R.z32[c8] + beta * R.p32[c8];
        cl.sync();
      }
    }
    total += its;
    // phi += rn x, mean removed
    double s[1] = {0.0};
    OWN(c9, N) {
      const double v = R.phi[c9] + rn * (double)R.x32[c9];
      R.phi[c9] = v;
      s[0] += v;
    }
    csum<1>(cl, sh, set, s);
    const double mean = s[0] / (double)N;
    OWN(c10, N) R.phi[c10] -= mean;
    cl.sync();
  }
  if (!(rn <= tol * 1.01) && rn > 0.0) flags |= 2;
  if (!isfinite(rn)) flags |= 4;
  // ---- node field of the next push, premultiplied by (q/m) dt/2: one FP64
  // difference and one product per component (as k_node_efield_mixed)
  const double esx = -R.tscale / (2.0 * g.dx), esy = -R.tscale / (2.0 * g.dy), esz = -R.tscale / (2.0 * g.dz);
  OWN(ce, N) {
    const int64_t c = ce;
    int i, j, k;
    ch_ijk(g, c, i, j, k);
    const int ip = i + 1 == g.Nx ? 0 : i + 1, im = i == 0 ? g.Nx - 1 : i - 1;
    const int jp = j + 1 == g.Ny ? 0 : j + 1, jm = j == 0 ? g.Ny - 1 : j - 1;
    const int kp = k + 1 == g.Nz ? 0 : k + 1, km = k == 0 ? g.Nz - 1 : k - 1;
    const int64_t row = ((int64_t)k * g.Ny + j) * g.Nx;
    const double dx = R.phi[row + ip] - R.phi[row + im];
    const double dy = R.phi[((int64_t)k * g.Ny + jp) * g.Nx + i] - R.phi[((int64_t)k * g.Ny + jm) * g.Nx + i];
    const double dz = R.phi[((int64_t)kp * g.Ny + j) * g.Nx + i] - R.phi[((int64_t)km * g.Ny + j) * g.Nx + i];
    R.E32[c] = make_float4((float)(dx * esx), (float)(dy * esy), (float)(dz * esz), 0.0f);
  }
  // ---- status (flags gathered from every CTA)
  double fl[1] = {(double)(flags & 1)};
  csum<1>(cl, sh, set, fl);
  if (rank == 0 && threadIdx.x == 0) {
    const int f = (fl[0] > 0.0 ? 1 : 0) | (flags & 6);
    R.out->iterations = total;
    R.out->refinements = ref;
    R.out->rnorm = rn;
    R.out->bnorm = bnorm;
    R.out->flags = f;
    R.out->status = (f & 5) ? (int)CH_ERR_NAN : (f & 2) ? (int)CH_ERR_NOT_CONVERGED : (int)CH_OK;
  }
  // no CTA leaves while another may still read its shared partials
  cl.sync();
}

#undef OWN

// Clusters of 16 CTAs (beyond the portable 8) are allowed once per device;
// false when the device refuses them.
bool batch_solve_allow_wide() {
  static std::atomic<uint32_t> ok{0}, tried{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const uint32_t bit = 1u << (dev & 31);
  if (!(tried.load() & bit)) {
    if (cudaFuncSetAttribute(k_batch_solve, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess)
      ok.fetch_or(bit);
    else
      cudaGetLastError();
    tried.fetch_or(bit);
  }
  return (ok.load() & bit) != 0;
}

cudaError_t launch_batch_solve(const BSolveRun* runs, int nruns, int cluster, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nruns * cluster), 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch_solve, runs);
  ::ch::note_launch();
  return e;
}

}  // namespace ch
