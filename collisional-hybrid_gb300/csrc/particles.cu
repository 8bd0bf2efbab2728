// particles.cu -- ion kernels of the hybrid-PIC hot path on sm_103a.
//
// Two state forms:
//   FP64 plain form: SoA x, y, z, vx, vy, vz (FP64, absolute positions, the
//     reference's RealVector semantics) + uint32 ion id.
//   mixed form: float4 pos = (ox, oy, oz, packed cell i | j<<11 | k<<22) with
//     within-cell offsets in [0, 1), float4 vel = (vx, vy, vz, id bits).
//     Absolute positions are rebuilt in FP64 as x0 + (i + ox) dx.
//
// One templated pass kernel per form implements UpdateVelocities
// (src/particles.c:628-643), UpdatePositions (:647-718) and
// CollectVlasovQuantities (:136-255); the phases are compile-time flags so
// that the separate entry points and the fused step share one code path.
// The CIC deposit accumulates 64-bit fixed-point integers (scale 2^s): the
// sums do not depend on the order of the additions, so the moments are
// identical run to run whatever the thread schedule or particle order.
#include "particles.cuh"

#include <atomic>
#include <cstddef>

#include "ion_dev.cuh"
#include "physics.cuh"

namespace ch {

// ------------------------------------------------------------------ helpers
// Mean relative speeds g of the mixed form are summed as integers of 2^-20:
// the FP64 partial sums are exact while the total stays below 2^33 (2^53
// units; 134 M ions of thermal speed 1 sum to about 2^28), so S does not
// depend on the order of the ions.
#define CH_G_UNIT (1.0 / 1048576.0)
__device__ __forceinline__ unsigned long long g_fixed(float g) {
  // g < 2^12 in any plasma the fixed-point deposit admits; 32-bit conversion
  return (unsigned long long)__float2uint_rn(g * 1048576.0f);
}

// Warp-aggregated increment of counts[key]; returns this lane's rank among
// the lanes that share its key, and the group's base from the atomic.
__device__ __forceinline__ uint32_t agg_inc(uint32_t* counts, uint32_t key, bool active) {
  const unsigned mask = __activemask();
  const unsigned grp = __match_any_sync(mask, active ? key : 0xFFFFFFFFu);
  const int leader = __ffs(grp) - 1;
  const int lane = threadIdx.x & 31;
  const uint32_t rank = __popc(grp & ((1u << lane) - 1u));
  uint32_t base = 0;
  if (active && lane == leader) base = atomicAdd(counts + key, (uint32_t)__popc(grp));
  base = __shfl_sync(mask, base, leader);
  return base + rank;
}

// Block-wide sum of K doubles into part[blockIdx.x * K + q], fixed order.
template <int K>
__device__ __forceinline__ void block_partials(double (&v)[K], double* __restrict__ part, int slot = -1) {
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
      if (lane == 0) part[(size_t)(slot < 0 ? (int)blockIdx.x : slot) * K + q] = x;
    }
  }
}

__device__ __forceinline__ void count_add(DevCounters* cnt, unsigned ncol, unsigned nref) {
  unsigned long long a = ncol, b = nref;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (a) atomicAdd(&cnt->collisions, a);
    if (b) atomicAdd(&cnt->refused, b);
  }
}

// ------------------------------------------------------------------ loader
// Inverse CDF of n(x) = 1 + sum_m a_m sin(2 pi m x/L + ph_m); same iteration
// as the oracle (safeguarded Newton, 40 iterations at most).
__device__ double inv_cdf_x(const ch_loader& L, double Lx, double u) {
  double target = u * Lx, lo = 0.0, hi = Lx, x = target;
  for (int it = 0; it < 40; ++it) {
    double F = x, dF = 1.0;
    for (int m = 1; m <= 3; ++m) {
      const double a = L.amp[m - 1];
      if (a == 0.0) continue;
      const double w = 2.0 * CH_PI * m / Lx;
      F += a * (cos(L.phase[m - 1]) - cos(w * x + L.phase[m - 1])) / w;
      dF += a * sin(w * x + L.phase[m - 1]);
    }
    const double r = F - target;
    if (r > 0.0) hi = x; else lo = x;
    double xn = x - r / dF;
    if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
    if (fabs(xn - x) <= 1e-15 * Lx) { x = xn; break; }
    x = xn;
  }
  if (x < 0.0) x = 0.0;
  if (x >= Lx) x = Lx * (1.0 - 1e-16);
  return x;
}

__device__ __forceinline__ void load_one(const GridDesc& g, const ch_loader& L, uint32_t seed_lo, uint32_t seed_hi,
                                         uint32_t run, uint32_t id, double out[6]) {
  const U4 a = ch_philox(id, CH_STEP_LOADER, (CH_PURPOSE_LOAD << 24) | 0u, run, seed_lo, seed_hi);
  const U4 b = ch_philox(id, CH_STEP_LOADER, (CH_PURPOSE_LOAD << 24) | 1u, run, seed_lo, seed_hi);
  out[0] = g.x0 + inv_cdf_x(L, g.Lx, ch_unit(a.x));
  out[1] = g.y0 + ch_unit(a.y) * g.Ly;
  out[2] = g.z0 + ch_unit(a.z) * g.Lz;
  const double r1 = sqrt(-2.0 * log(ch_unit(b.x))), t1 = 2.0 * CH_PI * ch_unit(b.y);
  const double r2 = sqrt(-2.0 * log(ch_unit(b.z))), t2 = 2.0 * CH_PI * ch_unit(b.w);
  out[3] = L.v0[0] + L.vT[0] * (r1 * cos(t1));
  out[4] = L.v0[1] + L.vT[1] * (r1 * sin(t1));
  out[5] = L.v0[2] + L.vT[2] * (r2 * cos(t2));
}

// FP64 absolute position -> (cell index, offset in [0, 1)), periodic.
__device__ __forceinline__ void locate(double x, double x0, double d, int n, int* i, double* f) {
  const double X = (x - x0) / d;
  const double fl = floor(X);
  int ii = (int)fl;
  *f = X - fl;
  ii %= n;
  if (ii < 0) ii += n;
  *i = ii;
}

__device__ __forceinline__ float4 pack_mixed(const GridDesc& g, const double* s) {
  int i, j, k;
  double fx, fy, fz;
  locate(s[0], g.x0, g.dx, g.Nx, &i, &fx);
  locate(s[1], g.y0, g.dy, g.Ny, &j, &fy);
  locate(s[2], g.z0, g.dz, g.Nz, &k, &fz);
  float ox = (float)fx, oy = (float)fy, oz = (float)fz;
  // rounding to FP32 may reach 1.0f: carry into the next cell
  if (ox >= 1.0f) { ox = 0.0f; i = (i + 1 == g.Nx) ? 0 : i + 1; }
  if (oy >= 1.0f) { oy = 0.0f; j = (j + 1 == g.Ny) ? 0 : j + 1; }
  if (oz >= 1.0f) { oz = 0.0f; k = (k + 1 == g.Nz) ? 0 : k + 1; }
  const uint32_t cell = (uint32_t)i | ((uint32_t)j << CH_PACK_BX) | ((uint32_t)k << (CH_PACK_BX + CH_PACK_BY));
  return make_float4(ox, oy, oz, __uint_as_float(cell));
}

__global__ void k_load_f64(GridDesc g, ch_loader L, uint32_t slo, uint32_t shi, uint32_t run, F64Particles P) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.np; i += (int64_t)gridDim.x * blockDim.x) {
    double s[6];
    load_one(g, L, slo, shi, run, (uint32_t)i, s);
    P.x[i] = s[0]; P.y[i] = s[1]; P.z[i] = s[2];
    P.vx[i] = s[3]; P.vy[i] = s[4]; P.vz[i] = s[5];
    P.id[i] = (uint32_t)i;
  }
}

__global__ void k_load_mixed(GridDesc g, ch_loader L, uint32_t slo, uint32_t shi, uint32_t run, MixParticles P) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.np; i += (int64_t)gridDim.x * blockDim.x) {
    double s[6];
    load_one(g, L, slo, shi, run, (uint32_t)i, s);
    P.pos[i] = pack_mixed(g, s);
    P.vel[i] = make_float4((float)s[3], (float)s[4], (float)s[5], __uint_as_float((uint32_t)i));
  }
}

// ------------------------------------------------------------------ placement loaders
// InitializePositions (src/particles.c:9-132) with the reference's
// --density-type choices; velocities Maxwellian as in load_one.  Positions
// use explicitly rounded arithmetic (no contraction) so that the CPU
// restatement of each placement gives the same bits.
struct SobolDirs {
  uint32_t v[3][32];
};

// Point n of the 3-D Sobol sequence in Gray-code order (Antonov & Saleev):
// the XOR of the direction numbers of the set bits of n ^ (n >> 1).
__device__ __forceinline__ void sobol_point(const SobolDirs& D, uint32_t n, double r[3]) {
  const uint32_t gc = n ^ (n >> 1);
  uint32_t x[3] = {0u, 0u, 0u};
  for (int k = 0; k < 32; ++k)
    if (gc & (1u << k)) {
      x[0] ^= D.v[0][k];
      x[1] ^= D.v[1][k];
      x[2] ^= D.v[2][k];
    }
  for (int d = 0; d < 3; ++d) r[d] = (double)x[d] * 2.3283064365386962890625e-10;  // 2^-32, exact
}

// SobolDistribution (src/distributions.c:96-128): v = r (L + d) - d/2,
// clamped to [p0 + 0.01 d, p1 - 0.01 d] as the reference does.
__device__ __forceinline__ double sobol_coord(double r, double L, double d, double p0, double p1) {
  const double v = __dsub_rn(__dmul_rn(r, __dadd_rn(L, d)), __dmul_rn(0.5, d));
  if (v < p0) return __dadd_rn(p0, __dmul_rn(0.01, d));
  if (v > p1) return __dsub_rn(p1, __dmul_rn(0.01, d));
  return v;
}

__device__ __forceinline__ void load_placed_one(const GridDesc& g, const ch_loader& L, const SobolDirs& D, int type,
                                                int64_t per_cell, uint32_t slo, uint32_t shi, uint32_t run,
                                                uint32_t id, double out[6]) {
  if (type == CH_DENSITY_FLAT_SOBOL) {
    double r[3];
    sobol_point(D, id + 1u, r);  // point 0 is the origin; the reference's first call initialises
    out[0] = sobol_coord(r[0], g.Lx, g.dx, g.x0, g.x0 + g.Lx);
    out[1] = sobol_coord(r[1], g.Ly, g.dy, g.y0, g.y0 + g.Ly);
    out[2] = sobol_coord(r[2], g.Lz, g.dz, g.z0, g.z0 + g.Lz);
  } else if (type == CH_DENSITY_UNIFORM) {
    // UniformDistribution (src/distributions.c:33-94): per_cell ions at the
    // centre of every cell, ion id in cell id mod N
    const int64_t c = (int64_t)id % g.N;
    const int i = (int)(c % g.Nx), j = (int)((c / g.Nx) % g.Ny), k = (int)(c / ((int64_t)g.Nx * g.Ny));
    out[0] = __dadd_rn(g.x0, __dmul_rn(g.dx, __dadd_rn((double)i, 0.5)));
    out[1] = __dadd_rn(g.y0, __dmul_rn(g.dy, __dadd_rn((double)j, 0.5)));
    out[2] = __dadd_rn(g.z0, __dmul_rn(g.dz, __dadd_rn((double)k, 0.5)));
    (void)per_cell;
  } else {
    // Rejection (src/distributions.c:143-232) of SinusoidalDistribution
    // (:131-141), n(x) = 1 + 0.25 sin(2 pi x) at the proposal's x = r L,
    // accepted when n > v max n with the bound max n = 1.25 (the reference
    // takes the maximum over integer points, where the sine vanishes)
    for (uint32_t a = 0; a < 256u; ++a) {
      const U4 q = ch_philox(id, CH_STEP_LOADER, (CH_PURPOSE_LOAD << 24) | (2u + a), run, slo, shi);
      const double x = __dmul_rn(ch_unit(q.x), g.Lx), y = __dmul_rn(ch_unit(q.y), g.Ly),
                   z = __dmul_rn(ch_unit(q.z), g.Lz);
      const double w = 1.0 + 0.25 * sin(2.0 * CH_PI * x);
      out[0] = g.x0 + x;
      out[1] = g.y0 + y;
      out[2] = g.z0 + z;
      if (w > __dmul_rn(ch_unit(q.w), 1.25)) break;
    }
  }
  const U4 b = ch_philox(id, CH_STEP_LOADER, (CH_PURPOSE_LOAD << 24) | 1u, run, slo, shi);
  const double r1 = sqrt(-2.0 * log(ch_unit(b.x))), t1 = 2.0 * CH_PI * ch_unit(b.y);
  const double r2 = sqrt(-2.0 * log(ch_unit(b.z))), t2 = 2.0 * CH_PI * ch_unit(b.w);
  out[3] = L.v0[0] + L.vT[0] * (r1 * cos(t1));
  out[4] = L.v0[1] + L.vT[1] * (r1 * sin(t1));
  out[5] = L.v0[2] + L.vT[2] * (r2 * cos(t2));
}

template <bool MIXED>
__global__ void k_load_placed(GridDesc g, ch_loader L, SobolDirs D, int type, int64_t per_cell, uint32_t slo,
                              uint32_t shi, uint32_t run, F64Particles P, MixParticles M) {
  const int64_t np = MIXED ? M.np : P.np;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
    double s[6];
    load_placed_one(g, L, D, type, per_cell, slo, shi, run, (uint32_t)i, s);
    if (MIXED) {
      M.pos[i] = pack_mixed(g, s);
      M.vel[i] = make_float4((float)s[3], (float)s[4], (float)s[5], __uint_as_float((uint32_t)i));
    } else {
      P.x[i] = s[0]; P.y[i] = s[1]; P.z[i] = s[2];
      P.vx[i] = s[3]; P.vy[i] = s[4]; P.vz[i] = s[5];
      P.id[i] = (uint32_t)i;
    }
  }
}

// Direction numbers of the first three Sobol dimensions (Joe & Kuo's table):
// dimension 1 the van der Corput sequence; dimension 2 the polynomial x + 1
// with m1 = 1; dimension 3 x^2 + x + 1 with m1 = 1, m2 = 3.  Bratley & Fox's
// recursion v_k = a1 v_{k-1} ^ ... ^ v_{k-s} ^ (v_{k-s} >> s).
static SobolDirs sobol_dirs() {
  SobolDirs D;
  for (int k = 0; k < 32; ++k) D.v[0][k] = 1u << (31 - k);
  D.v[1][0] = 1u << 31;
  for (int k = 1; k < 32; ++k) D.v[1][k] = D.v[1][k - 1] ^ (D.v[1][k - 1] >> 1);
  D.v[2][0] = 1u << 31;
  D.v[2][1] = 3u << 30;
  for (int k = 2; k < 32; ++k) D.v[2][k] = D.v[2][k - 1] ^ D.v[2][k - 2] ^ (D.v[2][k - 2] >> 2);
  return D;
}

void launch_load_placed(bool mixed, const GridDesc& g, const ch_loader& L, int type, uint64_t seed, uint32_t run,
                        F64Particles P, MixParticles M, int sms, cudaStream_t s) {
  const uint32_t lo = (uint32_t)seed, hi = (uint32_t)(seed >> 32);
  const SobolDirs D = sobol_dirs();
  const int64_t np = mixed ? M.np : P.np;
  const int64_t per_cell = np / (g.N > 0 ? g.N : 1);
  if (mixed)
    k_load_placed<true><<<grid_for(np, 256, sms, 8), 256, 0, s>>>(g, L, D, type, per_cell, lo, hi, run, P, M),
        ::ch::note_launch();
  else
    k_load_placed<false><<<grid_for(np, 256, sms, 8), 256, 0, s>>>(g, L, D, type, per_cell, lo, hi, run, P, M),
        ::ch::note_launch();
}

// AoS RealVector (x, y, z, r) staging -> state, id = index.
__global__ void k_aos_to_f64(const double4_32a* __restrict__ pos, const double4_32a* __restrict__ vel, F64Particles P) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.np; i += (int64_t)gridDim.x * blockDim.x) {
    const double4_32a p = pos[i], v = vel[i];
    P.x[i] = p.x; P.y[i] = p.y; P.z[i] = p.z;
    P.vx[i] = v.x; P.vy[i] = v.y; P.vz[i] = v.z;
    P.id[i] = (uint32_t)i;
  }
}

__global__ void k_aos_to_mixed(GridDesc g, const double4_32a* __restrict__ pos, const double4_32a* __restrict__ vel,
                               MixParticles P) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.np; i += (int64_t)gridDim.x * blockDim.x) {
    const double4_32a p = pos[i], v = vel[i];
    const double s[3] = {p.x, p.y, p.z};
    P.pos[i] = pack_mixed(g, s);
    P.vel[i] = make_float4((float)v.x, (float)v.y, (float)v.z, __uint_as_float((uint32_t)i));
  }
}

// state -> AoS staging in id order (undoes the cell sort).
__global__ void k_f64_to_aos(F64Particles P, double4_32a* __restrict__ pos, double4_32a* __restrict__ vel) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.np; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t id = P.id[i];
    pos[id] = make_double4_32a(P.x[i], P.y[i], P.z[i], 0.0);
    vel[id] = make_double4_32a(P.vx[i], P.vy[i], P.vz[i], 0.0);
  }
}

__global__ void k_mixed_to_aos(GridDesc g, MixParticles P, double4_32a* __restrict__ pos, double4_32a* __restrict__ vel) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.np; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 p = P.pos[i], v = P.vel[i];
    const uint32_t cell = __float_as_uint(p.w);
    const int ci = cell & (CH_MAX_NX - 1), cj = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1),
              ck = cell >> (CH_PACK_BX + CH_PACK_BY);
    const uint32_t id = __float_as_uint(v.w);
    pos[id] = make_double4_32a(g.x0 + ((double)ci + (double)p.x) * g.dx, g.y0 + ((double)cj + (double)p.y) * g.dy,
                           g.z0 + ((double)ck + (double)p.z) * g.dz, 0.0);
    vel[id] = make_double4_32a((double)v.x, (double)v.y, (double)v.z, 0.0);
  }
}

// ------------------------------------------------------------------ node field
// E = -grad phi by periodic central differences (the Escale of
// src/particles.c:391-393 applied at the nodes).
__global__ void k_node_efield_f64(GridDesc g, const double* __restrict__ phi, double* __restrict__ E) {
  const int64_t N = g.N;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    ch_ijk(g, c, i, j, k);
    const int ip = i + 1 == g.Nx ? 0 : i + 1, im = i == 0 ? g.Nx - 1 : i - 1;
    const int jp = j + 1 == g.Ny ? 0 : j + 1, jm = j == 0 ? g.Ny - 1 : j - 1;
    const int kp = k + 1 == g.Nz ? 0 : k + 1, km = k == 0 ? g.Nz - 1 : k - 1;
    const int64_t row = ((int64_t)k * g.Ny + j) * g.Nx;
    E[c] = -(phi[row + ip] - phi[row + im]) / (2.0 * g.dx);
    E[N + c] = -(phi[((int64_t)k * g.Ny + jp) * g.Nx + i] - phi[((int64_t)k * g.Ny + jm) * g.Nx + i]) / (2.0 * g.dy);
    E[2 * N + c] =
        -(phi[((int64_t)kp * g.Ny + j) * g.Nx + i] - phi[((int64_t)km * g.Ny + j) * g.Nx + i]) / (2.0 * g.dz);
  }
}

// -grad(phi) at the nodes by central differences, premultiplied by the push
// scale (q/m) dt/2.  s[d] = -(q/m)(dt/2) / (2 h_d) comes from the host, so a
// component is one FP64 difference and one product: FP64 division is slow
// on this part.
__global__ void k_node_efield_mixed(GridDesc g, double sx, double sy, double sz, const double* __restrict__ phi,
                                    float4* __restrict__ E) {
  const int64_t N = g.N;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    ch_ijk(g, c, i, j, k);
    const int ip = i + 1 == g.Nx ? 0 : i + 1, im = i == 0 ? g.Nx - 1 : i - 1;
    const int jp = j + 1 == g.Ny ? 0 : j + 1, jm = j == 0 ? g.Ny - 1 : j - 1;
    const int kp = k + 1 == g.Nz ? 0 : k + 1, km = k == 0 ? g.Nz - 1 : k - 1;
    const int64_t row = ((int64_t)k * g.Ny + j) * g.Nx;
    const double dx = phi[row + ip] - phi[row + im];
    const double dy = phi[((int64_t)k * g.Ny + jp) * g.Nx + i] - phi[((int64_t)k * g.Ny + jm) * g.Nx + i];
    const double dz = phi[((int64_t)kp * g.Ny + j) * g.Nx + i] - phi[((int64_t)km * g.Ny + j) * g.Nx + i];
    E[c] = make_float4((float)(dx * sx), (float)(dy * sy), (float)(dz * sz), 0.0f);
  }
}

// DifferenceVector as written (src/vectors.c:12-138): CH_FAITHFUL_D3 / D4.
__device__ void diffvec_faithful(const GridDesc& g, const double* __restrict__ phi, double X, double Y, double Z,
                                 uint32_t faithful, double f[3]) {
  const int ixl = (int)floor(X), iyl = (int)floor(Y), izl = (int)floor(Z);
  const double wxh = X - ixl, wyh = Y - iyl, wzh = Z - izl;
  const int ixh = ixl + 1, iyh = iyl + 1, izh = izl + 1;
  const bool onesided = (faithful & CH_FAITHFUL_D4) != 0;
  auto F = [&](int k, int j, int i) { return phi[ch_nid(g, i, j, k)]; };
  for (int d = 0; d < 3; ++d) {
    auto diff = [&](int k, int j, int i) -> double {
      if (d == 0) {
        if (onesided && i == g.Nx) return 3.0 * F(k, j, i) - 4.0 * F(k, j, i - 1) + F(k, j, i - 2);
        return F(k, j, i + 1) - F(k, j, i - 1);
      } else if (d == 1) {
        if (onesided && j == g.Ny) return 3.0 * F(k, j, i) - 4.0 * F(k, j - 1, i) + F(k, j - 2, i);
        return F(k, j + 1, i) - F(k, j - 1, i);
      }
      if (onesided && k == g.Nz) return 3.0 * F(k, j, i) - 4.0 * F(k - 1, j, i) + F(k - 2, j, i);
      return F(k + 1, j, i) - F(k - 1, j, i);
    };
    const double hhh = diff(izh, iyh, ixh), lhh = diff(izl, iyh, ixh), hlh = diff(izh, iyl, ixh),
                 llh = diff(izl, iyl, ixh), hhl = diff(izh, iyh, ixl), lhl = diff(izl, iyh, ixl),
                 hll = diff(izh, iyl, ixl), lll = diff(izl, iyl, ixl);
    const double whh = hlh + wyh * (hhh - hlh), whl = hll + wyh * (hhl - hll);
    const double wlh = llh + wyh * (lhh - llh), wll = lll + wyh * (lhl - lll);
    if (faithful & CH_FAITHFUL_D3) {
      const double Ewh = wlh + wxh * (whh - wlh), Ewl = wll + wxh * (whl - wll);
      f[d] = Ewl + wzh * (Ewh - Ewh);
    } else {
      const double Ezl = wll + wxh * (wlh - wll), Ezh = whl + wxh * (whh - whl);
      f[d] = Ezl + wzh * (Ezh - Ezl);
    }
  }
}


// ------------------------------------------------------------------ FP64 pass
// Block partials: 0 expected, 1 S(next).
// Colliding ions of the FP64 pass wait in a per-warp ring and run their
// event process 32 at a time, so the FP64 pipe (the bound of this form on
// GB300) is not spent on lanes idling through another lane's rejection loop.
#define CH_F64_QW 64
struct F64Queue {
  uint32_t ip[8][CH_F64_QW];
  double v[8][CH_F64_QW][3];
  double ls[8][CH_F64_QW];
};

// Finishes n <= 32 queued ions of the calling warp (warp-uniform head/n):
// the event process, the step's S term, the velocity and, with the move,
// the new position.
template <int PH>
__device__ __forceinline__ void f64_queue_round(F64Queue& Q, const StepConsts& c, F64Particles P, unsigned& head,
                                                unsigned n, double& gsum, unsigned& ncol, unsigned& nref) {
  const GridDesc& g = c.g;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if ((unsigned)lane < n) {
    const unsigned e = (head + lane) & (CH_F64_QW - 1);
    const int64_t ip = Q.ip[w][e];
    double v[3] = {Q.v[w][e][0], Q.v[w][e][1], Q.v[w][e][2]};
    ncol += ch_collide<double>(c, P.id[ip], Q.ls[w][e], v, &nref);
    const double qx = v[0] - c.vn0[0], qy = v[1] - c.vn0[1], qz = v[2] - c.vn0[2];
    gsum += ch_gmean<double>(sqrt(qx * qx + qy * qy + qz * qz), c.vnT);
    P.vx[ip] = v[0]; P.vy[ip] = v[1]; P.vz[ip] = v[2];
    if ((PH & PH_MOVE) && !(c.faithful & CH_FAITHFUL_D5)) {
      P.x[ip] = wrap_pos(P.x[ip] + v[0] * c.dt, g.x0, g.Lx);
      P.y[ip] = wrap_pos(P.y[ip] + v[1] * c.dt, g.y0, g.Ly);
      P.z[ip] = wrap_pos(P.z[ip] + v[2] * c.dt, g.z0, g.Lz);
    }
  }
  head += n;
  __syncwarp();  // the entries are read before later appends reuse them
}

template <int PH>
__global__ void __launch_bounds__(256) k_pass_f64(StepConsts c, F64Particles P, const double* __restrict__ E,
                                                  const double* __restrict__ phi, unsigned long long* __restrict__ acc,
                                                  double Nc, double sbar, DevCounters* cnt, double* part) {
  const GridDesc& g = c.g;
  const int64_t N = g.N;
  double vsum[2] = {0.0, 0.0};
  unsigned ncol = 0, nref = 0;
  int bad = 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool gather_faithful = (c.faithful & (CH_FAITHFUL_D3 | CH_FAITHFUL_D4)) != 0;
  constexpr bool QUEUE = (PH & PH_PUSH) != 0;
  extern __shared__ __align__(16) unsigned char smem_f64[];
  F64Queue& Q = *reinterpret_cast<F64Queue*>(smem_f64);
  unsigned qhead = 0, qtail = 0;  // warp-uniform
  // block-uniform iterations: the deposit's warp reduction and the queue
  // need every lane
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < P.np; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ip = base + threadIdx.x;
    const bool act = ip < P.np;
    double x = 0.0, y = 0.0, z = 0.0;
    double v[3] = {0.0, 0.0, 0.0};
    if (act) {
      x = P.x[ip]; y = P.y[ip]; z = P.z[ip];
      v[0] = P.vx[ip]; v[1] = P.vy[ip]; v[2] = P.vz[ip];
    }
    bool defer = false;
    double lscale = 0.0;
    if ((PH & PH_PUSH) && act) {
      const double X = (x - g.x0) / g.dx, Y = (y - g.y0) / g.dy, Z = (z - g.z0) / g.dz;
      double Ef[3];
      if (gather_faithful) {
        double f[3];
        diffvec_faithful(g, phi, X, Y, Z, c.faithful, f);
        Ef[0] = -f[0] / (2.0 * g.dx); Ef[1] = -f[1] / (2.0 * g.dy); Ef[2] = -f[2] / (2.0 * g.dz);
      } else {
        const double fi = floor(X), fj = floor(Y), fk = floor(Z);
        const double wx = X - fi, wy = Y - fj, wz = Z - fk;
        const int i = ch_wrap((int)fi, g.Nx), j = ch_wrap((int)fj, g.Ny), k = ch_wrap((int)fk, g.Nz);
        const int i1 = i + 1 == g.Nx ? 0 : i + 1, j1 = j + 1 == g.Ny ? 0 : j + 1, k1 = k + 1 == g.Nz ? 0 : k + 1;
        const int64_t c000 = ((int64_t)k * g.Ny + j) * g.Nx + i, c100 = ((int64_t)k * g.Ny + j) * g.Nx + i1,
                      c010 = ((int64_t)k * g.Ny + j1) * g.Nx + i, c110 = ((int64_t)k * g.Ny + j1) * g.Nx + i1,
                      c001 = ((int64_t)k1 * g.Ny + j) * g.Nx + i, c101 = ((int64_t)k1 * g.Ny + j) * g.Nx + i1,
                      c011 = ((int64_t)k1 * g.Ny + j1) * g.Nx + i, c111 = ((int64_t)k1 * g.Ny + j1) * g.Nx + i1;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const double* e = E + d * N;
          const double wll = e[c000] + wy * (e[c010] - e[c000]);
          const double wlh = e[c100] + wy * (e[c110] - e[c100]);
          const double whl = e[c001] + wy * (e[c011] - e[c001]);
          const double whh = e[c101] + wy * (e[c111] - e[c101]);
          const double ezl = wll + wx * (wlh - wll);
          const double ezh = whl + wx * (whh - whl);
          Ef[d] = ezl + wz * (ezh - ezl);
        }
      }
      if (c.push_E0) { Ef[0] += c.E0[0]; Ef[1] += c.E0[1]; Ef[2] += c.E0[2]; }
      ch_boris<double>(c, Ef, v);
      if (c.collide) {
        const double wx = v[0] - c.vn0[0], wy = v[1] - c.vn0[1], wz = v[2] - c.vn0[2];
        const double gi = ch_gmean<double>(sqrt(wx * wx + wy * wy + wz * wz), c.vnT);
        lscale = sbar > 0.0 ? (Nc * ch_neutral_density<double>(c, x)) / sbar : 0.0;
        const double lam = lscale * gi;
        vsum[0] += lam;
        // the first waiting time here; ions with an event inside the step
        // join the warp's queue, the others keep g of their velocity for S
        const U4 r0 = ch_philox(P.id[ip], c.step, CH_PURPOSE_COLLIDE << 24, c.run, c.seed_lo, c.seed_hi);
        defer = lam > 0.0 && -log(ch_unit(r0.x)) / lam < 1.0;
        if (!defer) vsum[1] += gi;
      }
      if (!defer) { P.vx[ip] = v[0]; P.vy[ip] = v[1]; P.vz[ip] = v[2]; }
    }
    if ((PH & PH_MOVE) && !(c.faithful & CH_FAITHFUL_D5) && act && !defer) {
      x = wrap_pos(x + v[0] * c.dt, g.x0, g.Lx);
      y = wrap_pos(y + v[1] * c.dt, g.y0, g.Ly);
      z = wrap_pos(z + v[2] * c.dt, g.z0, g.Lz);
      P.x[ip] = x; P.y[ip] = y; P.z[ip] = z;
    }
    if (QUEUE) {
      // append (at most 31 wait between iterations, so 32 more fit), then
      // full rounds
      const unsigned dm = __ballot_sync(0xffffffffu, defer);
      if (defer) {
        const unsigned e = (qtail + __popc(dm & ((1u << lane) - 1u))) & (CH_F64_QW - 1);
        Q.ip[w][e] = (uint32_t)ip;
        Q.v[w][e][0] = v[0]; Q.v[w][e][1] = v[1]; Q.v[w][e][2] = v[2];
        Q.ls[w][e] = lscale;
      }
      qtail += (unsigned)__popc(dm);
      __syncwarp();
      while (qtail - qhead >= 32u) f64_queue_round<PH>(Q, c, P, qhead, 32u, vsum[1], ncol, nref);
    }
    if (PH & PH_DEPOSIT) {
      bool ok = act;
      if (act && !(isfinite(x) && isfinite(y) && isfinite(z) && isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) {
        bad = 1;  // a non-finite ion is reported, never deposited
        ok = false;
      }
      int di = 0, dj = 0, dk = 0;
      double wx = 0.0, wy = 0.0, wz = 0.0;
      if (ok) {
        const double X = (x - g.x0) / g.dx, Y = (y - g.y0) / g.dy, Z = (z - g.z0) / g.dz;
        const double fi = floor(X), fj = floor(Y), fk = floor(Z);
        di = ch_wrap((int)fi, g.Nx); dj = ch_wrap((int)fj, g.Ny); dk = ch_wrap((int)fk, g.Nz);
        wx = X - fi; wy = Y - fj; wz = Z - fk;
      }
      deposit_cic_warp(g, acc, ok, di, dj, dk, wx, wy, wz, v[0], v[1], v[2], c.dep_scale);
    }
  }
  if (QUEUE) {
    while (qtail != qhead) f64_queue_round<PH>(Q, c, P, qhead, min(qtail - qhead, 32u), vsum[1], ncol, nref);
  }
  if (bad) atomicOr(&cnt->range_error, 2);
  if (PH & PH_PUSH) {
    count_add(cnt, ncol, nref);
    block_partials<2>(vsum, part);
  }
}

// ------------------------------------------------------------------ mixed pass, tiled
// The ions are sorted by cell; starts[c] is the first slot of cell c at the
// last sort.  One CTA owns a brick of TX x TY x TZ cells (persistent loop
// over bricks): it stages the node field of the brick plus a one-cell halo
// in shared memory, pushes the brick's ions (any ion still within one cell
// of its brick gathers from shared memory), and deposits into a shared
// fixed-point tile that is flushed to the global accumulators once per
// brick.  Within a warp, lanes whose ions share a cell are summed with
// integer warp reductions before one lane updates the shared tile.  Ions
// that left the halo, or move faster than CH_TILE_VMAX cells/dt units, take
// the direct global path.  Every sum is an integer sum (each contribution is
// rounded to a fixed-point integer first), so the moments do not depend on
// the order of the ions or of the threads.
#define TX 16
#define TY 4
#define TZ 4
#define BX (TX + 3)
#define BY (TY + 3)
#define BZ (TZ + 3)
#define BNODES (BX * BY * BZ)
#define CH_TILE_DSCALE 4194304.0f    // 2^22: density contributions (w <= 1)
#define CH_TILE_FSCALE 524288.0f     // 2^19: flux contributions (|v| < CH_TILE_VMAX)
#define CH_TILE_VMAX 8.0f
#define CH_TILE_DLOG2 22
#define CH_TILE_FLOG2 19
// Round-to-nearest-even of a b, |a b| <= 2^22, on the FP32 pipe: the exact
// product plus 1.5 * 2^23 lies in [2^23, 2^24), where floats are the
// integers, so the bits of fma(a, b, 1.5 * 2^23) are rint(a b) + CH_RNI_BIAS
// (the conversion unit runs at a fraction of the rate).
#define CH_RNI_BIAS 0x4B400000
__device__ __forceinline__ int rni_fma(float a, float b) { return __float_as_int(__fmaf_rn(a, b, 12582912.0f)); }

#define CH_PUSH_CTAS 4          // CTAs per SM of a pass without the deposit
#define CH_DEP_CTAS 3           // CTAs per SM of a deposit pass (72 KB of shared memory each)
#define CH_TILE_QCAP 512       // deferred colliding ions: one ring of CH_TILE_QW per warp
#define CH_TILE_QW (CH_TILE_QCAP / 8)
static_assert(CH_TILE_QW >= 64 && (CH_TILE_QW & (CH_TILE_QW - 1)) == 0,
              "a warp ring holds 31 pending + 32 new entries and is indexed modulo its size");

#define CH_TILE_K 4            // consecutive slots one thread deposits together
#define CH_DEP_RW 256          // ring of displaced ions per warp (31 waiting + 128 of a chunk fit)
#define CH_DEP_SEG 32768u      // ions of a brick deposited between two flushes of its tile

// Shared memory of one CTA of the tiled pass: [push part][header][deposit
// part].  A pass with the push allocates from the start; a deposit-only pass
// allocates from the header, so it needs no room for the field tile and the
// collision queue (tile_smem_base / tile_smem_bytes).
struct TileShared {
  // ---- push part
  alignas(16) float4 E[BNODES];
  // Ions whose first collision event falls inside the step are queued here
  // after the Boris push and finished (collide, move, deposit) together, so
  // the long collision code runs on full warps instead of one lane in 40.
  // Warp w owns entries [w CH_TILE_QW, (w + 1) CH_TILE_QW) as a ring.
  float4 q_pos[CH_TILE_QCAP];   // offsets + packed cell, before the move
  float4 q_vel[CH_TILE_QCAP];   // velocity after the push, rate scale in w
  uint32_t q_ip[CH_TILE_QCAP];
  uint32_t q_id[CH_TILE_QCAP];
  float q_t[CH_TILE_QCAP];      // elapsed time of the event process (waiting times so far)
  uint32_t q_st[CH_TILE_QCAP];  // event | proposal << 8
  // Thread t's next ion (position, velocity), copied in by cp.async while
  // the current one is pushed.
  alignas(16) float4 pf_pos[256];
  alignas(16) float4 pf_vel[256];
  // ---- header
  alignas(16) uint32_t rowbeg[TY * TZ];
  uint32_t pre[TY * TZ + 1];
  // ---- deposit part
  uint32_t d_ip[8 * CH_DEP_RW];  // per warp: ring of displaced ions (indices into the ion arrays)
  // per warp: a chunk's ions while they are loaded, then lane l's 32 sums in
  // row l (33 words: no bank conflicts)
  alignas(16) unsigned d_sum[8][32 * 33];
  // Fixed-point sums at the tile scale, each value v added as its low 16
  // bits to acc_lo and as v >> 16 to acc_hi: the sum is acc_hi 2^16 +
  // acc_lo, exact in any order while a segment of the brick adds fewer than
  // 2^16 values to a word (CH_DEP_SEG).
  unsigned acc_lo[4][BNODES];
  int acc_hi[4][BNODES];
};

template <int PH>
constexpr size_t tile_smem_skip() {  // bytes of TileShared a launch of PH does not allocate
  return (PH & (PH_PUSH | PH_MOVE)) ? 0 : offsetof(TileShared, rowbeg);
}
template <int PH>
constexpr size_t tile_smem_bytes() {
  return (PH & PH_DEPOSIT) ? sizeof(TileShared) - tile_smem_skip<PH>() : offsetof(TileShared, d_ip);
}
// The TileShared view of a launch's dynamic shared memory: for a
// deposit-only launch the allocation starts at the header, and the push part
// (never touched by such a launch) lies before it.
template <int PH>
__device__ __forceinline__ TileShared& tile_smem_base(unsigned char* smem) {
  return *reinterpret_cast<TileShared*>(smem - tile_smem_skip<PH>());
}

// value += v for a 64-bit integer kept in shared memory as two 32-bit words
// whose sum lo + 2^16 hi is the exact value whatever the order of adds.
// Adds v (|v| < 2^31) to a tile sum: two 32-bit reductions that need no
// returned value, so no carry round trip; neither word can overflow within
// a segment of at most CH_DEP_SEG ions (below 2^16 adds of under 2^16 to
// acc_lo, of under 2^15 in magnitude to acc_hi).
__device__ __forceinline__ void shared_add64(unsigned* lo, int* hi, long long v) {
  atomicAdd(lo, (unsigned)(v & 0xFFFF));
  atomicAdd(hi, (int)(v >> 16));
}

// Adds x to a tile sum from r = rni_fma(...) = rint(x) + CH_RNI_BIAS: the
// bias has zero low 16 bits, so r's low half is x's and r's high half
// exceeds x >> 16 by the bias's (r is positive: no sign to carry).
__device__ __forceinline__ void shared_add_rni(unsigned* lo, int* hi, int r) {
  atomicAdd(lo, (unsigned)r & 0xFFFFu);
  atomicAdd(hi, (int)((unsigned)r >> 16) - (CH_RNI_BIAS >> 16));
}

// One ion's 32 fixed-point contributions added lane by lane to the shared
// tile (node = the ion's cell within the box).
// The four moments are taken in an order rotated by lane & 3: lanes whose
// ions landed in the same cell (displaced together) then add to different
// words in each instruction instead of queueing on one.
__device__ __forceinline__ void tile_deposit_lane(TileShared& sh, int node, float wxh, float wyh, float wzh,
                                                  float vx, float vy, float vz) {
  const float wxl = 1.0f - wxh, wyl = 1.0f - wyh, wzl = 1.0f - wzh;
  const float w[8] = {wzl * wyl * wxl, wzl * wyl * wxh, wzl * wyh * wxl, wzl * wyh * wxh,
                      wzh * wyl * wxl, wzh * wyl * wxh, wzh * wyh * wxl, wzh * wyh * wxh};
  // moment m adds rint(a_m w): a = 2^22 (density), v 2^19 (fluxes), exact
  // products inside the FMA
  const float a0 = CH_TILE_DSCALE, a1 = vx * CH_TILE_FSCALE, a2 = vy * CH_TILE_FSCALE, a3 = vz * CH_TILE_FSCALE;
  const int s = threadIdx.x & 3;
  float ar[4];
  unsigned* lo[4];
  int* hi[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int m = (t + s) & 3;
    ar[t] = m == 0 ? a0 : m == 1 ? a1 : m == 2 ? a2 : a3;
    lo[t] = &sh.acc_lo[0][0] + m * BNODES + node;
    hi[t] = &sh.acc_hi[0][0] + m * BNODES + node;
  }
#pragma unroll
  for (int cn = 0; cn < 8; ++cn) {
    const int off = (cn & 1) + ((cn >> 1) & 1) * BX + (cn >> 2) * BX * BY;
#pragma unroll
    for (int t = 0; t < 4; ++t) shared_add_rni(lo[t] + off, hi[t] + off, rni_fma(ar[t], w[cn]));
  }
}

// An ion the tile does not take (outside the brick's halo, or a component of
// v at or above CH_TILE_VMAX) goes straight to the global accumulators with
// the tile's rounding: each contribution is the integer the tile would add,
// rint(w 2^22) and rint((v 2^19) w) of the same FP32 weights (products exact
// in FP64, ties to even as rni_fma), scaled by 2^shift to the accumulator
// scale.  So the moments do not depend on which path an ion takes, which
// depends on the order of the ions (their distance from the brick their slot
// belongs to).  Out-of-range values saturate in the conversion.
__device__ __forceinline__ void deposit_cic_tile_rounding(const GridDesc& g, unsigned long long* __restrict__ acc,
                                                          int i, int j, int k, float wxh, float wyh, float wzh,
                                                          float vx, float vy, float vz, int shift_d, int shift_f) {
  const float wxl = 1.0f - wxh, wyl = 1.0f - wyh, wzl = 1.0f - wzh;
  const float w[8] = {wzl * wyl * wxl, wzl * wyl * wxh, wzl * wyh * wxl, wzl * wyh * wxh,
                      wzh * wyl * wxl, wzh * wyl * wxh, wzh * wyh * wxl, wzh * wyh * wxh};
  const double fx = (double)(vx * CH_TILE_FSCALE), fy = (double)(vy * CH_TILE_FSCALE),
               fz = (double)(vz * CH_TILE_FSCALE);
  const double sd = ldexp(1.0, shift_d), sf = ldexp(1.0, shift_f);
  const int i1 = i + 1 == g.Nx ? 0 : i + 1, j1 = j + 1 == g.Ny ? 0 : j + 1, k1 = k + 1 == g.Nz ? 0 : k + 1;
  const int64_t N = g.N;
#pragma unroll
  for (int cn = 0; cn < 8; ++cn) {
    const int64_t nd = ((int64_t)((cn >> 2) ? k1 : k) * g.Ny + ((cn >> 1) & 1 ? j1 : j)) * g.Nx + ((cn & 1) ? i1 : i);
    const double wd = (double)w[cn];
    red_add(acc + nd, __double2ll_rn(rint(wd * (double)CH_TILE_DSCALE) * sd));
    red_add(acc + N + nd, __double2ll_rn(rint(fx * wd) * sf));
    red_add(acc + 2 * N + nd, __double2ll_rn(rint(fy * wd) * sf));
    red_add(acc + 3 * N + nd, __double2ll_rn(rint(fz * wd) * sf));
  }
}

// Box-relative cell offset of (i, j, k) from the box origin, periodic; the
// origin (wi0, wj0, wk0) is given wrapped into the grid, so one correction
// per axis brings the difference into [0, N).
__device__ __forceinline__ int box_key(const GridDesc& g, int i, int j, int k, int wi0, int wj0, int wk0,
                                       bool* inbox) {
  int di = i - wi0, dj = j - wj0, dk = k - wk0;
  di += di < 0 ? g.Nx : 0;
  dj += dj < 0 ? g.Ny : 0;
  dk += dk < 0 ? g.Nz : 0;
  *inbox = di <= BX - 2 && dj <= BY - 2 && dk <= BZ - 2;
  return (dk * BY + dj) * BX + di;
}

// Deposit of one brick whose ions' cells are current (a deposit-only pass).
// Warp w takes the chunks of 128 consecutive slots w, w + 8, ...; lane l the
// 4 slots 4l .. 4l+3 of a chunk (the ions of a cell are contiguous after a
// sort and mostly stay together between sorts, so the 4 usually share a
// cell), loaded coalesced through the warp's matrix area when the chunk lies
// in one brick row and straight from global memory otherwise.  A lane sums
// the 32 fixed-point contributions of its slots in the cell most of them
// share in registers; the sums of lanes whose cells agree are then added up
// through a matrix in shared memory (lane q sums entry q of each run of equal
// cells) and added to the brick once per run.  The other slots go to the warp's ring and are
// added lane by lane, 32 at a time: ions in another cell ("displaced": they
// moved since the last sort) to the brick's tile, ions outside the brick's
// halo or faster than CH_TILE_VMAX straight to the global accumulators, and
// non-finite ions are flagged (bad) and not deposited.
// The chunk itself runs without divergent branches: a slot the lane does not
// sum enters the same arithmetic with zero weights and zero velocity
// (selected, so that a non-finite ion adds nothing), and the accumulators
// start at minus the four biases of rni_fma.
// Every contribution is rounded to an integer before any addition, so the
// result does not depend on the order; no block barrier is needed.
// SCAT (a step that ends with a sort): every ion read is also written to
// slot dst_starts[its cell] + its rank of Q (the ranks come from the push's
// cell count), which is the counting sort's scatter; the deposit reads each
// ion anyway.  A separate instantiation, so that the plain deposit keeps
// its registers.
template <bool SCAT>
__device__ __forceinline__ void tile_deposit_direct(TileShared& sh, const StepConsts& c, MixParticles P,
                                                    unsigned long long* __restrict__ acc, uint32_t seg0,
                                                    uint32_t total, int wi0, int wj0, int wk0, int shift_d,
                                                    int shift_f, int& bad,
                                                    MixParticles Q, const uint32_t* __restrict__ dst_starts) {
  const GridDesc& g = c.g;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* ring = sh.d_ip + warp * CH_DEP_RW;
  const unsigned lt = (1u << lane) - 1u;
  unsigned dh = 0, dt = 0;  // warp-uniform ring head / tail
  // lanes l < n add the ring's next n ions
  auto drain = [&](unsigned n) {
    if ((unsigned)lane < n) {
      const uint32_t ip = ring[(dh + lane) & (CH_DEP_RW - 1)];
      const float4 p = P.pos[ip], v = P.vel[ip];
      const uint32_t cell = __float_as_uint(p.w);
      const int i = cell & (CH_MAX_NX - 1), j = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1),
                kz = cell >> (CH_PACK_BX + CH_PACK_BY);
      bool inbox;
      const int key = box_key(g, i, j, kz, wi0, wj0, wk0, &inbox);
      const bool finite =
          isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
      const bool slow = fabsf(v.x) >= CH_TILE_VMAX || fabsf(v.y) >= CH_TILE_VMAX || fabsf(v.z) >= CH_TILE_VMAX;
      if (!finite) bad = 1;  // not deposited
      else if (inbox && !slow) tile_deposit_lane(sh, key, p.x, p.y, p.z, v.x, v.y, v.z);
      else deposit_cic_tile_rounding(g, acc, i, j, kz, p.x, p.y, p.z, v.x, v.y, v.z, shift_d, shift_f);
    }
    dh += n;
    __syncwarp();  // the entries are read before later appends reuse them
  };
  // one pass more than there are chunks: the last one only drains the ring
  // (a single inlined copy of the drain)
  for (uint32_t cb = seg0 + (uint32_t)warp * 128u;; cb += (blockDim.x >> 5) * 128u) {
    const bool more = cb < total;  // warp-uniform
    if (more) {
      const uint32_t s0 = cb + 4u * (uint32_t)lane;
      const uint32_t cend = min(cb + 128u, total);
      // the row of the chunk's first slot (warp-uniform: the last row starting
      // at or before it, so empty rows are skipped)
      int rc = 0;
#pragma unroll
      for (int st = 8; st > 0; st >>= 1)
        if (rc + st < TY * TZ && sh.pre[rc + st] <= cb) rc += st;
      // slot -> index in the ion arrays; slots past the chunk's end read its
      // last ion and are masked below
      uint32_t ips[CH_TILE_K];
      const bool onerow = cend <= sh.pre[rc + 1];  // the chunk lies in one row (warp-uniform)
      const uint32_t base = sh.rowbeg[rc] - sh.pre[rc];
      if (onerow) {
#pragma unroll
        for (int k = 0; k < CH_TILE_K; ++k) ips[k] = min(s0 + k, cend - 1u) + base;
      } else {
#pragma unroll
        for (int k = 0; k < CH_TILE_K; ++k) {
          const uint32_t s = min(s0 + k, cend - 1u);
          int r = 0;
#pragma unroll
          for (int st = 8; st > 0; st >>= 1)
            if (r + st < TY * TZ && sh.pre[r + st] <= s) r += st;
          ips[k] = sh.rowbeg[r] + (s - sh.pre[r]);
        }
      }
      float4 pk[CH_TILE_K], vk[CH_TILE_K];
      if (onerow) {
        // Coalesced: lane l loads slots cb + 32 i + l and parks them in the
        // warp's matrix area (float4 q at q ^ ((q >> 3) & 7): neither the
        // stores nor the reads below conflict); it then reads its own four.
        // SCAT: the ions are scattered from here, where neighbouring lanes
        // hold neighbouring slots, which the push ranked in this lane order,
        // so a cell's ions leave for consecutive slots (full sectors).
        static_assert(CH_TILE_K == 4 && 8 * sizeof(float4) * 32 <= sizeof(sh.d_sum[0]), "a chunk fits the matrix area");
        float4* X = reinterpret_cast<float4*>(sh.d_sum[warp]);
#pragma unroll
        for (int i = 0; i < CH_TILE_K; ++i) {
          const uint32_t sl = cb + 32u * (uint32_t)i + (uint32_t)lane;
          const uint32_t ipc = min(sl, cend - 1u) + base;
          const float4 p = P.pos[ipc], v = P.vel[ipc];
          const int q = 32 * i + lane, qs = q ^ ((q >> 3) & 7);
          X[qs] = p;
          X[128 + qs] = v;
          if (SCAT && sl < cend) {
            const uint32_t cell = __float_as_uint(p.w);
            const uint32_t ci = cell & (CH_MAX_NX - 1), cj = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1),
                           ck = cell >> (CH_PACK_BX + CH_PACK_BY);
            const uint32_t d = dst_starts[(ck * (uint32_t)g.Ny + cj) * (uint32_t)g.Nx + ci] + P.rank[ipc];
            Q.pos[d] = p;
            Q.vel[d] = v;
          }
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < CH_TILE_K; ++k) {
          const int q = CH_TILE_K * lane + k, qs = q ^ ((q >> 3) & 7);
          pk[k] = X[qs];
          vk[k] = X[128 + qs];
        }
        __syncwarp();  // read before the lanes' sums overwrite the area
      } else {
#pragma unroll
        for (int k = 0; k < CH_TILE_K; ++k) { pk[k] = P.pos[ips[k]]; vk[k] = P.vel[ips[k]]; }
      }
      int keys[CH_TILE_K];
      bool other[CH_TILE_K];  // to the ring whatever the lane's cell
#pragma unroll
      for (int k = 0; k < CH_TILE_K; ++k) {
        const float4 p = pk[k], v = vk[k];
        const bool valid = s0 + k < cend;
        const uint32_t cell = __float_as_uint(p.w);
        const int i = cell & (CH_MAX_NX - 1), j = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1),
                  kz = cell >> (CH_PACK_BX + CH_PACK_BY);
        if (SCAT && valid && !onerow) {  // every ion, whether or not it is deposited here
          const uint32_t d = dst_starts[(kz * g.Ny + j) * g.Nx + i] + P.rank[ips[k]];
          Q.pos[d] = p;
          Q.vel[d] = v;
        }
        bool inbox;
        const int key = box_key(g, i, j, kz, wi0, wj0, wk0, &inbox);
        // |v| below the tile's bound and in-cell offsets (each in [0, 1))
        // summing below 3: both comparisons fail for NaN and infinities, so
        // a non-finite ion goes to the ring, where the drain flags it
        const bool fits = fabsf(v.x) < CH_TILE_VMAX && fabsf(v.y) < CH_TILE_VMAX && fabsf(v.z) < CH_TILE_VMAX &&
                          p.x + p.y + p.z < 3.0f;
        const bool take = valid && inbox && fits;
        keys[k] = take ? key : -1;
        other[k] = valid && !take;
      }
      // the cell most of the lane's slots share (ties: the earliest)
      int akey = -1, best = 0;
#pragma unroll
      for (int k = 0; k < CH_TILE_K; ++k) {
        int n = 0;
#pragma unroll
        for (int q = 0; q < CH_TILE_K; ++q) n += (keys[q] == keys[k]) ? 1 : 0;
        if (keys[k] >= 0 && n > best) { best = n; akey = keys[k]; }
      }
      // displaced, outside and fast slots to the ring (at most 31 wait there,
      // so 128 more fit)
#pragma unroll
      for (int k = 0; k < CH_TILE_K; ++k) {
        const bool dsp = other[k] || (keys[k] >= 0 && keys[k] != akey);
        const unsigned m = __ballot_sync(0xffffffffu, dsp);
        if (dsp) ring[(dt + __popc(m & lt)) & (CH_DEP_RW - 1)] = ips[k];
        dt += (unsigned)__popc(m);
      }
      // each slot adds rint(x) + CH_RNI_BIAS per entry; starting from minus
      // four biases leaves the exact sums, |sum| < 2^25
      constexpr unsigned a0 = 0u - (unsigned)CH_TILE_K * (unsigned)CH_RNI_BIAS;
      unsigned a[32];
#pragma unroll
      for (int k = 0; k < CH_TILE_K; ++k) {
        const bool use = keys[k] >= 0 && keys[k] == akey;
        const float wxh = use ? pk[k].x : 0.0f, wyh = use ? pk[k].y : 0.0f, oz = use ? pk[k].z : 0.0f;
        const float wxl = 1.0f - wxh, wyl = 1.0f - wyh;
        const float wzh = use ? oz : 0.0f, wzl = use ? 1.0f - oz : 0.0f;
        const float w[8] = {wzl * wyl * wxl, wzl * wyl * wxh, wzl * wyh * wxl, wzl * wyh * wxh,
                            wzh * wyl * wxl, wzh * wyl * wxh, wzh * wyh * wxl, wzh * wyh * wxh};
        // (v 2^19) w is v (w 2^19) exactly: the scale is a power of two
        const float fx = use ? vk[k].x * CH_TILE_FSCALE : 0.0f, fy = use ? vk[k].y * CH_TILE_FSCALE : 0.0f,
                    fz = use ? vk[k].z * CH_TILE_FSCALE : 0.0f;
#pragma unroll
        for (int cn = 0; cn < 8; ++cn) {
          a[cn] = (k == 0 ? a0 : a[cn]) + (unsigned)rni_fma(w[cn], CH_TILE_DSCALE);
          a[8 + cn] = (k == 0 ? a0 : a[8 + cn]) + (unsigned)rni_fma(fx, w[cn]);
          a[16 + cn] = (k == 0 ? a0 : a[16 + cn]) + (unsigned)rni_fma(fy, w[cn]);
          a[24 + cn] = (k == 0 ? a0 : a[24 + cn]) + (unsigned)rni_fma(fz, w[cn]);
        }
      }
      // Sums of lanes whose cells agree: lane l's 32 sums become row l of the
      // warp's matrix, and lane q walks column q down the rows, adding one sum
      // per run of equal cells (consecutive in sorted order) to node q & 7 of
      // that cell, moment q >> 3.  The run ends come from one ballot, so the
      // walk tests a bit of a warp-wide word per row instead of comparing cells.
      unsigned* M = sh.d_sum[warp];
#pragma unroll
      for (int q = 0; q < 32; ++q) M[lane * 33 + q] = a[q];
      const int up = __shfl_down_sync(0xffffffffu, akey, 1);
      const unsigned ends = __ballot_sync(0xffffffffu, lane == 31 || akey != up);  // row l ends a run
      __syncwarp();
      {
        const int cn = lane & 7, m = lane >> 3;
        const int off = (cn & 1) + ((cn >> 1) & 1) * BX + (cn >> 2) * BX * BY;
        int s2[2] = {0, 0};  // even and odd rows (two add chains); |sum| < 32 x 2^25
#pragma unroll
        for (int l = 0; l < 32; ++l) {
          s2[l & 1] += (int)M[l * 33 + lane];  // a lane without a cell holds zeros
          if ((ends >> l) & 1u) {
            const int kl = __shfl_sync(0xffffffffu, akey, l);
            const int sum = s2[0] + s2[1];
            if (kl >= 0 && sum != 0) shared_add64(&sh.acc_lo[m][kl + off], &sh.acc_hi[m][kl + off], sum);
            s2[0] = s2[1] = 0;
          }
        }
      }
      __syncwarp();  // ring entries visible, matrix read before the next chunk rewrites it
    }
    // full rounds of 32; after the last chunk, the rest
    while (dt - dh >= 32u || (!more && dt != dh)) drain(min(dt - dh, 32u));
    if (!more) break;
  }
}

// Adds the brick's tile to the global accumulators (tile sums are at the
// tile scale, 2^22 density and 2^19 flux, shifted to the accumulator scale
// 2^s) and, with zero, clears it for the next segment.  Each thread flushes
// and clears its own entries.
__device__ __forceinline__ void tile_flush(TileShared& sh, const GridDesc& g, unsigned long long* __restrict__ acc,
                                           int bi0, int bj0, int bk0, int shift_d, int shift_f, bool zero) {
  for (int q = threadIdx.x; q < 4 * BNODES; q += blockDim.x) {
    const int m = q / BNODES, nd = q % BNODES;
    const long long a = ((long long)sh.acc_hi[m][nd] * 65536 + (long long)sh.acc_lo[m][nd])
                        << (m == 0 ? shift_d : shift_f);
    if (zero) { sh.acc_lo[m][nd] = 0u; sh.acc_hi[m][nd] = 0; }
    if (a != 0) {
      const int bi = nd % BX, bj = (nd / BX) % BY, bk = nd / (BX * BY);
      const int gi = ch_wrap(bi0 + bi, g.Nx), gj = ch_wrap(bj0 + bj, g.Ny), gk = ch_wrap(bk0 + bk, g.Nz);
      atomicAdd(acc + (int64_t)m * g.N + ((int64_t)gk * g.Ny + gj) * g.Nx + gi, (unsigned long long)a);
    }
  }
}

// 16-byte asynchronous copy global -> shared (L2 only), and its group fences.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Moves one ion by v dt (cell units), wraps it into the grid and repacks the
// cell word.
__device__ __forceinline__ void tile_move_ion(const StepConsts& c, float4& p, const float v[3], int& i, int& j,
                                              int& k) {
  const GridDesc& g = c.g;
  float ox = p.x + v[0] * c.f.dtx, oy = p.y + v[1] * c.f.dty, oz = p.z + v[2] * c.f.dtz;
  float fx = floorf(ox), fy = floorf(oy), fz = floorf(oz);
  ox -= fx; oy -= fy; oz -= fz;
  // a tiny negative offset rounds up to 1.0f: that point is the start of
  // the next cell, so carry into it (as pack_mixed does)
  if (ox >= 1.0f) { ox = 0.0f; fx += 1.0f; }
  if (oy >= 1.0f) { oy = 0.0f; fy += 1.0f; }
  if (oz >= 1.0f) { oz = 0.0f; fz += 1.0f; }
  if (isfinite(fx) && isfinite(fy) && isfinite(fz)) {
    i = ch_wrap(i + (int)fx, g.Nx); j = ch_wrap(j + (int)fy, g.Ny); k = ch_wrap(k + (int)fz, g.Nz);
  }
  const uint32_t cell = (uint32_t)i | ((uint32_t)j << CH_PACK_BX) | ((uint32_t)k << (CH_PACK_BX + CH_PACK_BY));
  p = make_float4(ox, oy, oz, __uint_as_float(cell));
}

// The 8 node-field values around cell (i, j, k) from global memory.
__device__ __forceinline__ void tile_gather_global(const GridDesc& g, const float4* __restrict__ E, int i, int j, int k,
                                                   float4& e000, float4& e100, float4& e010, float4& e110,
                                                   float4& e001, float4& e101, float4& e011, float4& e111) {
  const int ii1 = i + 1 == g.Nx ? 0 : i + 1, jj1 = j + 1 == g.Ny ? 0 : j + 1, kk1 = k + 1 == g.Nz ? 0 : k + 1;
  const int64_t r00 = ((int64_t)k * g.Ny + j) * g.Nx, r10 = ((int64_t)k * g.Ny + jj1) * g.Nx,
                r01 = ((int64_t)kk1 * g.Ny + j) * g.Nx, r11 = ((int64_t)kk1 * g.Ny + jj1) * g.Nx;
  e000 = __ldg(E + r00 + i); e100 = __ldg(E + r00 + ii1); e010 = __ldg(E + r10 + i);
  e110 = __ldg(E + r10 + ii1); e001 = __ldg(E + r01 + i); e101 = __ldg(E + r01 + ii1);
  e011 = __ldg(E + r11 + i); e111 = __ldg(E + r11 + ii1);
}

// Trilinear gather of the node field (premultiplied by (q/m) dt/2) at the
// in-cell offsets of p, then the Boris push of v (src/particles.c:374-447);
// every kernel of the mixed form that pushes an ion calls this, so they
// agree bit for bit.
__device__ __forceinline__ void tile_boris(const StepConsts& c, const float4& e000, const float4& e100,
                                           const float4& e010, const float4& e110, const float4& e001,
                                           const float4& e101, const float4& e011, const float4& e111,
                                           const float4& p, bool cross, float v[3]) {
  const float t0 = c.f.t[0], t1 = c.f.t[1], t2 = c.f.t[2];
  const float s0 = c.f.s[0], s1 = c.f.s[1], s2 = c.f.s[2];
  const float wx = p.x, wy = p.y, wz = p.z;
  float Ef[3];
#define LERP3(f, d)                                                                \
{                                                                                \
  const float wll = e000.f + wy * (e010.f - e000.f);                             \
  const float wlh = e100.f + wy * (e110.f - e100.f);                             \
  const float whl = e001.f + wy * (e011.f - e001.f);                             \
  const float whh = e101.f + wy * (e111.f - e101.f);                             \
  const float ezl = wll + wx * (wlh - wll), ezh = whl + wx * (whh - whl);        \
  Ef[d] = ezl + wz * (ezh - ezl);                                                \
}
  LERP3(x, 0) LERP3(y, 1) LERP3(z, 2)
#undef LERP3
  if (c.push_E0) { Ef[0] += c.f.pE0[0]; Ef[1] += c.f.pE0[1]; Ef[2] += c.f.pE0[2]; }
  // Boris with E premultiplied by (q/m) dt/2
  const float vm0 = v[0] + Ef[0], vm1 = v[1] + Ef[1], vm2 = v[2] + Ef[2];
  float vp0 = vm0, vp1 = vm1, vp2 = vm2;
  if (cross) {
    const float q0 = vm0 + (vm1 * t2 - vm2 * t1);
    const float q1 = vm1 + (vm2 * t0 - vm0 * t2);
    const float q2 = vm2 + (vm0 * t1 - vm1 * t0);
    vp0 = vm0 + (q1 * s2 - q2 * s1);
    vp1 = vm1 + (q2 * s0 - q0 * s2);
    vp2 = vm2 + (q0 * s1 - q1 * s0);
  }
  v[0] = vp0 + Ef[0]; v[1] = vp1 + Ef[1]; v[2] = vp2 + Ef[2];
}

__device__ __forceinline__ float tile_gmean(const StepConsts& c, const float v[3]) {
  return ch_gmean<float>(ch_relspeed_rn(v[0], v[1], v[2], c.f.vn0[0], c.f.vn0[1], c.f.vn0[2]), c.f.vnT);
}

// One drain round of the calling warp's ring of deferred ions (warp-uniform
// head, tail and n <= 32): lane l < n advances entry head + l by one proposal
// of its current collision event (with the scatter and the next waiting time
// when the proposal is accepted).  Ions with further events go back to the
// tail; the others are finished: velocity stored, moved and counted in the
// new cell.  Needs no block barrier: only the warp touches its ring.
template <int PH>
__device__ __forceinline__ void tile_queue_round(TileShared& sh, const StepConsts& c, MixParticles P, uint32_t* hist,
                                                 unsigned& head, unsigned& tail, unsigned n, unsigned long long& gsum,
                                                 unsigned& ncol, unsigned& nref) {
  const GridDesc& g = c.g;
  const int lane = threadIdx.x & 31;
  const unsigned wbase = (threadIdx.x >> 5) * CH_TILE_QW;
  const bool move = (PH & PH_MOVE) && !(c.faithful & CH_FAITHFUL_D5);
  const bool act = (unsigned)lane < n;
  float4 qp = make_float4(0.f, 0.f, 0.f, 0.f), q4 = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t qip = 0, qid = 0, st = 0;
  float qtm = 0.0f;
  if (act) {
    const unsigned e = wbase + ((head + lane) & (CH_TILE_QW - 1));
    qp = sh.q_pos[e];
    q4 = sh.q_vel[e];
    qip = sh.q_ip[e];
    qid = sh.q_id[e];
    qtm = sh.q_t[e];
    st = sh.q_st[e];
  }
  __syncwarp();  // this round's entries are read before a re-queue reuses their slots
  float qv[3] = {q4.x, q4.y, q4.z};
  const float qsc = q4.w;
  uint32_t qe = st & 0xFFu, qit = st >> 8;
  bool done = false;
  float gf = 0.0f;  // g of the final velocity of a finished ion
  if (act) done = ch_collide_round<float>(c, qid, qsc, qv, qtm, qe, qit, &ncol, &nref, gf);
  const bool requeue = act && !done;
  const unsigned rm = __ballot_sync(0xffffffffu, requeue);
  if (requeue) {
    const unsigned e = wbase + ((tail + __popc(rm & ((1u << lane) - 1u))) & (CH_TILE_QW - 1));
    sh.q_pos[e] = qp;
    sh.q_vel[e] = make_float4(qv[0], qv[1], qv[2], qsc);
    sh.q_ip[e] = qip;
    sh.q_id[e] = qid;
    sh.q_t[e] = qtm;
    sh.q_st[e] = qe | (qit << 8);
  }
  tail += (unsigned)__popc(rm);
  head += n;
  __syncwarp();  // re-queued entries are visible to the lanes that read them next
  const bool fin = act && done;
  int qi = 0, qj = 0, qk = 0;
  if (fin) {
    gsum += g_fixed(gf);
    P.vel[qip] = make_float4(qv[0], qv[1], qv[2], __uint_as_float(qid));
    const uint32_t cell = __float_as_uint(qp.w);
    qi = cell & (CH_MAX_NX - 1); qj = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1);
    qk = cell >> (CH_PACK_BX + CH_PACK_BY);
    if (move) {
      tile_move_ion(c, qp, qv, qi, qj, qk);
      P.pos[qip] = qp;
    }
  }
  if (hist) {
    const uint32_t rk = agg_inc(hist, (uint32_t)(((int64_t)qk * g.Ny + qj) * g.Nx + qi), fin);
    if (fin && P.rank) P.rank[qip] = rk;
  }
}

// One brick of the tiled pass: tile index `tile` of the run described by c
// (starts, E, acc and hist are the run's own arrays; starts holds indices
// into P).  Per-thread sums go to vsum / gsum / ncol / nref / bad.  Deferred
// colliding ions wait in the warp's ring (head, tail); with CARRY the ring is
// left as it is at the end of the brick (the caller drains it after its last
// brick: possible when the finish of an ion does not use the brick, i.e.
// without the deposit, and the run's constants do not change between
// bricks), otherwise it is drained here.
template <int PH, bool CARRY, bool SCAT = false>
__device__ __forceinline__ void tile_pass(TileShared& sh, const StepConsts& c, MixParticles P,
                                          const float4* __restrict__ E, const uint32_t* __restrict__ starts,
                                          unsigned long long* __restrict__ acc, float pscale, int shift_d,
                                          int shift_f, uint32_t* hist, int tile, double (&vsum)[2],
                                          unsigned long long& gsum, unsigned& qhead, unsigned& qtail, unsigned& ncol,
                                          unsigned& nref, int& bad, MixParticles Q = MixParticles{},
                                          const uint32_t* dst_starts = nullptr) {
  static_assert(PH == PH_DEPOSIT || !(PH & PH_DEPOSIT), "the deposit has a launch of its own");
  static_assert(!(CARRY && (PH & PH_DEPOSIT)), "a deposit pass has no deferred ions to carry");
  const GridDesc& g = c.g;
  const int lane = threadIdx.x & 31;
  const unsigned wbase = (threadIdx.x >> 5) * CH_TILE_QW;
  const bool cross = !(c.faithful & CH_FAITHFUL_D2);
  const bool move = (PH & PH_MOVE) && !(c.faithful & CH_FAITHFUL_D5);
  const bool collide = (PH & PH_PUSH) && c.collide;
  const int ntx = (g.Nx + TX - 1) / TX, nty = (g.Ny + TY - 1) / TY;

  const int i0 = (tile % ntx) * TX, j0 = ((tile / ntx) % nty) * TY, k0 = (tile / (ntx * nty)) * TZ;
  const int i1 = min(i0 + TX, g.Nx), j1 = min(j0 + TY, g.Ny), k1 = min(k0 + TZ, g.Nz);
  const int bi0 = i0 - 1, bj0 = j0 - 1, bk0 = k0 - 1;  // box origin (node)
  const int wi0 = ch_wrap(bi0, g.Nx), wj0 = ch_wrap(bj0, g.Ny), wk0 = ch_wrap(bk0, g.Nz);  // wrapped into the grid
  __syncthreads();  // previous brick's flush is done
  // stage the node field and the row ranges (the deposit tile is clear: the
  // kernel clears it before its first brick, each flush after it)
  if (PH & PH_PUSH) {
    for (int q = threadIdx.x; q < BNODES; q += blockDim.x) {
      const int bi = q % BX, bj = (q / BX) % BY, bk = q / (BX * BY);
      const int gi = ch_wrap(bi0 + bi, g.Nx), gj = ch_wrap(bj0 + bj, g.Ny), gk = ch_wrap(bk0 + bk, g.Nz);
      sh.E[q] = __ldg(E + ((int64_t)gk * g.Ny + gj) * g.Nx + gi);
    }
  }
  if (threadIdx.x < 32) {  // lane r: row r (tk = k0 + r / TY, tj = j0 + r % TY); pre = scan of the counts
    static_assert(TY * TZ <= 32, "one lane per row of the brick");
    const int r = threadIdx.x, tk = k0 + r / TY, tj = j0 + r % TY;
    uint32_t b = 0, n = 0;
    if (r < TY * TZ && tk < k1 && tj < j1) {
      const int64_t cf = ((int64_t)tk * g.Ny + tj) * g.Nx + i0;
      b = starts[cf];
      n = starts[cf + (i1 - i0)] - b;
    }
    uint32_t x = n;  // inclusive scan over the lanes
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
      if (r >= d) x += y;
    }
    if (r < TY * TZ) {
      sh.rowbeg[r] = b;
      sh.pre[r] = x - n;
    }
    if (r == TY * TZ - 1) sh.pre[TY * TZ] = x;
  }
  __syncthreads();
  const uint32_t total = sh.pre[TY * TZ];
  // Per-brick sum of the expected events (reported only) in FP32; the
  // post-step mean relative speeds, which normalise the next step's rates,
  // go to gsum as integers of 2^-20 so that S is exact whatever the ion order.
  float tsum0 = 0.0f;
  if (PH == PH_DEPOSIT) {
    // segments of at most CH_DEP_SEG ions, the tile flushed between them
    for (uint32_t seg = 0; seg < total; seg += CH_DEP_SEG) {
      if (seg > 0) {
        __syncthreads();
        tile_flush(sh, g, acc, bi0, bj0, bk0, shift_d, shift_f, true);
        __syncthreads();
      }
      tile_deposit_direct<SCAT>(sh, c, P, acc, seg, min(total, seg + CH_DEP_SEG), wi0, wj0, wk0, shift_d, shift_f,
                                bad, Q, dst_starts);
    }
  }
  const uint32_t ptotal = total * (PH == PH_DEPOSIT ? 0u : 1u);  // ions the push / move loop visits
  // index of slot idx in the ion arrays (rows of the brick are contiguous)
  // (a thread's slots only increase, so its row is kept and advanced: the
  // last row that starts at or before the slot, past empty rows)
  int srow = 0;
  auto slot_ip = [&](uint32_t idx) -> uint32_t {
    while (srow + 1 < TY * TZ && sh.pre[srow + 1] <= idx) ++srow;
    return sh.rowbeg[srow] + (idx - sh.pre[srow]);
  };
  // Thread t's ions are slots t, t + 256, ...; the next one is copied into
  // the thread's own prefetch slot by cp.async while this one is pushed (only
  // thread t touches slot t, and it has read the slot before refilling it).
  uint32_t next_ip = 0;
  if (threadIdx.x < ptotal) {
    next_ip = slot_ip(threadIdx.x);
    cp_async16(&sh.pf_pos[threadIdx.x], P.pos + next_ip);
    cp_async16(&sh.pf_vel[threadIdx.x], P.vel + next_ip);
  }
  cp_async_commit();
#pragma unroll 1
  for (uint32_t base = 0; base < ptotal; base += blockDim.x) {
    const uint32_t idx = base + threadIdx.x;
    const bool active = idx < ptotal;
    const int64_t ip = next_ip;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f), vv = make_float4(0.f, 0.f, 0.f, 0.f);
    cp_async_wait_all();
    if (active) {
      p = sh.pf_pos[threadIdx.x];
      vv = sh.pf_vel[threadIdx.x];
    }
    if (idx + blockDim.x < ptotal) {
      next_ip = slot_ip(idx + blockDim.x);
      cp_async16(&sh.pf_pos[threadIdx.x], P.pos + next_ip);
      cp_async16(&sh.pf_vel[threadIdx.x], P.vel + next_ip);
    }
    cp_async_commit();
    int i = 0, j = 0, k = 0;
    float v[3] = {0.f, 0.f, 0.f};
    if (active) {
      const uint32_t cell = __float_as_uint(p.w);
      i = cell & (CH_MAX_NX - 1); j = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1); k = cell >> (CH_PACK_BX + CH_PACK_BY);
      v[0] = vv.x; v[1] = vv.y; v[2] = vv.z;
    }
    bool defer = false;
    float qscale = 0.0f, qt0 = 0.0f;  // rate scale and first waiting time of a deferred ion
    if ((PH & PH_PUSH) && active) {
      bool near;
      const int q = box_key(g, i, j, k, wi0, wj0, wk0, &near);
      float4 e000, e100, e010, e110, e001, e101, e011, e111;
      if (near) {
        e000 = sh.E[q]; e100 = sh.E[q + 1]; e010 = sh.E[q + BX]; e110 = sh.E[q + BX + 1];
        e001 = sh.E[q + BX * BY]; e101 = sh.E[q + BX * BY + 1]; e011 = sh.E[q + BX * BY + BX];
        e111 = sh.E[q + BX * BY + BX + 1];
      } else {
        tile_gather_global(g, E, i, j, k, e000, e100, e010, e110, e001, e101, e011, e111);
      }
      tile_boris(c, e000, e100, e010, e110, e001, e101, e011, e111, p, cross, v);
      if (collide) {
        const float gi = tile_gmean(c, v);
        float nd = 1.0f;
        if (c.nn_profile == CH_NN_GAUSSIAN_X)
          nd = ch_neutral_density<float>(c, (float)(g.x0 + ((double)i + (double)p.x) * g.dx));
        const float lscale = pscale * nd;
        const float lam = lscale * gi;
        tsum0 += lam;
        const uint32_t id = __float_as_uint(vv.w);
        const U4 r0 = ch_philox(id, c.step, CH_PURPOSE_COLLIDE << 24, c.run, c.seed_lo, c.seed_hi);
        // first event inside the step: -log(u) < lam  <=>  u > exp(-lam);
        // the queue keeps its waiting time
        const float u0 = ch_unitf(r0.x);
        if (lam > 0.0f && u0 > __expf(-lam)) {
          qt0 = ch_qdiv(-ch_log(u0), lam);
          defer = qt0 < 1.0f;
        }
        if (defer) qscale = lscale;
        else gsum += g_fixed(gi);
      }
      if (!defer) {
        vv.x = v[0]; vv.y = v[1]; vv.z = v[2];
        P.vel[ip] = vv;
      }
    }
    if (collide) {
      // append the deferred ions to the warp's ring (at most 31 entries
      // wait there between iterations, so 32 more fit)
      const unsigned dm = __ballot_sync(0xffffffffu, defer);
      if (defer) {
        const unsigned e = wbase + ((qtail + __popc(dm & ((1u << lane) - 1u))) & (CH_TILE_QW - 1));
        sh.q_pos[e] = p;
        sh.q_vel[e] = make_float4(v[0], v[1], v[2], qscale);
        sh.q_ip[e] = (uint32_t)ip;
        sh.q_id[e] = __float_as_uint(vv.w);
        sh.q_t[e] = qt0;
        sh.q_st[e] = 0u;
      }
      qtail += (unsigned)__popc(dm);
    }
    const bool go = active && !defer;
    if (move && go) tile_move_ion(c, p, v, i, j, k);
    if (move && go) P.pos[ip] = p;
    if (hist) {
      const uint32_t rk = agg_inc(hist, (uint32_t)(((int64_t)k * g.Ny + j) * g.Nx + i), go);
      if (go && P.rank) P.rank[ip] = rk;
    }
    if (collide) {
      __syncwarp();  // the appended entries are visible to every lane
      // full rounds as the ring fills (each advances 32 ions by one proposal)
      while (qtail - qhead >= 32u)
        tile_queue_round<PH>(sh, c, P, hist, qhead, qtail, 32u, gsum, ncol, nref);
    }
  }
  if (!CARRY) {
    while (qtail != qhead)
      tile_queue_round<PH>(sh, c, P, hist, qhead, qtail, min(qtail - qhead, 32u), gsum, ncol, nref);
  }
  vsum[0] += (double)tsum0;
  if (PH & PH_DEPOSIT) {
    __syncthreads();
    tile_flush(sh, g, acc, bi0, bj0, bk0, shift_d, shift_f, true);
  }
}

// Clears a deposit launch's tile before its first brick (tile_pass leaves it
// clear after each brick); the first tile_pass starts with a block barrier.
template <int PH>
__device__ __forceinline__ void tile_clear(TileShared& sh) {
  if (PH & PH_DEPOSIT) {
    for (int q = threadIdx.x; q < BNODES; q += blockDim.x) {
#pragma unroll
      for (int m = 0; m < 4; ++m) { sh.acc_lo[m][q] = 0u; sh.acc_hi[m][q] = 0; }
    }
  }
}

// A pass without the deposit carries deferred ions from brick to brick and
// drains the rings once, after the CTA's last brick.  SCAT: the deposit
// also scatters the ions into Q in the order of dst_starts.
template <int PH, bool SCAT = false>
__global__ void __launch_bounds__(256, (PH & PH_DEPOSIT) ? CH_DEP_CTAS : CH_PUSH_CTAS)
    k_pass_tiled(StepConsts c, MixParticles P, const float4* __restrict__ E, const uint32_t* __restrict__ starts,
                 unsigned long long* __restrict__ acc, float pscale, int shift_d, int shift_f, DevCounters* cnt,
                 double* part, uint32_t* hist, MixParticles Q, const uint32_t* dst_starts) {
  constexpr bool CARRY = !(PH & PH_DEPOSIT);
  extern __shared__ __align__(16) unsigned char smem_tiled[];
  TileShared& sh = tile_smem_base<PH>(smem_tiled);
  double vsum[2] = {0.0, 0.0};
  unsigned long long gsum = 0ull;
  unsigned qhead = 0, qtail = 0, ncol = 0, nref = 0;
  int bad = 0;
  const GridDesc& g = c.g;
  const int ntiles = ((g.Nx + TX - 1) / TX) * ((g.Ny + TY - 1) / TY) * ((g.Nz + TZ - 1) / TZ);
  tile_clear<PH>(sh);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
    tile_pass<PH, CARRY, SCAT>(sh, c, P, E, starts, acc, pscale, shift_d, shift_f, hist, tile, vsum, gsum, qhead,
                               qtail, ncol, nref, bad, Q, dst_starts);
  if (CARRY) {
    while (qtail != qhead)
      tile_queue_round<PH>(sh, c, P, hist, qhead, qtail, min(qtail - qhead, 32u), gsum, ncol, nref);
  }
  if (bad) atomicOr(&cnt->range_error, 2);
  if (PH & PH_PUSH) {
    vsum[1] = (double)gsum * CH_G_UNIT;
    count_add(cnt, ncol, nref);
    block_partials<2>(vsum, part);
  }
}
// ------------------------------------------------------------------ ensembles
// Every run's bricks in one persistent launch: brick t belongs to the run r
// with tile_off[r] <= t < tile_off[r + 1]; the run's constants are staged in
// shared memory and the brick is processed by the same tile_pass as a single
// run (its deferred ions finished inside the brick, as the next brick may
// belong to another run).  Brick partials are written per brick, so the run
// sums are formed in a fixed order afterwards.
// SCAT: the deposit also writes the ions to Q in the order of dst_starts
// (global slots, indexed by node_off[r] + cell), as the single-run pass.
template <int PH, bool SCAT = false>
__global__ void __launch_bounds__(256, (PH & PH_DEPOSIT) ? CH_DEP_CTAS : CH_PUSH_CTAS)
    k_batch_pass(BatchDev B, const uint32_t* dstep, MixParticles P, const float4* __restrict__ E,
                 const uint32_t* __restrict__ starts, unsigned long long* __restrict__ acc,
                 const double* __restrict__ sbar, int shift_d, int shift_f, uint32_t* hist, double* tile_part,
                 int* flags, MixParticles Q, const uint32_t* __restrict__ dst_starts) {
  extern __shared__ __align__(16) unsigned char smem_tiled[];
  TileShared& sh = tile_smem_base<PH>(smem_tiled);
  __shared__ StepConsts sc;
  __shared__ int s_run;
  __shared__ float s_pscale;
  constexpr int W = (int)(sizeof(StepConsts) / sizeof(uint32_t));
  static_assert(sizeof(StepConsts) % sizeof(uint32_t) == 0, "StepConsts is copied as words");
  tile_clear<PH>(sh);
  for (int t = blockIdx.x; t < B.total_tiles; t += gridDim.x) {
    __syncthreads();  // the previous brick is done with sc
    if (threadIdx.x == 0) {
      int lo = 0, hi = B.nruns;  // largest r with tile_off[r] <= t
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (B.tile_off[mid] <= t) lo = mid; else hi = mid;
      }
      s_run = lo;
    }
    __syncthreads();
    const int r = s_run;
    const BatchRunDev& R = B.runs[r];
    for (int w = threadIdx.x; w < W; w += blockDim.x)
      reinterpret_cast<uint32_t*>(&sc)[w] = reinterpret_cast<const uint32_t*>(&R.c)[w];
    if (threadIdx.x == 0) {  // one FP64 division per brick, not per thread
      const double S = sbar[r];
      s_pscale = S > 0.0 ? (float)(R.Nc / S) : 0.0f;
    }
    __syncthreads();
    if (threadIdx.x == 0) sc.step = *dstep;
    const int64_t no = R.node_off;
    const float pscale = s_pscale;
    double vsum[4] = {0.0, 0.0, 0.0, 0.0};
    double v2[2] = {0.0, 0.0};
    unsigned long long gsum = 0ull;
    unsigned qhead = 0, qtail = 0, ncol = 0, nref = 0;
    int bad = 0;
    // tile_pass starts with a barrier, after which sc.step is visible
    tile_pass<PH, false, SCAT>(sh, sc, P, E + no, starts + no, acc + 4 * no, pscale, shift_d, shift_f,
                               hist ? hist + no : nullptr, t - R.tile_off, v2, gsum, qhead, qtail, ncol, nref, bad,
                               Q, SCAT ? dst_starts + no : nullptr);
    if (bad) atomicOr(flags + r, 16);  // non-finite ion
    vsum[0] = v2[0]; vsum[1] = (double)gsum * CH_G_UNIT; vsum[2] = (double)ncol; vsum[3] = (double)nref;
    block_partials<4>(vsum, tile_part, t);
  }
}

__global__ void k_batch_runsum(BatchDev B, const double* __restrict__ tile_part, double* sums, double* sbar,
                               int* flags, uint32_t* dstep) {
  const int r = blockIdx.x;
  const int t0 = B.tile_off[r], t1 = B.tile_off[r + 1];
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int t = t0 + (int)threadIdx.x; t < t1; t += blockDim.x)
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] += tile_part[4 * (int64_t)t + q];
  block_partials<4>(v, sums, r);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (B.runs[r].c.collide) sbar[r] = sums[4 * r + 1];
    if (sums[4 * r + 3] >= 10.0) atomicOr(flags + r, 8);  // refusal limit (src/particles.c:603-605)
    if (r == 0) ++*dstep;  // the pass of this step has read it
  }
}

__global__ void k_batch_finalize(int64_t n4, unsigned long long* __restrict__ acc, double inv_scale,
                                 double* __restrict__ mom, int* flag) {
  int bad = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n4; c += (int64_t)gridDim.x * blockDim.x) {
    const long long a = (long long)acc[c];
    if (a > (1LL << 62) || a < -(1LL << 62)) bad = 1;
    mom[c] = (double)a * inv_scale;
    acc[c] = 0ull;
  }
  if (bad) atomicOr(flag, 1);
}

int tiles_of(const GridDesc& g) { return ((g.Nx + TX - 1) / TX) * ((g.Ny + TY - 1) / TY) * ((g.Nz + TZ - 1) / TZ); }

#undef TX
#undef TY
#undef TZ
#undef BX
#undef BY
#undef BZ
#undef BNODES

// ------------------------------------------------------------------ S at upload
__global__ void k_sbar_f64(F64Particles P, double vnT, double vn0x, double vn0y, double vn0z, double* part) {
  double s[1] = {0.0};
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < P.np; ip += (int64_t)gridDim.x * blockDim.x) {
    const double wx = P.vx[ip] - vn0x, wy = P.vy[ip] - vn0y, wz = P.vz[ip] - vn0z;
    s[0] += ch_gmean<double>(sqrt(wx * wx + wy * wy + wz * wz), vnT);
  }
  block_partials<1>(s, part);
}

__global__ void k_sbar_mixed(MixParticles P, float vnT, float vn0x, float vn0y, float vn0z, double* part) {
  double s[1] = {0.0};
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < P.np; ip += (int64_t)gridDim.x * blockDim.x) {
    const float4 v = P.vel[ip];
    s[0] += (double)g_fixed(ch_gmean<float>(ch_relspeed_rn(v.x, v.y, v.z, vn0x, vn0y, vn0z), vnT)) * CH_G_UNIT;
  }
  block_partials<1>(s, part);
}

// Fixed-order sum of per-block partials: out[q] = sum_b part[b*K + q].
__global__ void k_reduce_partials(const double* __restrict__ part, int nblocks, int K, double* out) {
  __shared__ double sm[32];
  for (int q = 0; q < K; ++q) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += part[(size_t)b * K + q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      double t = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (threadIdx.x == 0) out[q] = t;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ moments
// Fixed-point accumulators -> FP64 moments (SoA n, Gx, Gy, Gz), optional
// reset, block partials of the four global sums, and the range check: the
// density contributions are non-negative, so a wrapped sum shows up as a
// negative or near-limit value.
__global__ void k_finalize_moments(int64_t N, unsigned long long* __restrict__ acc, double inv_scale, int reset,
                                   double* __restrict__ mom, double* part, DevCounters* cnt) {
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  int bad = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long a = (long long)acc[q * N + c];
      if (q == 0 && (a < 0 || a > (1LL << 61))) bad = 1;
      const double v = (double)a * inv_scale;
      mom[q * N + c] = v;
      s[q] += v;
      if (reset) acc[q * N + c] = 0ull;
    }
  }
  if (bad) atomicOr(&cnt->range_error, 1);
  block_partials<4>(s, part);
}

// ------------------------------------------------------------------ counting sort
// key = natural cell index (k*Ny + j)*Nx + i of the ion's current cell.
__device__ __forceinline__ uint32_t key_f64(const GridDesc& g, double x, double y, double z) {
  int i, j, k;
  double f;
  locate(x, g.x0, g.dx, g.Nx, &i, &f);
  locate(y, g.y0, g.dy, g.Ny, &j, &f);
  locate(z, g.z0, g.dz, g.Nz, &k, &f);
  return (uint32_t)(((int64_t)k * g.Ny + j) * g.Nx + i);
}
__device__ __forceinline__ uint32_t key_mixed(const GridDesc& g, float w) {
  const uint32_t cell = __float_as_uint(w);
  const uint32_t i = cell & (CH_MAX_NX - 1), j = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1),
                 k = cell >> (CH_PACK_BX + CH_PACK_BY);
  return (k * (uint32_t)g.Ny + j) * (uint32_t)g.Nx + i;
}

__global__ void k_hist_f64(GridDesc g, F64Particles P, uint32_t* counts, uint32_t* keys) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_pad = (P.np + 31) / 32 * 32;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < n_pad; ip += stride) {
    const bool act = ip < P.np;
    uint32_t key = 0;
    if (act) key = key_f64(g, P.x[ip], P.y[ip], P.z[ip]);
    agg_inc(counts, key, act);
    if (act) keys[ip] = key;
  }
}

__global__ void k_hist_mixed(GridDesc g, MixParticles P, uint32_t* counts, uint32_t* keys) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_pad = (P.np + 31) / 32 * 32;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < n_pad; ip += stride) {
    const bool act = ip < P.np;
    uint32_t key = 0;
    if (act) key = key_mixed(g, P.pos[ip].w);
    agg_inc(counts, key, act);
    if (act) keys[ip] = key;
  }
}

__global__ void k_scatter_f64(F64Particles P, F64Particles Q, const uint32_t* __restrict__ keys, uint32_t* cursor) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_pad = (P.np + 31) / 32 * 32;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < n_pad; ip += stride) {
    const bool act = ip < P.np;
    const uint32_t key = act ? keys[ip] : 0u;
    const uint32_t dst = agg_inc(cursor, key, act);
    if (act) {
      Q.x[dst] = P.x[ip]; Q.y[dst] = P.y[ip]; Q.z[dst] = P.z[ip];
      Q.vx[dst] = P.vx[ip]; Q.vy[dst] = P.vy[ip]; Q.vz[dst] = P.vz[ip];
      Q.id[dst] = P.id[ip];
    }
  }
}

__global__ void k_scatter_mixed(GridDesc g, MixParticles P, MixParticles Q, uint32_t* cursor) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_pad = (P.np + 31) / 32 * 32;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < n_pad; ip += stride) {
    const bool act = ip < P.np;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    if (act) p = P.pos[ip];
    const uint32_t key = act ? key_mixed(g, p.w) : 0u;
    const uint32_t dst = agg_inc(cursor, key, act);
    if (act) {
      Q.pos[dst] = p;
      Q.vel[dst] = P.vel[ip];
    }
  }
}

// Exclusive scan of counts[0..n) into starts[0..n] (three phases).

__global__ void k_scan_blocks(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t* block_sums,
                              int64_t n) {
  __shared__ uint32_t sm[1024];
  const int64_t base = (int64_t)blockIdx.x * 1024;
  const int t = threadIdx.x;  // 512 threads, 2 items each
  uint32_t a = base + 2 * t < n ? in[base + 2 * t] : 0u;
  uint32_t b = base + 2 * t + 1 < n ? in[base + 2 * t + 1] : 0u;
  sm[2 * t] = a;
  sm[2 * t + 1] = b;
  // Blelloch up-sweep / down-sweep
  int off = 1;
  for (int d = 512; d > 0; d >>= 1) {
    __syncthreads();
    if (t < d) {
      const int ai = off * (2 * t + 1) - 1, bi = off * (2 * t + 2) - 1;
      sm[bi] += sm[ai];
    }
    off <<= 1;
  }
  if (t == 0) {
    block_sums[blockIdx.x] = sm[1023];
    sm[1023] = 0;
  }
  for (int d = 1; d < 1024; d <<= 1) {
    off >>= 1;
    __syncthreads();
    if (t < d) {
      const int ai = off * (2 * t + 1) - 1, bi = off * (2 * t + 2) - 1;
      const uint32_t tmp = sm[ai];
      sm[ai] = sm[bi];
      sm[bi] += tmp;
    }
  }
  __syncthreads();
  if (base + 2 * t < n) out[base + 2 * t] = sm[2 * t];
  if (base + 2 * t + 1 < n) out[base + 2 * t + 1] = sm[2 * t + 1];
}

__global__ void k_scan_sums(uint32_t* block_sums, int nb, uint32_t* total) {
  // single block, serial over chunks of 1024 with a running offset
  __shared__ uint32_t sm[1024];
  uint32_t run = 0;
  for (int base = 0; base < nb; base += 1024) {
    const int t = threadIdx.x;
    const int idx = base + t;
    const uint32_t v = idx < nb ? block_sums[idx] : 0u;
    sm[t] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const uint32_t add = t >= off ? sm[t - off] : 0u;
      __syncthreads();
      sm[t] += add;
      __syncthreads();
    }
    if (idx < nb) block_sums[idx] = run + sm[t] - v;  // exclusive
    const uint32_t chunk = sm[1023];
    __syncthreads();
    run += chunk;
  }
  if (threadIdx.x == 0) *total = run;
}

__global__ void k_scan_add(uint32_t* out, const uint32_t* block_sums, int64_t n, uint32_t* cursor) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const uint32_t v = out[i] + block_sums[i / 1024];
    out[i] = v;
    cursor[i] = v;
  }
}

__global__ void k_batch_hist(BatchDev B, MixParticles P, uint32_t* counts) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_pad = (P.np + 31) / 32 * 32;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < n_pad; ip += stride) {
    const bool act = ip < P.np;
    uint32_t key = 0u;
    if (act) {
      int lo = 0, hi = B.nruns;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (B.ion_off[mid] <= ip) lo = mid; else hi = mid;
      }
      const BatchRunDev& R = B.runs[lo];
      key = (uint32_t)R.node_off + key_mixed(R.c.g, P.pos[ip].w);
    }
    agg_inc(counts, key, act);
  }
}

__global__ void k_batch_scatter(BatchDev B, MixParticles P, MixParticles Q, uint32_t* cursor) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_pad = (P.np + 31) / 32 * 32;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < n_pad; ip += stride) {
    const bool act = ip < P.np;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t key = 0u;
    if (act) {
      p = P.pos[ip];
      int lo = 0, hi = B.nruns;  // run of slot ip
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (B.ion_off[mid] <= ip) lo = mid; else hi = mid;
      }
      const BatchRunDev& R = B.runs[lo];
      key = (uint32_t)R.node_off + key_mixed(R.c.g, p.w);
    }
    const uint32_t dst = agg_inc(cursor, key, act);
    if (act) {
      Q.pos[dst] = p;
      Q.vel[dst] = P.vel[ip];
    }
  }
}

// ------------------------------------------------------------------ launchers
int grid_for(int64_t n, int threads, int sms, int per_sm) {
  int64_t need = (n + threads - 1) / threads;
  int64_t cap = (int64_t)sms * per_sm;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

void launch_load(bool mixed, const GridDesc& g, const ch_loader& L, uint64_t seed, uint32_t run, F64Particles P,
                 MixParticles M, int sms, cudaStream_t s) {
  const uint32_t lo = (uint32_t)seed, hi = (uint32_t)(seed >> 32);
  if (mixed) k_load_mixed<<<grid_for(M.np, 256, sms, 8), 256, 0, s>>>(g, L, lo, hi, run, M), ::ch::note_launch();
  else k_load_f64<<<grid_for(P.np, 256, sms, 8), 256, 0, s>>>(g, L, lo, hi, run, P), ::ch::note_launch();
}

// dst <- src in 16-byte words (bytes a multiple of 16, both 16-byte
// aligned); dst may be mapped host memory.  Four independent words per
// thread and iteration keep enough bytes in flight for the host link.
__global__ void k_stream_copy(uint4* __restrict__ dst, const uint4* __restrict__ src, int64_t n16) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n16; i += stride) dst[i] = src[i];
}

// Host AoS (16-byte aligned, e.g. mapped host memory) -> mixed state:
// 16-byte loads, two ions per thread and iteration in flight.
__global__ void k_aos_to_mixed_u16(GridDesc g, const double2* __restrict__ pos, const double2* __restrict__ vel,
                                   MixParticles P) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.np; i += stride) {
    const double2 p0 = pos[2 * i], p1 = pos[2 * i + 1], v0 = vel[2 * i], v1 = vel[2 * i + 1];
    const double s[3] = {p0.x, p0.y, p1.x};
    P.pos[i] = pack_mixed(g, s);
    P.vel[i] = make_float4((float)v0.x, (float)v0.y, (float)v1.x, __uint_as_float((uint32_t)i));
  }
}

__global__ void k_aos_to_f64_u16(const double2* __restrict__ pos, const double2* __restrict__ vel, F64Particles P) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.np; i += stride) {
    const double2 p0 = pos[2 * i], p1 = pos[2 * i + 1], v0 = vel[2 * i], v1 = vel[2 * i + 1];
    P.x[i] = p0.x; P.y[i] = p0.y; P.z[i] = p1.x;
    P.vx[i] = v0.x; P.vy[i] = v0.y; P.vz[i] = v1.x;
    P.id[i] = (uint32_t)i;
  }
}

// ------------------------------------------------------------------ host arrays in ion-id order
// slot_of_id[id] = the slot that holds ion id.
__global__ void k_slot_map(MixParticles P, uint32_t* __restrict__ slot_of_id) {
  const float* vw = reinterpret_cast<const float*>(P.vel) + 3;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < P.np; s += (int64_t)gridDim.x * blockDim.x)
    slot_of_id[__float_as_uint(vw[4 * s])] = (uint32_t)s;
}

// Mixed state -> AoS arrays (4 doubles per ion) in id order, ids
// [i_begin, i_end): warp w converts ions i0 .. i0+31 (read from their slots)
// into shared memory and then writes them out as 512 contiguous bytes per
// instruction.
__global__ void __launch_bounds__(256) k_mixed_to_host(GridDesc g, MixParticles P,
                                                       const uint32_t* __restrict__ slot_of_id,
                                                       double2* __restrict__ pos, double2* __restrict__ vel,
                                                       int64_t i_begin, int64_t i_end) {
  __shared__ double2 bp[8][64], bv[8][64];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i0 = i_begin + (blockIdx.x * (int64_t)(blockDim.x >> 5) + w) * 32; i0 < i_end; i0 += nw * 32) {
    const int64_t i = i0 + lane;
    if (i < i_end) {
      const uint32_t s = slot_of_id[i];
      const float4 p = P.pos[s], v = P.vel[s];
      const uint32_t cell = __float_as_uint(p.w);
      const int ci = cell & (CH_MAX_NX - 1), cj = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1),
                ck = cell >> (CH_PACK_BX + CH_PACK_BY);
      bp[w][2 * lane] = make_double2(g.x0 + ((double)ci + (double)p.x) * g.dx, g.y0 + ((double)cj + (double)p.y) * g.dy);
      bp[w][2 * lane + 1] = make_double2(g.z0 + ((double)ck + (double)p.z) * g.dz, 0.0);
      bv[w][2 * lane] = make_double2((double)v.x, (double)v.y);
      bv[w][2 * lane + 1] = make_double2((double)v.z, 0.0);
    }
    __syncwarp();
    const int64_t n2 = 2 * (i_end - i0 < 32 ? i_end - i0 : 32);  // 16-byte words of this chunk
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int q = lane + 32 * h;
      if (q < n2) {
        pos[2 * i0 + q] = bp[w][q];
        vel[2 * i0 + q] = bv[w][q];
      }
    }
    __syncwarp();  // the buffers are written out before the next chunk refills them
  }
}

// Host AoS arrays in id order -> mixed state, each ion back into the slot it
// had (slot_of_id), so that the order of the ions, and with it the brick
// ranges of the last sort, stay as they were.  Reads as k_mixed_to_host
// writes: 512 contiguous bytes per warp instruction.
__global__ void __launch_bounds__(256) k_host_to_mixed(GridDesc g, const double2* __restrict__ pos,
                                                       const double2* __restrict__ vel,
                                                       const uint32_t* __restrict__ slot_of_id, MixParticles P) {
  __shared__ double2 bp[8][64], bv[8][64];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i0 = (blockIdx.x * (int64_t)(blockDim.x >> 5) + w) * 32; i0 < P.np; i0 += nw * 32) {
    const int64_t n2 = 2 * (P.np - i0 < 32 ? P.np - i0 : 32);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int q = lane + 32 * h;
      if (q < n2) {
        bp[w][q] = pos[2 * i0 + q];
        bv[w][q] = vel[2 * i0 + q];
      }
    }
    __syncwarp();
    const int64_t i = i0 + lane;
    if (i < P.np) {
      const double2 p0 = bp[w][2 * lane], p1 = bp[w][2 * lane + 1], v0 = bv[w][2 * lane], v1 = bv[w][2 * lane + 1];
      const double sx[3] = {p0.x, p0.y, p1.x};
      const uint32_t s = slot_of_id[i];
      P.pos[s] = pack_mixed(g, sx);
      P.vel[s] = make_float4((float)v0.x, (float)v0.y, (float)v1.x, __uint_as_float((uint32_t)i));
    }
    __syncwarp();
  }
}

// One step's push, collisions and move of ions held by the host in id order
// (registered RealVector arrays, read and written in place over the host
// link).  Warp w takes ions i0 .. i0+31: with `read` its lanes load the
// chunk's 1 KB of positions and velocities one chunk ahead (in registers,
// so the next chunk travels over the link while this one is pushed), put it
// in shared memory, pack each ion into the mixed form and keep a copy in B
// (the ions as uploaded); otherwise they take the ions from their slots in
// P.  Each lane then pushes its ion with the arithmetic of the tiled pass
// (tile_gather_global, tile_boris, the same collision draws and rounds,
// tile_move_ion), stores it back into its slot of P for the deposit and,
// with `write`, puts the FP64 result into shared memory, which the warp
// writes out over the link 512 contiguous bytes per instruction.  The link
// carries the upload and the download at once (about 1.6x the rate of one
// direction).  Block partials: the expected events, S of the pushed
// velocities (for the next step) and S of the velocities read, integer sums
// of 2^-20 units, exact in any order.
__global__ void __launch_bounds__(256, 2) k_host_push(StepConsts c, double2* pos, double2* vel,
                                                      const uint32_t* __restrict__ slot_of_id, MixParticles P,
                                                      MixParticles B, const float4* __restrict__ E, float pscale,
                                                      uint32_t* hist, int read, int write, DevCounters* cnt,
                                                      double* part) {
  __shared__ double2 bp[8][64], bv[8][64];
  const GridDesc& g = c.g;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  const bool cross = !(c.faithful & CH_FAITHFUL_D2);
  const bool move = !(c.faithful & CH_FAITHFUL_D5);
  float tsum = 0.0f;
  unsigned long long gsum = 0ull, ssum = 0ull;
  unsigned ncol = 0, nref = 0;
  double2 rp0 = make_double2(0.0, 0.0), rp1 = rp0, rv0 = rp0, rv1 = rp0;
  auto fetch = [&](int64_t c0) {
    if (read && c0 < P.np) {
      const int64_t m2 = 2 * (P.np - c0 < 32 ? P.np - c0 : 32);
      if (lane < m2) { rp0 = pos[2 * c0 + lane]; rv0 = vel[2 * c0 + lane]; }
      if (lane + 32 < m2) { rp1 = pos[2 * c0 + lane + 32]; rv1 = vel[2 * c0 + lane + 32]; }
    }
  };
  int64_t i0 = (blockIdx.x * (int64_t)(blockDim.x >> 5) + w) * 32;
  fetch(i0);
  for (; i0 < P.np; i0 += nw * 32) {
    const int64_t n2 = 2 * (P.np - i0 < 32 ? P.np - i0 : 32);  // 16-byte words of this chunk
    if (read) {
      if (lane < n2) { bp[w][lane] = rp0; bv[w][lane] = rv0; }
      if (lane + 32 < n2) { bp[w][lane + 32] = rp1; bv[w][lane + 32] = rv1; }
      fetch(i0 + nw * 32);
    }
    __syncwarp();
    const int64_t ia = i0 + lane;
    const bool active = ia < P.np;
    uint32_t slot = 0;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f), vv = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
      slot = slot_of_id[ia];
      if (read) {
        const double2 p0 = bp[w][2 * lane], p1 = bp[w][2 * lane + 1], v0 = bv[w][2 * lane], v1 = bv[w][2 * lane + 1];
        const double sx[3] = {p0.x, p0.y, p1.x};
        p = pack_mixed(g, sx);
        vv = make_float4((float)v0.x, (float)v0.y, (float)v1.x, __uint_as_float((uint32_t)ia));
        B.pos[slot] = p;
        B.vel[slot] = vv;
      } else {
        p = P.pos[slot];
        vv = P.vel[slot];
      }
    }
    const uint32_t cell = __float_as_uint(p.w);
    int i = cell & (CH_MAX_NX - 1), j = (cell >> CH_PACK_BX) & (CH_MAX_NY - 1), k = cell >> (CH_PACK_BX + CH_PACK_BY);
    float v[3] = {vv.x, vv.y, vv.z};
    if (active) {
      if (read && c.collide) ssum += g_fixed(tile_gmean(c, v));
      float4 e000, e100, e010, e110, e001, e101, e011, e111;
      tile_gather_global(g, E, i, j, k, e000, e100, e010, e110, e001, e101, e011, e111);
      tile_boris(c, e000, e100, e010, e110, e001, e101, e011, e111, p, cross, v);
      if (c.collide) {
        const float gi = tile_gmean(c, v);
        float nd = 1.0f;
        if (c.nn_profile == CH_NN_GAUSSIAN_X)
          nd = ch_neutral_density<float>(c, (float)(g.x0 + ((double)i + (double)p.x) * g.dx));
        const float lscale = pscale * nd;
        const float lam = lscale * gi;
        tsum += lam;
        const uint32_t id = __float_as_uint(vv.w);
        const U4 r0 = ch_philox(id, c.step, CH_PURPOSE_COLLIDE << 24, c.run, c.seed_lo, c.seed_hi);
        const float u0 = ch_unitf(r0.x);
        bool defer = false;
        float qt = 0.0f;
        if (lam > 0.0f && u0 > __expf(-lam)) {
          qt = ch_qdiv(-ch_log(u0), lam);
          defer = qt < 1.0f;
        }
        if (defer) {
          // the event process of the tiled pass's rings, run to its end here
          uint32_t qe = 0, qit = 0;
          float gf = 0.0f;
          while (!ch_collide_round<float>(c, id, lscale, v, qt, qe, qit, &ncol, &nref, gf)) {
          }
          gsum += g_fixed(gf);
        } else {
          gsum += g_fixed(gi);
        }
      }
      vv.x = v[0]; vv.y = v[1]; vv.z = v[2];
      if (move) tile_move_ion(c, p, v, i, j, k);
      P.pos[slot] = p;
      P.vel[slot] = vv;
    }
    if (hist) {
      const uint32_t rk = agg_inc(hist, (uint32_t)(((int64_t)k * g.Ny + j) * g.Nx + i), active);
      if (active && P.rank) P.rank[slot] = rk;
    }
    __syncwarp();  // every lane has read its ion from the buffers before they are refilled
    if (write) {
      if (active) {
        const uint32_t cw = __float_as_uint(p.w);
        const int ci = cw & (CH_MAX_NX - 1), cj = (cw >> CH_PACK_BX) & (CH_MAX_NY - 1),
                  ck = cw >> (CH_PACK_BX + CH_PACK_BY);
        bp[w][2 * lane] = make_double2(g.x0 + ((double)ci + (double)p.x) * g.dx, g.y0 + ((double)cj + (double)p.y) * g.dy);
        bp[w][2 * lane + 1] = make_double2(g.z0 + ((double)ck + (double)p.z) * g.dz, 0.0);
        bv[w][2 * lane] = make_double2((double)vv.x, (double)vv.y);
        bv[w][2 * lane + 1] = make_double2((double)vv.z, 0.0);
      }
      __syncwarp();
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = lane + 32 * h;
        if (q < n2) {
          pos[2 * i0 + q] = bp[w][q];
          vel[2 * i0 + q] = bv[w][q];
        }
      }
    }
    __syncwarp();  // the buffers are written out before the next chunk refills them
  }
  double vs[3] = {(double)tsum, (double)gsum * CH_G_UNIT, (double)ssum * CH_G_UNIT};
  count_add(cnt, ncol, nref);
  block_partials<3>(vs, part);
}

int launch_host_push(const StepConsts& c, void* pos, void* vel, const uint32_t* slot_of_id, MixParticles M,
                     MixParticles B, const float4* E32, double Nc, double sbar, uint32_t* hist, bool read, bool write,
                     DevCounters* cnt, double* part, int sms, cudaStream_t s) {
  const float pscale = sbar > 0.0 ? (float)(Nc / sbar) : 0.0f;
  const int nb = grid_for(M.np, 256, sms, 4);
  k_host_push<<<nb, 256, 0, s>>>(c, (double2*)pos, (double2*)vel, slot_of_id, M, B, E32, pscale, hist, read ? 1 : 0,
                                 write ? 1 : 0, cnt, part),
      ::ch::note_launch();
  return nb;
}

void launch_slot_map(MixParticles M, uint32_t* slot_of_id, int sms, cudaStream_t s) {
  k_slot_map<<<grid_for(M.np, 256, sms, 8), 256, 0, s>>>(M, slot_of_id), ::ch::note_launch();
}
void launch_mixed_to_host(const GridDesc& g, MixParticles M, const uint32_t* slot_of_id, void* pos, void* vel,
                          int64_t i_begin, int64_t i_end, int sms, cudaStream_t s) {
  k_mixed_to_host<<<grid_for(i_end - i_begin, 256, sms, 8), 256, 0, s>>>(
      g, M, slot_of_id, static_cast<double2*>(pos), static_cast<double2*>(vel), i_begin, i_end),
      ::ch::note_launch();
}
void launch_host_to_mixed(const GridDesc& g, const void* pos, const void* vel, const uint32_t* slot_of_id,
                          MixParticles M, int sms, cudaStream_t s) {
  k_host_to_mixed<<<grid_for(M.np, 256, sms, 8), 256, 0, s>>>(g, static_cast<const double2*>(pos),
                                                                      static_cast<const double2*>(vel), slot_of_id, M),
      ::ch::note_launch();
}

void launch_aos_in_u16(bool mixed, const GridDesc& g, const void* pos, const void* vel, F64Particles P,
                       MixParticles M, int sms, cudaStream_t s) {
  const double2* p = static_cast<const double2*>(pos);
  const double2* v = static_cast<const double2*>(vel);
  if (mixed) k_aos_to_mixed_u16<<<grid_for(M.np, 256, sms, 16), 256, 0, s>>>(g, p, v, M), ::ch::note_launch();
  else k_aos_to_f64_u16<<<grid_for(P.np, 256, sms, 16), 256, 0, s>>>(p, v, P), ::ch::note_launch();
}

void launch_stream_copy(void* dst, const void* src, uint64_t bytes, int sms, cudaStream_t s) {
  const int64_t n16 = (int64_t)(bytes / 16);
  k_stream_copy<<<grid_for(n16, 256, sms, 8), 256, 0, s>>>(static_cast<uint4*>(dst), static_cast<const uint4*>(src),
                                                           n16), ::ch::note_launch();
}

void launch_aos_in(bool mixed, const GridDesc& g, const double4_32a* pos, const double4_32a* vel, F64Particles P,
                   MixParticles M, int sms, cudaStream_t s) {
  if (mixed) k_aos_to_mixed<<<grid_for(M.np, 256, sms, 8), 256, 0, s>>>(g, pos, vel, M), ::ch::note_launch();
  else k_aos_to_f64<<<grid_for(P.np, 256, sms, 8), 256, 0, s>>>(pos, vel, P), ::ch::note_launch();
}

void launch_aos_out(bool mixed, const GridDesc& g, F64Particles P, MixParticles M, double4_32a* pos, double4_32a* vel,
                    int sms, cudaStream_t s) {
  if (mixed) k_mixed_to_aos<<<grid_for(M.np, 256, sms, 8), 256, 0, s>>>(g, M, pos, vel), ::ch::note_launch();
  else k_f64_to_aos<<<grid_for(P.np, 256, sms, 8), 256, 0, s>>>(P, pos, vel), ::ch::note_launch();
}

void launch_node_efield(bool mixed, const GridDesc& g, double tscale, const double* phi, double* E64, float4* E32,
                        int sms, cudaStream_t s) {
  if (mixed)
    k_node_efield_mixed<<<grid_for(g.N, 256, sms, 8), 256, 0, s>>>(g, -tscale / (2.0 * g.dx), -tscale / (2.0 * g.dy),
                                                                   -tscale / (2.0 * g.dz), phi, E32),
        ::ch::note_launch();
  else k_node_efield_f64<<<grid_for(g.N, 256, sms, 8), 256, 0, s>>>(g, phi, E64), ::ch::note_launch();
}

// The tiled pass needs more than the default 48 KB of dynamic shared memory;
// the attribute is set once per device and instantiation.
template <int PH, bool SCAT = false>
static void tiled_smem_attr() {
  static std::atomic<uint32_t> done{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const uint32_t bit = 1u << (dev & 31);
  if (done.load() & bit) return;
  // a failure here surfaces as the launch error of the pass
  if (cudaFuncSetAttribute(k_pass_tiled<PH, SCAT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)tile_smem_bytes<PH>()) == cudaSuccess)
    done.fetch_or(bit);
}

template <int PH>
static int pass_one(bool mixed, const StepConsts& c, F64Particles P, MixParticles M, const double* E64,
                    const float4* E32, const double* phi, unsigned long long* acc, double Nc, double sbar,
                    DevCounters* cnt, double* part, const uint32_t* starts, uint32_t* hist, int sms,
                    cudaStream_t s) {
  const int64_t np = mixed ? M.np : P.np;
  int nb = grid_for(np, 256, sms, 8);
  if (mixed) {
    if constexpr (PH == PH_DEPOSIT || !(PH & PH_DEPOSIT)) {  // launch_pass splits the rest
    const float pscale = sbar > 0.0 ? (float)(Nc / sbar) : 0.0f;
    const int ntiles = ((c.g.Nx + 15) / 16) * ((c.g.Ny + 3) / 4) * ((c.g.Nz + 3) / 4);
    const int per_sm = (PH & PH_DEPOSIT) ? CH_DEP_CTAS : CH_PUSH_CTAS;
    nb = ntiles < per_sm * sms ? ntiles : per_sm * sms;
    const int s2 = (int)lround(log2(c.dep_scale));
    tiled_smem_attr<PH>();
    k_pass_tiled<PH><<<nb, 256, tile_smem_bytes<PH>(), s>>>(c, M, E32, starts, acc, pscale, s2 - CH_TILE_DLOG2,
                                                         s2 - CH_TILE_FLOG2, cnt, part, hist, MixParticles{},
                                                         (const uint32_t*)nullptr),
        ::ch::note_launch();
    }
  } else {
    // the queue of colliding ions (18 KB of shared memory) only with the push
    const size_t smem = (PH & PH_PUSH) ? sizeof(F64Queue) : 0;
    if (smem) {
      static bool attr = false;
      if (!attr) {
        cudaFuncSetAttribute(k_pass_f64<PH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
      }
    }
    k_pass_f64<PH><<<nb, 256, smem, s>>>(c, P, E64, phi, acc, Nc, sbar, cnt, part), ::ch::note_launch();
  }
  return nb;
}

int launch_pass(bool mixed, int phases, const StepConsts& c, F64Particles P, MixParticles M, const double* E64,
                const float4* E32, const double* phi, unsigned long long* acc, double Nc, double sbar,
                DevCounters* cnt, double* part, const uint32_t* starts, uint32_t* hist, int sms, cudaStream_t s) {
  // the mixed pass deposits in a launch of its own (the push / move launch
  // writes the block partials, so its grid size is returned)
  if (mixed && (phases & PH_DEPOSIT) && (phases & (PH_PUSH | PH_MOVE))) {
    const int nb = launch_pass(mixed, phases & (PH_PUSH | PH_MOVE), c, P, M, E64, E32, phi, acc, Nc, sbar, cnt, part,
                               starts, hist, sms, s);
    launch_pass(mixed, PH_DEPOSIT, c, P, M, E64, E32, phi, acc, Nc, sbar, cnt, part, starts, nullptr, sms, s);
    return nb;
  }
#define CH_PASS(PHV) pass_one<PHV>(mixed, c, P, M, E64, E32, phi, acc, Nc, sbar, cnt, part, starts, hist, sms, s)
  switch (phases) {
    case PH_PUSH: return CH_PASS(PH_PUSH);
    case PH_MOVE: return CH_PASS(PH_MOVE);
    case PH_DEPOSIT: return CH_PASS(PH_DEPOSIT);
    case PH_MOVE | PH_DEPOSIT: return CH_PASS(PH_MOVE | PH_DEPOSIT);
    case PH_PUSH | PH_MOVE: return CH_PASS(PH_PUSH | PH_MOVE);
    default: return CH_PASS(PH_PUSH | PH_MOVE | PH_DEPOSIT);
  }
#undef CH_PASS
}

int launch_sbar(bool mixed, const StepConsts& c, F64Particles P, MixParticles M, double* part, int sms,
                cudaStream_t s) {
  const int64_t np = mixed ? M.np : P.np;
  const int nb = grid_for(np, 256, sms, 8);
  if (mixed)
    k_sbar_mixed<<<nb, 256, 0, s>>>(M, (float)c.vnT, (float)c.vn0[0], (float)c.vn0[1], (float)c.vn0[2], part), ::ch::note_launch();
  else
    k_sbar_f64<<<nb, 256, 0, s>>>(P, c.vnT, c.vn0[0], c.vn0[1], c.vn0[2], part), ::ch::note_launch();
  return nb;
}

void launch_reduce_partials(const double* part, int nblocks, int K, double* out, cudaStream_t s) {
  k_reduce_partials<<<1, 256, 0, s>>>(part, nblocks, K, out), ::ch::note_launch();
}

int launch_finalize(int64_t N, unsigned long long* acc, double inv_scale, int reset, double* mom, double* part,
                    DevCounters* cnt, int sms, cudaStream_t s) {
  const int nb = grid_for(N, 256, sms, 4);
  k_finalize_moments<<<nb, 256, 0, s>>>(N, acc, inv_scale, reset, mom, part, cnt), ::ch::note_launch();
  return nb;
}

// Exclusive scan of counts into starts (starts[N] = total); cursor gets a
// copy of starts.
void launch_scan(int64_t N, const uint32_t* counts, uint32_t* starts, uint32_t* cursor, uint32_t* block_sums,
                 cudaStream_t s) {
  const int nsb = (int)((N + 1023) / 1024);
  k_scan_blocks<<<nsb, 512, 0, s>>>(counts, starts, block_sums, N), ::ch::note_launch();
  k_scan_sums<<<1, 1024, 0, s>>>(block_sums, nsb, starts + N), ::ch::note_launch();
  k_scan_add<<<(int)((N + 255) / 256), 256, 0, s>>>(starts, block_sums, N, cursor), ::ch::note_launch();
}

// The deposit of a step that ends with a sort: ions read in the order of
// `starts` are deposited and written to Q in the order of dst_starts (the
// scan of the push's cell count, with the ions' ranks in M.rank).
void launch_deposit_sort(const StepConsts& c, MixParticles M, MixParticles MQ, const uint32_t* starts,
                         const uint32_t* dst_starts, unsigned long long* acc, DevCounters* cnt, int sms,
                         cudaStream_t s) {
  const int ntiles = ((c.g.Nx + 15) / 16) * ((c.g.Ny + 3) / 4) * ((c.g.Nz + 3) / 4);
  const int nb = ntiles < CH_DEP_CTAS * sms ? ntiles : CH_DEP_CTAS * sms;
  const int s2 = (int)lround(log2(c.dep_scale));
  tiled_smem_attr<PH_DEPOSIT, true>();
  k_pass_tiled<PH_DEPOSIT, true><<<nb, 256, tile_smem_bytes<PH_DEPOSIT>(), s>>>(
      c, M, (const float4*)nullptr, starts, acc, 0.0f, s2 - CH_TILE_DLOG2, s2 - CH_TILE_FLOG2, cnt, (double*)nullptr,
      (uint32_t*)nullptr, MQ, dst_starts),
      ::ch::note_launch();
}

void launch_sort(bool mixed, const GridDesc& g, F64Particles P, F64Particles Q, MixParticles M, MixParticles MQ,
                 uint32_t* counts, uint32_t* starts, uint32_t* cursor, uint32_t* keys, uint32_t* block_sums, int sms,
                 cudaStream_t s) {
  const int64_t np = mixed ? M.np : P.np;
  const int64_t N = g.N;
  const int nb = grid_for(np, 256, sms, 8);
  cudaMemsetAsync(counts, 0, sizeof(uint32_t) * N, s);
  if (mixed) k_hist_mixed<<<nb, 256, 0, s>>>(g, M, counts, keys), ::ch::note_launch();
  else k_hist_f64<<<nb, 256, 0, s>>>(g, P, counts, keys), ::ch::note_launch();
  const int nsb = (int)((N + 1023) / 1024);
  k_scan_blocks<<<nsb, 512, 0, s>>>(counts, starts, block_sums, N), ::ch::note_launch();
  k_scan_sums<<<1, 1024, 0, s>>>(block_sums, nsb, starts + N), ::ch::note_launch();
  k_scan_add<<<(int)((N + 255) / 256), 256, 0, s>>>(starts, block_sums, N, cursor), ::ch::note_launch();
  if (mixed) k_scatter_mixed<<<nb, 256, 0, s>>>(g, M, MQ, cursor), ::ch::note_launch();
  else k_scatter_f64<<<nb, 256, 0, s>>>(P, Q, keys, cursor), ::ch::note_launch();
}

// ------------------------------------------------------------------ ensemble launchers
template <int PH, bool SCAT = false>
static void batch_smem_attr() {
  static std::atomic<uint32_t> done{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const uint32_t bit = 1u << (dev & 31);
  if (done.load() & bit) return;
  if (cudaFuncSetAttribute(k_batch_pass<PH, SCAT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)tile_smem_bytes<PH>()) == cudaSuccess)
    done.fetch_or(bit);
}

void batch_pass_prepare() {
  batch_smem_attr<PH_PUSH | PH_MOVE>();
  batch_smem_attr<PH_DEPOSIT>();
  batch_smem_attr<PH_DEPOSIT, true>();
}

void launch_batch_pass(int phases, const BatchDev& B, const uint32_t* dstep, MixParticles P, const float4* E,
                       const uint32_t* starts, unsigned long long* acc, const double* sbar, int dep_log2,
                       uint32_t* hist, double* tile_part, int* flags, int ctas_per_sm, int sms, cudaStream_t s,
                       MixParticles Q, const uint32_t* dst_starts) {
  const int sd = dep_log2 - CH_TILE_DLOG2, sf = dep_log2 - CH_TILE_FLOG2;
  auto grid = [&](int per_sm) { return B.total_tiles < per_sm * sms ? B.total_tiles : per_sm * sms; };
  // the deposit is a launch of its own
  if (phases & (PH_PUSH | PH_MOVE)) {
    k_batch_pass<PH_PUSH | PH_MOVE><<<grid(CH_PUSH_CTAS), 256, tile_smem_bytes<PH_PUSH | PH_MOVE>(), s>>>(
        B, dstep, P, E, starts, acc, sbar, sd, sf, hist, tile_part, flags, MixParticles{}, nullptr),
        ::ch::note_launch();
  }
  if (phases & PH_DEPOSIT) {
    const int nb = grid(ctas_per_sm < 1 ? 1 : ctas_per_sm);
    if (dst_starts)
      k_batch_pass<PH_DEPOSIT, true><<<nb, 256, tile_smem_bytes<PH_DEPOSIT>(), s>>>(
          B, dstep, P, E, starts, acc, sbar, sd, sf, nullptr, tile_part, flags, Q, dst_starts),
          ::ch::note_launch();
    else
      k_batch_pass<PH_DEPOSIT><<<nb, 256, tile_smem_bytes<PH_DEPOSIT>(), s>>>(
          B, dstep, P, E, starts, acc, sbar, sd, sf, nullptr, tile_part, flags, MixParticles{}, nullptr),
          ::ch::note_launch();
  }
}

void launch_batch_runsum(const BatchDev& B, const double* tile_part, double* sums, double* sbar, int* flags,
                         uint32_t* dstep, cudaStream_t s) {
  k_batch_runsum<<<B.nruns, 256, 0, s>>>(B, tile_part, sums, sbar, flags, dstep), ::ch::note_launch();
}

void launch_batch_hist(const BatchDev& B, MixParticles M, uint32_t* counts, int sms, cudaStream_t s) {
  k_batch_hist<<<grid_for(M.np, 256, sms, 8), 256, 0, s>>>(B, M, counts), ::ch::note_launch();
}

void launch_batch_finalize(int64_t n4, unsigned long long* acc, double inv_scale, double* mom, int* flag, int sms,
                           cudaStream_t s) {
  k_batch_finalize<<<grid_for(n4, 256, sms, 4), 256, 0, s>>>(n4, acc, inv_scale, mom, flag), ::ch::note_launch();
}

void launch_batch_sort(const BatchDev& B, int64_t Ntot, MixParticles M, MixParticles MQ, uint32_t* counts,
                       uint32_t* starts, uint32_t* cursor, uint32_t* block_sums, int sms, cudaStream_t s) {
  const int nsb = (int)((Ntot + 1023) / 1024);
  k_scan_blocks<<<nsb, 512, 0, s>>>(counts, starts, block_sums, Ntot), ::ch::note_launch();
  k_scan_sums<<<1, 1024, 0, s>>>(block_sums, nsb, starts + Ntot), ::ch::note_launch();
  k_scan_add<<<(int)((Ntot + 255) / 256), 256, 0, s>>>(starts, block_sums, Ntot, cursor), ::ch::note_launch();
  k_batch_scatter<<<grid_for(M.np, 256, sms, 8), 256, 0, s>>>(B, M, MQ, cursor), ::ch::note_launch();
}

}  // namespace ch
