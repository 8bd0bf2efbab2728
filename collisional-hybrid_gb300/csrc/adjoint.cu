// adjoint.cu -- discrete adjoint of the FP64 step (ch_adjoint_*).
//
// The model: ions loaded with density perturbation amplitude `amp`, then
// per step s: node field E = -D phi_s, trilinear gather, Boris push,
// ion-neutral collisions, move, CIC deposit, potential solve A(n) phi = P b(n,
// Gamma, E0).  Parameters theta = (E0, vn0, amp).  The collision events of a
// recorded run -- which ions collide, how often, their neutral velocity
// offset V - vn0 and scattering draws, refusals -- are frozen: a replay at
// another theta applies the same events with V = vn0 + offset, so the model
// is a smooth function of theta and central differences converge.
//
// The reverse sweep walks the steps backwards.  Per step it solves the
// transposed operator (A is symmetric for kappa_e = 0, so the same multigrid
// CG), forms the adjoints of the RHS and of A(n) with respect to the
// moments, and runs one ion kernel that recomputes the step's push,
// collisions and move from the stored pre-step state and pulls the adjoints
// back through deposit, move, scatter (Jacobian by forward-mode duals),
// Boris and gather.  Ion states are checkpointed every k steps; a segment is
// recomputed (ions only: phi and the moments of every step are kept) before
// it is reversed.
#include <math.h>
#include <string.h>

#include <new>
#include <vector>

#include "ion_dev.cuh"
#include "particles.cuh"
#include "physics.cuh"
#include "solver_dev.cuh"

using namespace ch;

ch_status ch_fail(ch_status code, const char* fmt, ...);
ch_status ch_cuda_fail(cudaError_t e, const char* what, const char* file, int line);

namespace {

constexpr int ADJ_MAX_EVENTS = CH_MAX_EVENTS;

// One frozen collision event.  Events of one ion in one step are linked
// through `next` from first[ion].
struct AdjEvent {
  double n[3];       // neutral velocity offset V - vn0
  double uz, uphi;   // scattering draws (cos theta*, azimuth / 2 pi)
  int32_t next;
  uint32_t flags;    // 1: refused (no velocity change)
};

// ---------------------------------------------------------------- duals
// Value and derivatives along three seed directions.
struct D3 {
  double v, d[3];
};
__device__ __forceinline__ D3 dconst(double a) { return D3{a, {0.0, 0.0, 0.0}}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return D3{a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return D3{a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) {
  return D3{a.v * b.v, {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1], a.d[2] * b.v + a.v * b.d[2]}};
}
__device__ __forceinline__ D3 operator*(double s, D3 a) { return D3{s * a.v, {s * a.d[0], s * a.d[1], s * a.d[2]}}; }
__device__ __forceinline__ D3 operator/(D3 a, D3 b) {
  const double q = a.v / b.v;
  return D3{q, {(a.d[0] - q * b.d[0]) / b.v, (a.d[1] - q * b.d[1]) / b.v, (a.d[2] - q * b.d[2]) / b.v}};
}
__device__ __forceinline__ D3 dsqrt(D3 a) {
  const double r = sqrt(a.v);
  const double k = r > 0.0 ? 0.5 / r : 0.0;
  return D3{r, {k * a.d[0], k * a.d[1], k * a.d[2]}};
}
__device__ __forceinline__ double val(double a) { return a; }
__device__ __forceinline__ double val(D3 a) { return a.v; }
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }

// g(vr) = (mn/M) |vr| Rot(vr) u: the relative part of the centre-of-mass
// scatter (src/particles.c:552-591), u = (uperp cos 2pi uphi, uperp sin 2pi
// uphi, uz) rotated so that z maps onto the direction of vr.  The scattered
// velocity is vc + g(v - V), vc = (mi v + mn V) / M.
template <typename T>
__device__ __forceinline__ void scatter_rel(const T vr[3], double ux, double uy, double uz, double fac, T g[3]) {
  const T r2 = vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2];
  const T r = dsqrt(r2);
  const T rho = dsqrt(vr[0] * vr[0] + vr[1] * vr[1]);
  if (val(rho) > 0.0) {
    const T costht = vr[2] / r, sintht = rho / r;
    const T cosphi = vr[0] / rho, sinphi = vr[1] / rho;
    const T ux1 = uz * sintht + ux * costht, uz1 = uz * costht - ux * sintht;
    const T ux2 = ux1 * cosphi - uy * sinphi, uy2 = ux1 * sinphi + uy * cosphi;
    g[0] = fac * (r * ux2); g[1] = fac * (r * uy2); g[2] = fac * (r * uz1);
  } else {
    // vr along z (measure zero): sintht = 0, cosphi = 1
    const double cz = val(r) > 0.0 ? (val(vr[2]) > 0.0 ? 1.0 : -1.0) : 1.0;
    g[0] = fac * (r * (ux * cz)); g[1] = fac * (r * uy); g[2] = fac * (r * (uz * cz));
  }
}
__device__ __forceinline__ D3 operator*(D3 a, double s) { return s * a; }
__device__ __forceinline__ D3 operator+(D3 a, double s) { return D3{a.v + s, {a.d[0], a.d[1], a.d[2]}}; }

__device__ __forceinline__ void unit_u(double uz, double uphi, double* ux, double* uy) {
  const double up = sqrt(fmax(0.0, 1.0 - uz * uz));
  double s, c;
  sincos(2.0 * CH_PI * uphi, &s, &c);
  *ux = up * c;
  *uy = up * s;
}

// Scattered velocity of one event (value only).
__device__ __forceinline__ void scatter_apply(double v[3], const double V[3], double uz, double uphi, double mi,
                                              double mn) {
  const double M = mi + mn;
  double ux, uy;
  unit_u(uz, uphi, &ux, &uy);
  const double vr[3] = {v[0] - V[0], v[1] - V[1], v[2] - V[2]};
  double g[3];
  scatter_rel<double>(vr, ux, uy, uz, mn / M, g);
  for (int d = 0; d < 3; ++d) v[d] = (mi * v[d] + mn * V[d]) / M + g[d];
}

// Vector-Jacobian product of one event: given vbar (adjoint of the scattered
// velocity), returns the adjoint of the pre-event velocity in vbar and adds
// the adjoint of V (= of vn0) to Vbar.
__device__ __forceinline__ void scatter_vjp(const double v[3], const double V[3], double uz, double uphi, double mi,
                                            double mn, double vbar[3], double Vbar[3]) {
  const double M = mi + mn;
  double ux, uy;
  unit_u(uz, uphi, &ux, &uy);
  D3 vr[3];
  for (int d = 0; d < 3; ++d) {
    vr[d] = dconst(v[d] - V[d]);
    vr[d].d[d] = 1.0;
  }
  D3 g[3];
  scatter_rel<D3>(vr, ux, uy, uz, mn / M, g);
  double jt[3];  // J_g^T vbar
  for (int q = 0; q < 3; ++q) jt[q] = g[0].d[q] * vbar[0] + g[1].d[q] * vbar[1] + g[2].d[q] * vbar[2];
  for (int q = 0; q < 3; ++q) {
    Vbar[q] += (mn / M) * vbar[q] - jt[q];
    vbar[q] = (mi / M) * vbar[q] + jt[q];
  }
}

// Trilinear weights of a position: cell (i, j, k), corner weights W[8]
// (corner q: bit 0 x, bit 1 y, bit 2 z) and their gradients dW[8][3].
struct Cic {
  int i, j, k;
  double W[8], dW[8][3];
};
__device__ __forceinline__ void cic(const GridDesc& g, double x, double y, double z, Cic& c) {
  const double X = (x - g.x0) / g.dx, Y = (y - g.y0) / g.dy, Z = (z - g.z0) / g.dz;
  const double fi = floor(X), fj = floor(Y), fk = floor(Z);
  const double wx = X - fi, wy = Y - fj, wz = Z - fk;
  c.i = ch_wrap((int)fi, g.Nx); c.j = ch_wrap((int)fj, g.Ny); c.k = ch_wrap((int)fk, g.Nz);
  for (int q = 0; q < 8; ++q) {
    const double ax = (q & 1) ? wx : 1.0 - wx, ay = (q & 2) ? wy : 1.0 - wy, az = (q & 4) ? wz : 1.0 - wz;
    const double sx = (q & 1) ? 1.0 : -1.0, sy = (q & 2) ? 1.0 : -1.0, sz = (q & 4) ? 1.0 : -1.0;
    c.W[q] = ax * ay * az;
    c.dW[q][0] = sx * ay * az / g.dx;
    c.dW[q][1] = ax * sy * az / g.dy;
    c.dW[q][2] = ax * ay * sz / g.dz;
  }
}
__device__ __forceinline__ int64_t corner_node(const GridDesc& g, const Cic& c, int q) {
  const int i = (q & 1) ? (c.i + 1 == g.Nx ? 0 : c.i + 1) : c.i;
  const int j = (q & 2) ? (c.j + 1 == g.Ny ? 0 : c.j + 1) : c.j;
  const int k = (q & 4) ? (c.k + 1 == g.Nz ? 0 : c.k + 1) : c.k;
  return ((int64_t)k * g.Ny + j) * g.Nx + i;
}

// Trilinear gather of the node field (3 x N SoA), the order of the FP64 pass.
__device__ __forceinline__ void gather_E(const GridDesc& g, const double* E, double x, double y, double z,
                                         double Ef[3]) {
  const double X = (x - g.x0) / g.dx, Y = (y - g.y0) / g.dy, Z = (z - g.z0) / g.dz;
  const double fi = floor(X), fj = floor(Y), fk = floor(Z);
  const double wx = X - fi, wy = Y - fj, wz = Z - fk;
  const int i = ch_wrap((int)fi, g.Nx), j = ch_wrap((int)fj, g.Ny), k = ch_wrap((int)fk, g.Nz);
  const int i1 = i + 1 == g.Nx ? 0 : i + 1, j1 = j + 1 == g.Ny ? 0 : j + 1, k1 = k + 1 == g.Nz ? 0 : k + 1;
  const int64_t c000 = ((int64_t)k * g.Ny + j) * g.Nx + i, c100 = ((int64_t)k * g.Ny + j) * g.Nx + i1,
                c010 = ((int64_t)k * g.Ny + j1) * g.Nx + i, c110 = ((int64_t)k * g.Ny + j1) * g.Nx + i1,
                c001 = ((int64_t)k1 * g.Ny + j) * g.Nx + i, c101 = ((int64_t)k1 * g.Ny + j) * g.Nx + i1,
                c011 = ((int64_t)k1 * g.Ny + j1) * g.Nx + i, c111 = ((int64_t)k1 * g.Ny + j1) * g.Nx + i1;
  for (int d = 0; d < 3; ++d) {
    const double* e = E + d * g.N;
    const double wll = e[c000] + wy * (e[c010] - e[c000]);
    const double wlh = e[c100] + wy * (e[c110] - e[c100]);
    const double whl = e[c001] + wy * (e[c011] - e[c001]);
    const double whh = e[c101] + wy * (e[c111] - e[c101]);
    const double ezl = wll + wx * (wlh - wll);
    const double ezh = whl + wx * (whh - whl);
    Ef[d] = ezl + wz * (ezh - ezl);
  }
}

// Poisson event process of one ion (as ch_collide<double>), recording every
// event.  Returns false when the event pool overflowed.
__device__ bool collide_record(const StepConsts& c, uint32_t id, double lscale, double v[3], AdjEvent* ev,
                               unsigned* ev_count, unsigned cap, int32_t* first_slot) {
  const double sig = c.vnT, m1 = c.m1, mi = c.mi, mn = c.mn;
  double t = 0.0;
  int32_t prev = -1;
  for (uint32_t e = 0; e < ADJ_MAX_EVENTS; ++e) {
    const double wx = v[0] - c.vn0[0], wy = v[1] - c.vn0[1], wz = v[2] - c.vn0[2];
    const double w = sqrt(wx * wx + wy * wy + wz * wz);
    const double lam = lscale * ch_gmean<double>(w, sig);
    if (!(lam > 0.0)) break;
    const U4 r0 = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8), c.run, c.seed_lo, c.seed_hi);
    t += -log(ch_unit(r0.x)) / lam;
    if (!(t < 1.0)) break;
    double n[3] = {0.0, 0.0, 0.0}, uz = 0.0, uphi = 0.0;
    bool ok = false;
    for (uint32_t it = 0; it < 64 && !ok; ++it) {
      const U4 a = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8) | (1 + 2 * it), c.run, c.seed_lo,
                             c.seed_hi);
      const U4 b = ch_philox(id, c.step, (CH_PURPOSE_COLLIDE << 24) | (e << 8) | (2 + 2 * it), c.run, c.seed_lo,
                             c.seed_hi);
      if (ch_unit(a.x) * (w + m1) < w) {
        double s1, c1, s2, c2;
        const double r1 = sqrt(-2.0 * log(ch_unit(a.y)));
        sincos(2.0 * CH_PI * ch_unit(a.z), &s1, &c1);
        const double r2 = sqrt(-2.0 * log(ch_unit(a.w)));
        sincos(2.0 * CH_PI * ch_unit(b.x), &s2, &c2);
        n[0] = sig * (r1 * c1); n[1] = sig * (r1 * s1); n[2] = sig * (r2 * c2);
      } else {
        const double sp = sig * sqrt(-2.0 * log(ch_unit(a.y) * ch_unit(a.z)));
        const double ct = 2.0 * ch_unit(a.w) - 1.0;
        const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
        double sph, cph;
        sincos(2.0 * CH_PI * ch_unit(b.x), &sph, &cph);
        n[0] = sp * st * cph; n[1] = sp * st * sph; n[2] = sp * ct;
      }
      const double V[3] = {c.vn0[0] + n[0], c.vn0[1] + n[1], c.vn0[2] + n[2]};
      const double dV = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      const double rx = v[0] - V[0], ry = v[1] - V[1], rz = v[2] - V[2];
      if (ch_unit(b.y) * (w + dV) < sqrt(rx * rx + ry * ry + rz * rz)) {
        ok = true;
        uz = 2.0 * ch_unit(b.z) - 1.0;
        uphi = ch_unit(b.w);
      }
    }
    uint32_t flags = ok ? 0u : 1u;
    if (ok) {
      const double V[3] = {c.vn0[0] + n[0], c.vn0[1] + n[1], c.vn0[2] + n[2]};
      double vf[3] = {v[0], v[1], v[2]};
      scatter_apply(vf, V, uz, uphi, mi, mn);
      const double vfr = sqrt(vf[0] * vf[0] + vf[1] * vf[1] + vf[2] * vf[2]);
      if (vfr / c.viTr > 10.0) flags = 1u;  // refused (src/particles.c:597-606)
      else { v[0] = vf[0]; v[1] = vf[1]; v[2] = vf[2]; }
    }
    const unsigned slot = atomicAdd(ev_count, 1u);
    if (slot >= cap) return false;
    AdjEvent& E = ev[slot];
    E.n[0] = n[0]; E.n[1] = n[1]; E.n[2] = n[2];
    E.uz = uz; E.uphi = uphi; E.next = -1; E.flags = flags;
    if (prev < 0) *first_slot = (int32_t)slot;
    else ev[prev].next = (int32_t)slot;
    prev = (int32_t)slot;
  }
  return true;
}

enum { ADJ_RECORD = 0, ADJ_REPLAY = 1, ADJ_RECOMPUTE = 2 };

// One forward step of every ion.  RECORD draws and stores the events,
// REPLAY applies stored ones (and deposits), RECOMPUTE replays without the
// deposit (rebuilding pre-step states of a segment).  part (block partials,
// K = 2): sum of v_x after the step, sum of g for the next step's S.
template <int MODE>
__global__ void __launch_bounds__(256) k_adj_fwd(StepConsts c, F64Particles P, const double* __restrict__ E,
                                                 unsigned long long* __restrict__ acc, AdjEvent* ev,
                                                 unsigned* ev_count, unsigned cap, int32_t* __restrict__ first,
                                                 double Nc, const double* __restrict__ S, double* part, int* err) {
  const GridDesc& g = c.g;
  double vs[2] = {0.0, 0.0};
  int overflow = 0;
  const double pscale = (MODE == ADJ_RECORD && *S > 0.0) ? Nc / *S : 0.0;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < P.np; ip += (int64_t)gridDim.x * blockDim.x) {
    double x = P.x[ip], y = P.y[ip], z = P.z[ip];
    double v[3] = {P.vx[ip], P.vy[ip], P.vz[ip]};
    double Ef[3];
    gather_E(g, E, x, y, z, Ef);
    if (c.push_E0) { Ef[0] += c.E0[0]; Ef[1] += c.E0[1]; Ef[2] += c.E0[2]; }
    ch_boris<double>(c, Ef, v);
    if (c.collide) {
      if (MODE == ADJ_RECORD) {
        int32_t f = -1;
        const double wx = v[0] - c.vn0[0], wy = v[1] - c.vn0[1], wz = v[2] - c.vn0[2];
        const double lscale = pscale * ch_neutral_density<double>(c, x);
        const double lam = lscale * ch_gmean<double>(sqrt(wx * wx + wy * wy + wz * wz), c.vnT);
        const U4 r0 = ch_philox((uint32_t)ip, c.step, CH_PURPOSE_COLLIDE << 24, c.run, c.seed_lo, c.seed_hi);
        if (lam > 0.0 && -log(ch_unit(r0.x)) / lam < 1.0)
          if (!collide_record(c, (uint32_t)ip, lscale, v, ev, ev_count, cap, &f)) overflow = 1;
        first[ip] = f;
        const double qx = v[0] - c.vn0[0], qy = v[1] - c.vn0[1], qz = v[2] - c.vn0[2];
        vs[1] += ch_gmean<double>(sqrt(qx * qx + qy * qy + qz * qz), c.vnT);
      } else {
        for (int32_t e = first[ip]; e >= 0; e = ev[e].next) {
          const AdjEvent& A = ev[e];
          if (A.flags & 1u) continue;
          const double V[3] = {c.vn0[0] + A.n[0], c.vn0[1] + A.n[1], c.vn0[2] + A.n[2]};
          scatter_apply(v, V, A.uz, A.uphi, c.mi, c.mn);
        }
      }
    }
    vs[0] += v[0];
    x = wrap_pos(x + v[0] * c.dt, g.x0, g.Lx);
    y = wrap_pos(y + v[1] * c.dt, g.y0, g.Ly);
    z = wrap_pos(z + v[2] * c.dt, g.z0, g.Lz);
    P.x[ip] = x; P.y[ip] = y; P.z[ip] = z;
    P.vx[ip] = v[0]; P.vy[ip] = v[1]; P.vz[ip] = v[2];
    if (MODE != ADJ_RECOMPUTE) {
      const double X = (x - g.x0) / g.dx, Y = (y - g.y0) / g.dy, Z = (z - g.z0) / g.dz;
      const double fi = floor(X), fj = floor(Y), fk = floor(Z);
      deposit_cic<double>(g, acc, ch_wrap((int)fi, g.Nx), ch_wrap((int)fj, g.Ny), ch_wrap((int)fk, g.Nz), X - fi,
                          Y - fj, Z - fk, v[0], v[1], v[2], c.dep_scale);
    }
  }
  if (overflow) atomicOr(err, 1);
  partials<2>(vs, part);
}

// Node part of the reverse of one solve: lam solves A lam = P phibar (mean
// free).  nbar, Gbar: adjoints of the moments; part (K = 3): sum lam D_d n.
__global__ void __launch_bounds__(256) k_adj_node(GridDesc g, DevCoefs<double> C, double E0x, double E0y,
                                                  double E0z, double cth, double cG, const double* __restrict__ n,
                                                  const double* __restrict__ phi, const double* __restrict__ lam,
                                                  double* __restrict__ nbar, double* __restrict__ Gbar,
                                                  double* part) {
  double e0[3] = {0.0, 0.0, 0.0};
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < g.N; m += (int64_t)gridDim.x * blockDim.x) {
    const Nb b = neighbours(g, m);
    const double Dx = (lam[b.e] - lam[b.w]) / (2.0 * g.dx), Dy = (lam[b.n] - lam[b.s]) / (2.0 * g.dy),
                 Dz = (lam[b.u] - lam[b.d]) / (2.0 * g.dz);
    const double lc = lam[m];
    const double Ll = (lam[b.e] - 2.0 * lc + lam[b.w]) / (g.dx * g.dx) +
                      (lam[b.n] - 2.0 * lc + lam[b.s]) / (g.dy * g.dy) +
                      (lam[b.u] - 2.0 * lc + lam[b.d]) / (g.dz * g.dz);
    const double pc = phi[m];
    // -(d (A(n) phi) / d n)^T lam: each face term s (n_f + n_c)(phi_f - phi_c)
    const double op = C.sxx * ((lc - lam[b.e]) * (phi[b.e] - pc) + (lc - lam[b.w]) * (phi[b.w] - pc)) +
                      C.syy * ((lc - lam[b.n]) * (phi[b.n] - pc) + (lc - lam[b.s]) * (phi[b.s] - pc)) +
                      C.szz * ((lc - lam[b.u]) * (phi[b.u] - pc) + (lc - lam[b.d]) * (phi[b.d] - pc));
    nbar[m] = -(E0x * Dx + E0y * Dy + E0z * Dz) + cth * Ll - op;
    Gbar[m] = -cG * Dx;
    Gbar[g.N + m] = -cG * Dy;
    Gbar[2 * g.N + m] = -cG * Dz;
    e0[0] += lc * (n[b.e] - n[b.w]) / (2.0 * g.dx);
    e0[1] += lc * (n[b.n] - n[b.s]) / (2.0 * g.dy);
    e0[2] += lc * (n[b.u] - n[b.d]) / (2.0 * g.dz);
  }
  partials<3>(e0, part);
}

// phibar = D^T(-Ebar) = sum_d D_d Ebar_d, plus w phi (the objective's
// mean-square term).
__global__ void k_adj_phibar(GridDesc g, const double* __restrict__ Ebar, const double* __restrict__ phi, double w,
                             double* __restrict__ out) {
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < g.N; m += (int64_t)gridDim.x * blockDim.x) {
    const Nb b = neighbours(g, m);
    const double* Ex = Ebar;
    const double* Ey = Ebar + g.N;
    const double* Ez = Ebar + 2 * g.N;
    out[m] = (Ex[b.e] - Ex[b.w]) / (2.0 * g.dx) + (Ey[b.n] - Ey[b.s]) / (2.0 * g.dy) +
             (Ez[b.u] - Ez[b.d]) / (2.0 * g.dz) + w * phi[m];
  }
}

// Reverse of one ion step.  In: the pre-step state (X_s, V_s), the adjoints
// of the post-step state in Xb/Vb and of its moments (nbar, Gbar), the
// objective's flux weight for the post-step velocity.  Out: adjoints of the
// pre-step state in Xb/Vb, the node-field adjoint Ebar (accumulated), part
// (K = 6): vn0bar (3), E0bar through the push (3, push_E0 only).
__global__ void __launch_bounds__(256) k_adj_ion(StepConsts c, const double* __restrict__ RbT, F64Particles P,
                                                 const double* __restrict__ E, const AdjEvent* __restrict__ ev,
                                                 const int32_t* __restrict__ first, const double* __restrict__ nbar,
                                                 const double* __restrict__ Gbar, double vxw, double* Xb, double* Yb,
                                                 double* Zb, double* VXb, double* VYb, double* VZb, double* Ebar,
                                                 double* part) {
  const GridDesc& g = c.g;
  const int64_t N = g.N;
  double acc6[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const double tau = c.tscale;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < P.np; ip += (int64_t)gridDim.x * blockDim.x) {
    const double x = P.x[ip], y = P.y[ip], z = P.z[ip];
    double v[3] = {P.vx[ip], P.vy[ip], P.vz[ip]};
    // ---- recompute the step
    double Ef[3];
    gather_E(g, E, x, y, z, Ef);
    if (c.push_E0) { Ef[0] += c.E0[0]; Ef[1] += c.E0[1]; Ef[2] += c.E0[2]; }
    ch_boris<double>(c, Ef, v);
    double vpre[ADJ_MAX_EVENTS][3];
    int32_t eid[ADJ_MAX_EVENTS];
    int ne = 0;
    if (c.collide) {
      for (int32_t e = first[ip]; e >= 0 && ne < ADJ_MAX_EVENTS; e = ev[e].next) {
        const AdjEvent& A = ev[e];
        if (A.flags & 1u) continue;
        vpre[ne][0] = v[0]; vpre[ne][1] = v[1]; vpre[ne][2] = v[2];
        eid[ne++] = e;
        const double V[3] = {c.vn0[0] + A.n[0], c.vn0[1] + A.n[1], c.vn0[2] + A.n[2]};
        scatter_apply(v, V, A.uz, A.uphi, c.mi, c.mn);
      }
    }
    const double x1 = wrap_pos(x + v[0] * c.dt, g.x0, g.Lx), y1 = wrap_pos(y + v[1] * c.dt, g.y0, g.Ly),
                 z1 = wrap_pos(z + v[2] * c.dt, g.z0, g.Lz);
    // ---- adjoint of the post-step state: deposit and objective
    double xb[3] = {Xb[ip], Yb[ip], Zb[ip]};
    double vb[3] = {VXb[ip] + vxw, VYb[ip], VZb[ip]};
    {
      Cic q;
      cic(g, x1, y1, z1, q);
      for (int k = 0; k < 8; ++k) {
        const int64_t nd = corner_node(g, q, k);
        const double gx = Gbar[nd], gy = Gbar[N + nd], gz = Gbar[2 * N + nd];
        vb[0] += q.W[k] * gx; vb[1] += q.W[k] * gy; vb[2] += q.W[k] * gz;
        const double s = nbar[nd] + v[0] * gx + v[1] * gy + v[2] * gz;
        xb[0] += q.dW[k][0] * s; xb[1] += q.dW[k][1] * s; xb[2] += q.dW[k][2] * s;
      }
    }
    // ---- move: x1 = x + dt v
    for (int d = 0; d < 3; ++d) vb[d] += c.dt * xb[d];
    // ---- collisions, last event first
    for (int k = ne - 1; k >= 0; --k) {
      const AdjEvent& A = ev[eid[k]];
      const double V[3] = {c.vn0[0] + A.n[0], c.vn0[1] + A.n[1], c.vn0[2] + A.n[2]};
      scatter_vjp(vpre[k], V, A.uz, A.uphi, c.mi, c.mn, vb, acc6);
    }
    // ---- Boris: vB = Rb (v + tau E) + tau E
    double vbs[3], Eb[3];
    for (int r = 0; r < 3; ++r) vbs[r] = RbT[3 * r] * vb[0] + RbT[3 * r + 1] * vb[1] + RbT[3 * r + 2] * vb[2];
    for (int d = 0; d < 3; ++d) Eb[d] = tau * (vbs[d] + vb[d]);
    if (c.push_E0) { acc6[3] += Eb[0]; acc6[4] += Eb[1]; acc6[5] += Eb[2]; }
    // ---- gather
    {
      Cic q;
      cic(g, x, y, z, q);
      for (int k = 0; k < 8; ++k) {
        const int64_t nd = corner_node(g, q, k);
        atomicAdd(Ebar + nd, q.W[k] * Eb[0]);
        atomicAdd(Ebar + N + nd, q.W[k] * Eb[1]);
        atomicAdd(Ebar + 2 * N + nd, q.W[k] * Eb[2]);
        const double s = E[nd] * Eb[0] + E[N + nd] * Eb[1] + E[2 * N + nd] * Eb[2];
        xb[0] += q.dW[k][0] * s; xb[1] += q.dW[k][1] * s; xb[2] += q.dW[k][2] * s;
      }
    }
    Xb[ip] = xb[0]; Yb[ip] = xb[1]; Zb[ip] = xb[2];
    VXb[ip] = vbs[0]; VYb[ip] = vbs[1]; VZb[ip] = vbs[2];
  }
  partials<6>(acc6, part);
}

// Deposit adjoint of the initial state (X_0 only; V_0 does not depend on
// theta) and the amplitude derivative: part (K = 1) sum Xbar dx0/damp.
__global__ void k_adj_initial(GridDesc g, F64Particles P, const double* __restrict__ nbar,
                              const double* __restrict__ Gbar, const double* __restrict__ Xb,
                              const double* __restrict__ dxda, double* part) {
  const int64_t N = g.N;
  double a[1] = {0.0};
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < P.np; ip += (int64_t)gridDim.x * blockDim.x) {
    Cic q;
    cic(g, P.x[ip], P.y[ip], P.z[ip], q);
    double xb = Xb[ip];
    for (int k = 0; k < 8; ++k) {
      const int64_t nd = corner_node(g, q, k);
      const double s = nbar[nd] + P.vx[ip] * Gbar[nd] + P.vy[ip] * Gbar[N + nd] + P.vz[ip] * Gbar[2 * N + nd];
      xb += q.dW[k][0] * s;
    }
    a[0] += xb * dxda[ip];
  }
  partials<1>(a, part);
}

// dx0/damp of the inverse-CDF loader: F(x) = x + sum_m a_m (cos p_m -
// cos(w_m x + p_m)) / w_m, so dx/da_1 = -(cos p_1 - cos(w_1 x + p_1)) / w_1
// / F'(x).
__global__ void k_adj_dxda(GridDesc g, ch_loader L, F64Particles P, double* dxda) {
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < P.np; ip += (int64_t)gridDim.x * blockDim.x) {
    const double x = P.x[ip] - g.x0;
    double dF = 1.0;
    for (int m = 1; m <= 3; ++m) {
      const double w = 2.0 * CH_PI * m / g.Lx;
      dF += L.amp[m - 1] * sin(w * x + L.phase[m - 1]);
    }
    const double w1 = 2.0 * CH_PI / g.Lx;
    dxda[ip] = -((cos(L.phase[0]) - cos(w1 * x + L.phase[0])) / w1) / dF;
  }
}

__global__ void k_adj_sum(int64_t N, const double* __restrict__ a, const double* __restrict__ b, double* part) {
  double s[2] = {0.0, 0.0};
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < N; m += (int64_t)gridDim.x * blockDim.x) {
    s[0] += a[m];
    s[1] += a[m] * (b ? b[m] : a[m]);
  }
  partials<2>(s, part);
}

__global__ void k_adj_sub(int64_t N, double* a, const double* mean_from, double scale) {
  const double mean = mean_from[0] * scale;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < N; m += (int64_t)gridDim.x * blockDim.x)
    a[m] -= mean;
}

int64_t collision_count(const ch_params& p, int64_t np) {
  const double viTr = sqrt(p.viT[0] * p.viT[0] + p.viT[1] * p.viT[1] + p.viT[2] * p.viT[2]);
  const double dvx = p.vi0[0] - p.vn0[0], dvy = p.vi0[1] - p.vn0[1], dvz = p.vi0[2] - p.vn0[2];
  const double vrm = 4.0 * viTr + sqrt(dvx * dvx + dvy * dvy + dvz * dvz);
  const double vn0r = sqrt(p.vn0[0] * p.vn0[0] + p.vn0[1] * p.vn0[1] + p.vn0[2] * p.vn0[2]);
  const double den = (p.vnT + vn0r) * sqrt(p.mn / p.mi);
  if (!(den > 0.0)) return np;
  const double v = ((double)np * p.nui * p.dt * vrm) / den;
  if (v >= (double)np) return np;
  if (v < 0.0) return 0;
  return (int64_t)v;
}

}  // namespace

struct ch_adjoint {
  ch_params p{};
  ch_loader L{};
  ch_adjoint_config cfg{};
  GridDesc g{};
  int64_t np = 0;
  int sms = 1, device = 0;
  cudaStream_t stream = nullptr;
  PotentialSolver solver;
  std::vector<void*> allocs;
  F64Particles cur{};                 // working state
  std::vector<F64Particles> ckpt;     // state s = k * checkpoint_every
  std::vector<F64Particles> seg;      // pre-step states of segment seg_holds
  int seg_holds = -1;
  double *phi_all = nullptr, *mom_all = nullptr;  // (nsteps + 1) x N, x 4N
  double *E64 = nullptr, *Ebar = nullptr, *phibar = nullptr, *lam = nullptr, *nbar = nullptr, *Gbar = nullptr,
         *rhs = nullptr, *dxda = nullptr, *RbT = nullptr;
  double *Xb[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  unsigned long long* acc = nullptr;
  DevCounters* cnt = nullptr;
  double *part = nullptr, *red = nullptr, *hred = nullptr;
  int* err = nullptr;
  AdjEvent* ev = nullptr;
  unsigned* ev_count = nullptr;
  unsigned ev_cap = 0;
  int32_t* first = nullptr;           // nsteps x np
  double theta_rec[CH_ADJ_NTHETA] = {0};
  bool recorded = false;
  double J_rec = 0.0;
  ch_adjoint_timing timing{};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int nb = 1;
};

template <typename T>
static T* adj_alloc(ch_adjoint* a, size_t n, cudaError_t* e) {
  void* p = nullptr;
  if (*e == cudaSuccess) *e = cudaMalloc(&p, sizeof(T) * (n ? n : 1));
  if (*e != cudaSuccess) return nullptr;
  a->allocs.push_back(p);
  return static_cast<T*>(p);
}

static F64Particles adj_state(ch_adjoint* a, cudaError_t* e) {
  F64Particles P{};
  P.x = adj_alloc<double>(a, a->np, e); P.y = adj_alloc<double>(a, a->np, e); P.z = adj_alloc<double>(a, a->np, e);
  P.vx = adj_alloc<double>(a, a->np, e); P.vy = adj_alloc<double>(a, a->np, e); P.vz = adj_alloc<double>(a, a->np, e);
  P.id = adj_alloc<uint32_t>(a, a->np, e);
  P.np = a->np;
  return P;
}

static void copy_state(F64Particles& dst, const F64Particles& src, cudaStream_t s) {
  const size_t b = sizeof(double) * src.np;
  cudaMemcpyAsync(dst.x, src.x, b, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(dst.y, src.y, b, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(dst.z, src.z, b, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(dst.vx, src.vx, b, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(dst.vy, src.vy, b, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(dst.vz, src.vz, b, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(dst.id, src.id, sizeof(uint32_t) * src.np, cudaMemcpyDeviceToDevice, s);
}

extern "C" ch_status ch_adjoint_destroy(ch_adjoint* a) {
  if (!a) return CH_OK;
  if (a->stream) cudaStreamSynchronize(a->stream);
  a->solver.release();
  for (void* p : a->allocs) cudaFree(p);
  if (a->hred) cudaFreeHost(a->hred);
  if (a->e0) cudaEventDestroy(a->e0);
  if (a->e1) cudaEventDestroy(a->e1);
  if (a->stream) cudaStreamDestroy(a->stream);
  delete a;
  return CH_OK;
}

extern "C" ch_status ch_adjoint_create(const ch_params* p, int64_t np, const ch_loader* L,
                                       const ch_adjoint_config* cfg, int32_t device, ch_adjoint** out) {
  if (!p || !L || !cfg || !out || np < 1) return ch_fail(CH_ERR_ARG, "ch_adjoint_create: bad arguments");
  *out = nullptr;
  if (cfg->nsteps < 1 || cfg->checkpoint_every < 1 || cfg->window < 1 || cfg->window > cfg->nsteps)
    return ch_fail(CH_ERR_ARG, "adjoint: need nsteps >= 1, checkpoint_every >= 1, 1 <= window <= nsteps");
  if (p->kappa_e[0] != 0.0 || p->kappa_e[1] != 0.0 || p->kappa_e[2] != 0.0)
    return ch_fail(CH_ERR_UNSUPPORTED, "adjoint: kappa_e must be 0 (the transposed solve reuses the symmetric CG)");
  if (p->lhs_type != CH_LHS_FULL || p->rhs_type != CH_RHS_FULL || p->faithful != 0)
    return ch_fail(CH_ERR_UNSUPPORTED, "adjoint: full LHS/RHS, no as-written defects");
  if (p->nn_profile != CH_NN_UNIFORM) return ch_fail(CH_ERR_UNSUPPORTED, "adjoint: uniform neutral density");
  if (np > 0xFFFFFFFFll) return ch_fail(CH_ERR_ARG, "at most 2^32-1 ions");
  if (p->Nx < 3 || p->Ny < 3 || p->Nz < 3 || (int64_t)p->Nx * p->Ny * p->Nz >= (1LL << 31))
    return ch_fail(CH_ERR_ARG, "adjoint: grid %dx%dx%d (at least 3 and at most 2^31-1 nodes)", p->Nx, p->Ny, p->Nz);
  if (device >= 0) CH_CUDA_OK(cudaSetDevice(device));
  ch_adjoint* a = new (std::nothrow) ch_adjoint();
  if (!a) return ch_fail(CH_ERR_NOMEM, "host allocation");
  a->p = *p;
  a->p.precision = CH_FP64;
  a->p.ksp_type = CH_KSP_CG;
  a->p.pc_type = CH_PC_MG;
  a->L = *L;
  a->cfg = *cfg;
  a->np = np;
  CH_CUDA_OK(cudaGetDevice(&a->device));
  CH_CUDA_OK(cudaDeviceGetAttribute(&a->sms, cudaDevAttrMultiProcessorCount, a->device));
  cudaError_t e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&a->e1);
  GridDesc& g = a->g;
  g.Nx = p->Nx; g.Ny = p->Ny; g.Nz = p->Nz;
  ch_grid_finish(g);
  g.x0 = p->x0; g.y0 = p->y0; g.z0 = p->z0;
  g.Lx = p->x1 - p->x0; g.Ly = p->y1 - p->y0; g.Lz = p->z1 - p->z0;
  g.dx = g.Lx / p->Nx; g.dy = g.Ly / p->Ny; g.dz = g.Lz / p->Nz;
  const int64_t N = g.N;
  const int S = cfg->nsteps, K = cfg->checkpoint_every;
  const int nck = (S + K - 1) / K;
  a->cur = adj_state(a, &e);
  for (int k = 0; k < nck; ++k) a->ckpt.push_back(adj_state(a, &e));
  for (int k = 0; k < K; ++k) a->seg.push_back(adj_state(a, &e));
  a->phi_all = adj_alloc<double>(a, (size_t)(S + 1) * N, &e);
  a->mom_all = adj_alloc<double>(a, (size_t)(S + 1) * 4 * N, &e);
  a->E64 = adj_alloc<double>(a, 3 * N, &e);
  a->Ebar = adj_alloc<double>(a, 3 * N, &e);
  a->phibar = adj_alloc<double>(a, N, &e);
  a->lam = adj_alloc<double>(a, N, &e);
  a->nbar = adj_alloc<double>(a, N, &e);
  a->Gbar = adj_alloc<double>(a, 3 * N, &e);
  a->rhs = adj_alloc<double>(a, N, &e);
  a->dxda = adj_alloc<double>(a, np, &e);
  a->RbT = adj_alloc<double>(a, 9, &e);
  for (auto& q : a->Xb) q = adj_alloc<double>(a, np, &e);
  a->acc = adj_alloc<unsigned long long>(a, 4 * N, &e);
  a->cnt = adj_alloc<DevCounters>(a, 1, &e);
  a->nb = grid_for(np > N ? np : N, 256, a->sms, 8);
  a->part = adj_alloc<double>(a, (size_t)a->nb * 8, &e);
  a->red = adj_alloc<double>(a, 16, &e);
  a->err = adj_alloc<int>(a, 1, &e);
  // frozen events: Nc per step with margin
  const double nc = p->mn > 0.0 ? (double)collision_count(*p, np) : 0.0;
  const double capd = (double)S * (1.5 * nc + 4096.0);
  a->ev_cap = (unsigned)(capd < 4.0e9 ? capd : 4.0e9);
  a->ev = adj_alloc<AdjEvent>(a, a->ev_cap, &e);
  a->ev_count = adj_alloc<unsigned>(a, 1, &e);
  a->first = adj_alloc<int32_t>(a, (size_t)S * np, &e);
  if (e == cudaSuccess) e = cudaMallocHost(&a->hred, sizeof(double) * 16);
  if (e != cudaSuccess) {
    ch_adjoint_destroy(a);
    return ch_cuda_fail(e, "ch_adjoint_create", __FILE__, __LINE__);
  }
  ch_status rc = a->solver.init(a->p, g, a->sms);
  if (rc) { ch_adjoint_destroy(a); return rc; }
  *out = a;
  return CH_OK;
}

static StepConsts adj_consts(const ch_adjoint* a, const double* theta, int64_t step) {
  const ch_params& p = a->p;
  StepConsts k;
  memset(&k, 0, sizeof(k));
  k.g = a->g;
  k.tscale = 0.5 * (p.qi / p.mi) * p.dt;
  double tt = 0.0;
  for (int d = 0; d < 3; ++d) { k.t[d] = k.tscale * p.B0[d]; tt += k.t[d] * k.t[d]; }
  for (int d = 0; d < 3; ++d) k.s[d] = 2.0 * k.t[d] / (1.0 + tt);
  for (int d = 0; d < 3; ++d) k.E0[d] = theta[d];
  k.push_E0 = p.push_E0;
  k.dt = p.dt;
  k.collide = p.mn > 0.0;
  k.vnT = p.vnT;
  for (int d = 0; d < 3; ++d) k.vn0[d] = theta[3 + d];
  k.mi = p.mi;
  k.mn = p.mn;
  k.viTr = sqrt(p.viT[0] * p.viT[0] + p.viT[1] * p.viT[1] + p.viT[2] * p.viT[2]);
  k.m1 = 2.0 * p.vnT * sqrt(2.0 / CH_PI);
  k.nn_profile = CH_NN_UNIFORM;
  k.seed_lo = (uint32_t)p.seed;
  k.seed_hi = (uint32_t)(p.seed >> 32);
  k.run = p.run;
  k.step = (uint32_t)step;
  // fixed-point scale 2^50: the deposit's rounding (2^-50 per contribution)
  // stays far below the changes of a finite-difference step; densities up to
  // 8192 per node keep within the int64 range
  k.dep_scale = ldexp(1.0, 50);
  ch_consts_finish(k);
  return k;
}

// Transpose of the Boris map vB = Rb v- (src/particles.c:374-447), Rb = I +
// C_s (I + C_t) with C_a x = x cross a.
static void boris_rbt(const StepConsts& k, double RbT[9]) {
  double Rb[9];
  for (int col = 0; col < 3; ++col) {
    double e[3] = {0.0, 0.0, 0.0};
    e[col] = 1.0;
    const double q[3] = {e[0] + (e[1] * k.t[2] - e[2] * k.t[1]), e[1] + (e[2] * k.t[0] - e[0] * k.t[2]),
                         e[2] + (e[0] * k.t[1] - e[1] * k.t[0])};
    const double r[3] = {e[0] + (q[1] * k.s[2] - q[2] * k.s[1]), e[1] + (q[2] * k.s[0] - q[0] * k.s[2]),
                         e[2] + (q[0] * k.s[1] - q[1] * k.s[0])};
    for (int row = 0; row < 3; ++row) Rb[3 * row + col] = r[row];
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) RbT[3 * r + c] = Rb[3 * c + r];
}

// moments (4N) of the current state -> mom_all[k]
static void deposit_state(ch_adjoint* a, const StepConsts& k0, int k) {
  const int64_t N = a->g.N;
  MixParticles none{};
  const int nb = launch_pass(false, PH_DEPOSIT, k0, a->cur, none, nullptr, nullptr, nullptr, a->acc, 0.0, 0.0,
                             a->cnt, a->part, nullptr, nullptr, a->sms, a->stream);
  (void)nb;
  launch_finalize(N, a->acc, 1.0 / k0.dep_scale, 1, a->mom_all + (size_t)k * 4 * N, a->part, a->cnt, a->sms,
                  a->stream);
}

// sum and sum of squares of a grid vector into red[q], red[q + 1]
static void grid_sums(ch_adjoint* a, const double* v, int q) {
  k_adj_sum<<<a->nb, 256, 0, a->stream>>>(a->g.N, v, nullptr, a->part), ::ch::note_launch();
  launch_reduce_partials(a->part, a->nb, 2, a->red + q, a->stream);
}

// phi_k = solve(mom_k), warm start phi_{k-1}; E0 from theta.
static ch_status solve_state(ch_adjoint* a, int k) {
  const int64_t N = a->g.N;
  double* phi = a->phi_all + (size_t)k * N;
  const double* mom = a->mom_all + (size_t)k * 4 * N;
  if (k > 0) CH_CUDA_OK(cudaMemcpyAsync(phi, phi - N, sizeof(double) * N, cudaMemcpyDeviceToDevice, a->stream));
  else CH_CUDA_OK(cudaMemsetAsync(phi, 0, sizeof(double) * N, a->stream));
  a->solver.build_rhs(mom, a->rhs, a->stream);
  SolveStats st{};
  ch_status rc = a->solver.solve(mom, a->rhs, phi, &st, a->stream);
  if (rc == CH_ERR_NOT_CONVERGED)
    return ch_fail(rc, "adjoint forward solve %d: ||r|| = %.3e, ||b|| = %.3e", k, st.rnorm, st.bnorm);
  return rc;
}

extern "C" ch_status ch_adjoint_forward(ch_adjoint* a, const double* theta, int32_t record, double* J) {
  if (!a || !theta) return ch_fail(CH_ERR_ARG, "null argument");
  if (!record && !a->recorded) return ch_fail(CH_ERR_STATE, "replay needs a recorded run");
  cudaStream_t s = a->stream;
  const GridDesc& g = a->g;
  const int64_t N = g.N;
  const int S = a->cfg.nsteps, K = a->cfg.checkpoint_every, W = a->cfg.window;
  const int last_seg = (S - 1) / K;
  cudaEventRecord(a->e0, s);
  a->solver.set_E0(theta);
  // initial state at amp = theta[6]
  ch_loader L = a->L;
  L.amp[0] = theta[6];
  if (fabs(L.amp[0]) + fabs(L.amp[1]) + fabs(L.amp[2]) >= 1.0) return ch_fail(CH_ERR_ARG, "amplitudes sum >= 1");
  MixParticles none{};
  launch_load(false, g, L, a->p.seed, a->p.run, a->cur, none, a->sms, s);
  StepConsts k0 = adj_consts(a, theta, 0);
  if (record) {
    k_adj_dxda<<<a->nb, 256, 0, s>>>(g, L, a->cur, a->dxda), ::ch::note_launch();
    CH_CUDA_OK(cudaMemsetAsync(a->ev_count, 0, sizeof(unsigned), s));
    CH_CUDA_OK(cudaMemsetAsync(a->err, 0, sizeof(int), s));
    // S of the loaded ions (as after a ch_ctx load)
    if (k0.collide) {
      const int nb = launch_sbar(false, k0, a->cur, none, a->part, a->sms, s);
      launch_reduce_partials(a->part, nb, 1, a->red + 8, s);
    }
  }
  CH_CUDA_OK(cudaMemsetAsync(a->acc, 0, sizeof(unsigned long long) * 4 * N, s));
  deposit_state(a, k0, 0);
  ch_status rc = solve_state(a, 0);
  if (rc) return rc;
  const double Nc = k0.collide ? (double)collision_count(a->p, a->np) : 0.0;
  double Jsum = 0.0;
  const double wflux = a->cfg.flux_weight / ((double)W * (double)N);
  const double wphi = a->cfg.phi_weight / ((double)W * (double)N);
  for (int st = 0; st < S; ++st) {
    if (record) {
      if (st % K == 0) copy_state(a->ckpt[st / K], a->cur, s);
      if (st / K == last_seg) copy_state(a->seg[st - last_seg * K], a->cur, s);
    }
    const StepConsts k = adj_consts(a, theta, st);
    launch_node_efield(false, g, k.tscale, a->phi_all + (size_t)st * N, a->E64, nullptr, a->sms, s);
    int32_t* first = a->first + (size_t)st * a->np;
    if (record)
      k_adj_fwd<ADJ_RECORD><<<a->nb, 256, 0, s>>>(k, a->cur, a->E64, a->acc, a->ev, a->ev_count, a->ev_cap, first,
                                                  Nc, a->red + 8, a->part, a->err), ::ch::note_launch();
    else
      k_adj_fwd<ADJ_REPLAY><<<a->nb, 256, 0, s>>>(k, a->cur, a->E64, a->acc, a->ev, a->ev_count, a->ev_cap, first,
                                                  Nc, a->red + 8, a->part, a->err), ::ch::note_launch();
    launch_reduce_partials(a->part, a->nb, 2, a->red, s);  // red[0] = sum vx, red[1] = S next
    if (record && k.collide) CH_CUDA_OK(cudaMemcpyAsync(a->red + 8, a->red + 1, sizeof(double), cudaMemcpyDeviceToDevice, s));
    launch_finalize(N, a->acc, 1.0 / k.dep_scale, 1, a->mom_all + (size_t)(st + 1) * 4 * N, a->part, a->cnt, a->sms,
                    s);
    rc = solve_state(a, st + 1);
    if (rc) return rc;
    if (st >= S - W) {
      grid_sums(a, a->phi_all + (size_t)(st + 1) * N, 2);  // red[3] = sum phi^2
      CH_CUDA_OK(cudaMemcpyAsync(a->hred, a->red, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
      CH_CUDA_OK(cudaStreamSynchronize(s));
      Jsum += wflux * a->hred[0] + wphi * a->hred[3];
    }
  }
  int herr = 0;
  CH_CUDA_OK(cudaMemcpyAsync(&herr, a->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  cudaEventRecord(a->e1, s);
  CH_CUDA_OK(cudaStreamSynchronize(s));
  if (herr) return ch_fail(CH_ERR_RANGE, "adjoint: collision event pool (%u) overflowed", a->ev_cap);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a->e0, a->e1);
  a->timing.forward_ms = ms;
  if (record) {
    unsigned ne = 0;
    CH_CUDA_OK(cudaMemcpy(&ne, a->ev_count, sizeof(unsigned), cudaMemcpyDeviceToHost));
    a->timing.events = ne;
    a->recorded = true;
    a->seg_holds = last_seg;  // the forward run stored the last segment
    for (int q = 0; q < CH_ADJ_NTHETA; ++q) a->theta_rec[q] = theta[q];
    a->J_rec = Jsum;
  }
  if (J) *J = Jsum;
  return CH_OK;
}

// lam = solve(A(n_k), P phibar); zero start.
static ch_status adjoint_solve(ch_adjoint* a, int k) {
  const int64_t N = a->g.N;
  cudaStream_t s = a->stream;
  grid_sums(a, a->phibar, 4);
  k_adj_sub<<<a->nb, 256, 0, s>>>(N, a->phibar, a->red + 4, 1.0 / (double)N), ::ch::note_launch();
  CH_CUDA_OK(cudaMemsetAsync(a->lam, 0, sizeof(double) * N, s));
  SolveStats st{};
  ch_status rc = a->solver.solve(a->mom_all + (size_t)k * 4 * N, a->phibar, a->lam, &st, s);
  if (rc == CH_ERR_NOT_CONVERGED)
    return ch_fail(rc, "adjoint solve %d: ||r|| = %.3e, ||b|| = %.3e", k, st.rnorm, st.bnorm);
  return rc;
}

extern "C" ch_status ch_adjoint_gradient(ch_adjoint* a, double* grad, double* J) {
  if (!a || !grad) return ch_fail(CH_ERR_ARG, "null argument");
  if (!a->recorded) return ch_fail(CH_ERR_STATE, "record a forward run first");
  cudaStream_t s = a->stream;
  const GridDesc& g = a->g;
  const int64_t N = g.N;
  const int S = a->cfg.nsteps, K = a->cfg.checkpoint_every, W = a->cfg.window;
  const double* theta = a->theta_rec;
  const double wflux = a->cfg.flux_weight / ((double)W * (double)N);
  const double wphi = a->cfg.phi_weight / ((double)W * (double)N);
  cudaEventRecord(a->e0, s);
  a->solver.set_E0(theta);
  const StepConsts k0 = adj_consts(a, theta, 0);
  double RbT[9];
  boris_rbt(k0, RbT);
  CH_CUDA_OK(cudaMemcpyAsync(a->RbT, RbT, sizeof(RbT), cudaMemcpyHostToDevice, s));
  for (auto* q : a->Xb) CH_CUDA_OK(cudaMemsetAsync(q, 0, sizeof(double) * a->np, s));
  CH_CUDA_OK(cudaMemsetAsync(a->Ebar, 0, sizeof(double) * 3 * N, s));
  double gE0[3] = {0.0, 0.0, 0.0}, gvn0[3] = {0.0, 0.0, 0.0};
  double recompute_ms = 0.0;
  // phibar of the last state: the objective only
  k_adj_phibar<<<a->nb, 256, 0, s>>>(g, a->Ebar, a->phi_all + (size_t)S * N, 2.0 * wphi, a->phibar),
      ::ch::note_launch();
  const int nseg = (S + K - 1) / K;
  for (int sg = nseg - 1; sg >= 0; --sg) {
    const int s0 = sg * K, s1 = (s0 + K < S) ? s0 + K : S;
    if (sg != a->seg_holds) {
      // rebuild the segment's pre-step states from its checkpoint
      cudaEvent_t r0, r1;
      cudaEventCreate(&r0);
      cudaEventCreate(&r1);
      cudaEventRecord(r0, s);
      copy_state(a->cur, a->ckpt[sg], s);
      for (int st = s0; st < s1; ++st) {
        copy_state(a->seg[st - s0], a->cur, s);
        const StepConsts k = adj_consts(a, theta, st);
        launch_node_efield(false, g, k.tscale, a->phi_all + (size_t)st * N, a->E64, nullptr, a->sms, s);
        k_adj_fwd<ADJ_RECOMPUTE><<<a->nb, 256, 0, s>>>(k, a->cur, a->E64, a->acc, a->ev, a->ev_count, a->ev_cap,
                                                       a->first + (size_t)st * a->np, 0.0, a->red + 8, a->part,
                                                       a->err), ::ch::note_launch();
      }
      cudaEventRecord(r1, s);
      cudaEventSynchronize(r1);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, r0, r1);
      recompute_ms += ms;
      cudaEventDestroy(r0);
      cudaEventDestroy(r1);
      a->seg_holds = sg;
    }
    for (int st = s1 - 1; st >= s0; --st) {
      const int kpost = st + 1;  // state produced by step st
      // adjoint of phi_kpost is in phibar (gather of step kpost + objective)
      ch_status rc = adjoint_solve(a, kpost);
      if (rc) return rc;
      k_adj_node<<<a->nb, 256, 0, s>>>(g, dev_coefs<double>(op_coefs(a->p, g)), theta[0], theta[1], theta[2],
                                       a->p.cth, a->p.cG, a->mom_all + (size_t)kpost * 4 * N,
                                       a->phi_all + (size_t)kpost * N, a->lam, a->nbar, a->Gbar, a->part),
          ::ch::note_launch();
      launch_reduce_partials(a->part, a->nb, 3, a->red + 8, s);
      CH_CUDA_OK(cudaMemcpyAsync(a->hred + 8, a->red + 8, sizeof(double) * 3, cudaMemcpyDeviceToHost, s));
      const StepConsts k = adj_consts(a, theta, st);
      launch_node_efield(false, g, k.tscale, a->phi_all + (size_t)st * N, a->E64, nullptr, a->sms, s);
      CH_CUDA_OK(cudaMemsetAsync(a->Ebar, 0, sizeof(double) * 3 * N, s));
      const double vxw = (kpost > S - W) ? wflux : 0.0;
      k_adj_ion<<<a->nb, 256, 0, s>>>(k, a->RbT, a->seg[st - s0], a->E64, a->ev, a->first + (size_t)st * a->np,
                                      a->nbar, a->Gbar, vxw, a->Xb[0], a->Xb[1], a->Xb[2], a->Xb[3], a->Xb[4],
                                      a->Xb[5], a->Ebar, a->part), ::ch::note_launch();
      launch_reduce_partials(a->part, a->nb, 6, a->red, s);
      CH_CUDA_OK(cudaMemcpyAsync(a->hred, a->red, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
      // phibar of state st: gather of step st, objective if st is in the window
      const double w = (st > S - W) ? 2.0 * wphi : 0.0;
      k_adj_phibar<<<a->nb, 256, 0, s>>>(g, a->Ebar, a->phi_all + (size_t)st * N, w, a->phibar), ::ch::note_launch();
      CH_CUDA_OK(cudaStreamSynchronize(s));
      for (int d = 0; d < 3; ++d) {
        gE0[d] += a->hred[8 + d] + a->hred[3 + d];
        gvn0[d] += a->hred[d];
      }
    }
  }
  // initial solve and load
  ch_status rc = adjoint_solve(a, 0);
  if (rc) return rc;
  k_adj_node<<<a->nb, 256, 0, s>>>(g, dev_coefs<double>(op_coefs(a->p, g)), theta[0], theta[1], theta[2], a->p.cth,
                                   a->p.cG, a->mom_all, a->phi_all, a->lam, a->nbar, a->Gbar, a->part),
      ::ch::note_launch();
  launch_reduce_partials(a->part, a->nb, 3, a->red + 8, s);
  // initial positions at amp (the checkpoint of state 0)
  k_adj_initial<<<a->nb, 256, 0, s>>>(g, a->ckpt[0], a->nbar, a->Gbar, a->Xb[0], a->dxda, a->part),
      ::ch::note_launch();
  launch_reduce_partials(a->part, a->nb, 1, a->red + 12, s);
  CH_CUDA_OK(cudaMemcpyAsync(a->hred + 8, a->red + 8, sizeof(double) * 5, cudaMemcpyDeviceToHost, s));
  cudaEventRecord(a->e1, s);
  CH_CUDA_OK(cudaStreamSynchronize(s));
  for (int d = 0; d < 3; ++d) gE0[d] += a->hred[8 + d];
  for (int d = 0; d < 3; ++d) grad[d] = gE0[d];
  for (int d = 0; d < 3; ++d) grad[3 + d] = gvn0[d];
  grad[6] = a->hred[12];
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a->e0, a->e1);
  a->timing.gradient_ms = ms;
  a->timing.recompute_ms = recompute_ms;
  if (J) *J = a->J_rec;
  return CH_OK;
}

extern "C" ch_status ch_adjoint_events(ch_adjoint* a, int64_t* count, int32_t* step, uint32_t* ion, int32_t* flags,
                                       double* data) {
  if (!a || !count) return ch_fail(CH_ERR_ARG, "null argument");
  if (!a->recorded) return ch_fail(CH_ERR_STATE, "record a forward run first");
  unsigned ne = 0;
  CH_CUDA_OK(cudaMemcpy(&ne, a->ev_count, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (!step || !ion || !flags || !data) {
    *count = ne;
    return CH_OK;
  }
  if (*count < (int64_t)ne) return ch_fail(CH_ERR_ARG, "arrays hold %lld events, %u needed", (long long)*count, ne);
  std::vector<AdjEvent> ev(ne);
  std::vector<int32_t> first((size_t)a->np);
  CH_CUDA_OK(cudaMemcpy(ev.data(), a->ev, sizeof(AdjEvent) * ne, cudaMemcpyDeviceToHost));
  int64_t q = 0;
  for (int st = 0; st < a->cfg.nsteps; ++st) {
    CH_CUDA_OK(cudaMemcpy(first.data(), a->first + (size_t)st * a->np, sizeof(int32_t) * a->np,
                          cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < a->np; ++i)
      for (int32_t e = first[i]; e >= 0; e = ev[e].next) {
        step[q] = st;
        ion[q] = (uint32_t)i;
        flags[q] = (int32_t)ev[e].flags;
        for (int d = 0; d < 3; ++d) data[5 * q + d] = ev[e].n[d];
        data[5 * q + 3] = ev[e].uz;
        data[5 * q + 4] = ev[e].uphi;
        ++q;
      }
  }
  *count = q;
  return CH_OK;
}

extern "C" ch_status ch_adjoint_get_timing(ch_adjoint* a, ch_adjoint_timing* out) {
  if (!a || !out) return ch_fail(CH_ERR_ARG, "null argument");
  *out = a->timing;
  return CH_OK;
}
