/*
 * oracle.c -- FP64 CPU restatement of the hybrid-PIC hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
 * Nothing in the product links or calls this file.
 *
 * Compiled with -ffp-contract=off so that x86-64 and aarch64 round alike.
 * Grid vectors are in DMDA natural order idx = (k*Ny + j)*Nx + i; the
 * moment vector interleaves {n, Gx, Gy, Gz} per node like GridNode.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI 3.14159265358979323846

/* Philox counter word 2 = purpose << 24 | block.  Shared with the GPU. */
#define PURPOSE_COLLIDE 1u
#define PURPOSE_LOAD 2u
#define STEP_LOADER 0xFFFFFFFFu

static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------------ */
/* Philox4x32-10: ten rounds of the 4x32 bijection with the Weyl key
 * schedule; multipliers and key increments as published (SC'11, Table 2). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * x0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * x2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ x1 ^ k0;
    uint32_t n2 = hi0 ^ x3 ^ k1;
    x0 = n0; x1 = lo1; x2 = n2; x3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

static inline double unit(uint32_t r) { return ((double)r + 0.5) * 2.3283064365386962890625e-10; }

static inline void draw(const ch_params* p, uint32_t id, uint32_t step, uint32_t purpose,
                        uint32_t block, uint32_t out[4]) {
  uint32_t ctr[4] = {id, step, (purpose << 24) | block, p->run};
  uint32_t key[2] = {(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
  orc_philox4x32_10(ctr, key, out);
}

/* ------------------------------------------------------------------ */
typedef struct grid {
  int Nx, Ny, Nz;
  int64_t N;
  double x0, y0, z0, Lx, Ly, Lz, dx, dy, dz;
} grid;

/* Cell spacing d = L/N (src/setup.c:47-49). */
static grid mkgrid(const ch_params* p) {
  grid g;
  g.Nx = p->Nx; g.Ny = p->Ny; g.Nz = p->Nz;
  g.N = (int64_t)p->Nx * p->Ny * p->Nz;
  g.x0 = p->x0; g.y0 = p->y0; g.z0 = p->z0;
  g.Lx = p->x1 - p->x0; g.Ly = p->y1 - p->y0; g.Lz = p->z1 - p->z0;
  g.dx = g.Lx / p->Nx; g.dy = g.Ly / p->Ny; g.dz = g.Lz / p->Nz;
  return g;
}

static inline int wrap(int i, int n) { i %= n; return i < 0 ? i + n : i; }
static inline int64_t nid(const grid* g, int i, int j, int k) {
  return ((int64_t)wrap(k, g->Nz) * g->Ny + wrap(j, g->Ny)) * g->Nx + wrap(i, g->Nx);
}

/* ------------------------------------------------------------------ */
/* Loader: inverse CDF of n(x) = 1 + sum_m a_m sin(2 pi m x/L + ph_m) in x,
 * uniform y, z, Maxwellian v.  Replaces src/particles.c:9-132 for the
 * synthetic plasmas (the reference's loaders are fixed at 1+0.25 sin). */
static double inv_cdf_x(const ch_loader* L, double Lx, double u) {
  double target = u * Lx, lo = 0.0, hi = Lx, x = target;
  for (int it = 0; it < 40; ++it) {
    double F = x, dF = 1.0;
    for (int m = 1; m <= 3; ++m) {
      double a = L->amp[m - 1];
      if (a == 0.0) continue;
      double w = 2.0 * PI * m / Lx;
      F += a * (cos(L->phase[m - 1]) - cos(w * x + L->phase[m - 1])) / w;
      dF += a * sin(w * x + L->phase[m - 1]);
    }
    double r = F - target;
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

int orc_load(const ch_params* p, const ch_loader* L, orc_particles* P) {
  grid g = mkgrid(p);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t i = 0; i < P->np; ++i) {
    uint32_t a[4], b[4];
    draw(p, (uint32_t)i, STEP_LOADER, PURPOSE_LOAD, 0, a);
    draw(p, (uint32_t)i, STEP_LOADER, PURPOSE_LOAD, 1, b);
    P->x[i] = g.x0 + inv_cdf_x(L, g.Lx, unit(a[0]));
    P->y[i] = g.y0 + unit(a[1]) * g.Ly;
    P->z[i] = g.z0 + unit(a[2]) * g.Lz;
    double r1 = sqrt(-2.0 * log(unit(b[0]))), t1 = 2.0 * PI * unit(b[1]);
    double r2 = sqrt(-2.0 * log(unit(b[2]))), t2 = 2.0 * PI * unit(b[3]);
    P->vx[i] = L->v0[0] + L->vT[0] * (r1 * cos(t1));
    P->vy[i] = L->v0[1] + L->vT[1] * (r1 * sin(t1));
    P->vz[i] = L->v0[2] + L->vT[2] * (r2 * cos(t2));
  }
  return 0;
}

/* The reference's --density-type placements (src/particles.c:9-132,
 * src/distributions.c:33-232), restated for the device loader
 * ch_particles_load_placed: flat-sobol (0), uniform (3), sinusoidal (4).
 * Velocities as orc_load. */
static void sobol_directions(uint32_t v[3][32]) {
  /* first three Sobol dimensions (Joe & Kuo): van der Corput; x + 1 with
   * m1 = 1; x^2 + x + 1 with m1 = 1, m2 = 3; v_k by Bratley & Fox's
   * recursion, as 32-bit fractions */
  for (int k = 0; k < 32; ++k) v[0][k] = 1u << (31 - k);
  v[1][0] = 1u << 31;
  for (int k = 1; k < 32; ++k) v[1][k] = v[1][k - 1] ^ (v[1][k - 1] >> 1);
  v[2][0] = 1u << 31;
  v[2][1] = 3u << 30;
  for (int k = 2; k < 32; ++k) v[2][k] = v[2][k - 1] ^ v[2][k - 2] ^ (v[2][k - 2] >> 2);
}

/* SobolDistribution (src/distributions.c:96-128): v = r (L + d) - d/2,
 * clamped to [p0 + 0.01 d, p1 - 0.01 d]. */
static double sobol_coord(double r, double L, double d, double p0, double p1) {
  double v = r * (L + d) - 0.5 * d;
  if (v < p0) return p0 + 0.01 * d;
  if (v > p1) return p1 - 0.01 * d;
  return v;
}

int orc_load_placed(const ch_params* p, const ch_loader* L, int type, orc_particles* P) {
  grid g = mkgrid(p);
  if (type != 0 && type != 3 && type != 4) return CH_ERR_UNSUPPORTED;
  if (type == 3 && P->np % g.N != 0) return CH_ERR_ARG;
  uint32_t dirs[3][32];
  sobol_directions(dirs);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t i = 0; i < P->np; ++i) {
    const uint32_t id = (uint32_t)i;
    if (type == 0) {
      /* point id + 1 in Gray-code order (Antonov & Saleev) */
      const uint32_t n = id + 1u, gc = n ^ (n >> 1);
      uint32_t x[3] = {0u, 0u, 0u};
      for (int k = 0; k < 32; ++k)
        if (gc & (1u << k))
          for (int d = 0; d < 3; ++d) x[d] ^= dirs[d][k];
      P->x[i] = sobol_coord((double)x[0] * 2.3283064365386962890625e-10, g.Lx, g.dx, g.x0, g.x0 + g.Lx);
      P->y[i] = sobol_coord((double)x[1] * 2.3283064365386962890625e-10, g.Ly, g.dy, g.y0, g.y0 + g.Ly);
      P->z[i] = sobol_coord((double)x[2] * 2.3283064365386962890625e-10, g.Lz, g.dz, g.z0, g.z0 + g.Lz);
    } else if (type == 3) {
      /* UniformDistribution (src/distributions.c:33-94), every cell */
      const int64_t c = (int64_t)id % g.N;
      const int ci = (int)(c % g.Nx), cj = (int)((c / g.Nx) % g.Ny), ck = (int)(c / ((int64_t)g.Nx * g.Ny));
      P->x[i] = g.x0 + g.dx * ((double)ci + 0.5);
      P->y[i] = g.y0 + g.dy * ((double)cj + 0.5);
      P->z[i] = g.z0 + g.dz * ((double)ck + 0.5);
    } else {
      /* Rejection (src/distributions.c:143-232) of 1 + 0.25 sin(2 pi x)
       * (:131-141) with the bound 1.25 */
      for (uint32_t a = 0; a < 256u; ++a) {
        uint32_t q[4];
        draw(p, id, STEP_LOADER, PURPOSE_LOAD, 2u + a, q);
        const double x = unit(q[0]) * g.Lx, y = unit(q[1]) * g.Ly, z = unit(q[2]) * g.Lz;
        const double w = 1.0 + 0.25 * sin(2.0 * PI * x);
        P->x[i] = g.x0 + x;
        P->y[i] = g.y0 + y;
        P->z[i] = g.z0 + z;
        if (w > unit(q[3]) * 1.25) break;
      }
    }
    uint32_t b[4];
    draw(p, id, STEP_LOADER, PURPOSE_LOAD, 1, b);
    double r1 = sqrt(-2.0 * log(unit(b[0]))), t1 = 2.0 * PI * unit(b[1]);
    double r2 = sqrt(-2.0 * log(unit(b[2]))), t2 = 2.0 * PI * unit(b[3]);
    P->vx[i] = L->v0[0] + L->vT[0] * (r1 * cos(t1));
    P->vy[i] = L->v0[1] + L->vT[1] * (r1 * sin(t1));
    P->vz[i] = L->v0[2] + L->vT[2] * (r2 * cos(t2));
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* DifferenceVector (src/vectors.c:12-138).  Values are read through a
 * periodic wrap, which equals the ghost-width-1 local array of the
 * reference for every index it touches. */
static inline double F3(const grid* g, const double* phi, int k, int j, int i) {
  return phi[nid(g, i, j, k)];
}

void orc_difference_vector(const ch_params* p, const double* phi, double X, double Y, double Z,
                           uint32_t faithful, double f[3]) {
  grid g = mkgrid(p);
  const grid* G = &g;
  int ixl = (int)floor(X), iyl = (int)floor(Y), izl = (int)floor(Z);
  double wxh = X - ixl, wyh = Y - iyl, wzh = Z - izl;
  int ixh = ixl + 1, iyh = iyl + 1, izh = izl + 1;
  int onesided = (faithful & CH_FAITHFUL_D4) != 0;
  for (int d = 0; d < 3; ++d) {
    double hhh, lhh, hlh, llh, hhl, lhl, hll, lll; /* names: (z, y, x) */
    /* difference of the node (k, j, i) along d; at an upper index equal to
     * N the as-written code uses the backward one-sided formula. */
#define DIFF(k, j, i, up)                                                                     \
  ((d == 0) ? ((onesided && (up) && (i) == G->Nx)                                             \
                   ? 3.0 * F3(G, phi, k, j, i) - 4.0 * F3(G, phi, k, j, (i)-1) + F3(G, phi, k, j, (i)-2) \
                   : F3(G, phi, k, j, (i) + 1) - F3(G, phi, k, j, (i)-1))                     \
   : (d == 1) ? ((onesided && (up) && (j) == G->Ny)                                           \
                     ? 3.0 * F3(G, phi, k, j, i) - 4.0 * F3(G, phi, k, (j)-1, i) + F3(G, phi, k, (j)-2, i) \
                     : F3(G, phi, k, (j) + 1, i) - F3(G, phi, k, (j)-1, i))                   \
              : ((onesided && (up) && (k) == G->Nz)                                           \
                     ? 3.0 * F3(G, phi, k, j, i) - 4.0 * F3(G, phi, (k)-1, j, i) + F3(G, phi, (k)-2, j, i) \
                     : F3(G, phi, (k) + 1, j, i) - F3(G, phi, (k)-1, j, i)))
    int upx = (d == 0), upy = (d == 1), upz = (d == 2);
    hhh = DIFF(izh, iyh, ixh, upx || upy || upz);
    lhh = DIFF(izl, iyh, ixh, upx || upy);
    hlh = DIFF(izh, iyl, ixh, upx || upz);
    llh = DIFF(izl, iyl, ixh, upx);
    hhl = DIFF(izh, iyh, ixl, upy || upz);
    lhl = DIFF(izl, iyh, ixl, upy);
    hll = DIFF(izh, iyl, ixl, upz);
    lll = DIFF(izl, iyl, ixl, 0);
#undef DIFF
    /* y lerps at the four (z, x) corners (src/vectors.c:61-64) */
    double whh = hlh + wyh * (hhh - hlh);
    double whl = hll + wyh * (hhl - hll);
    double wlh = llh + wyh * (lhh - llh);
    double wll = lll + wyh * (lhl - lll);
    if (faithful & CH_FAITHFUL_D3) {
      /* as written (src/vectors.c:65-67): z lerp with the x weight, then a
       * zero-width z lerp, leaving the x=low column only */
      double Ewh = wlh + wxh * (whh - wlh);
      double Ewl = wll + wxh * (whl - wll);
      f[d] = Ewl + wzh * (Ewh - Ewh);
    } else {
      double Ezl = wll + wxh * (wlh - wll);
      double Ezh = whl + wxh * (whh - whl);
      f[d] = Ezl + wzh * (Ezh - Ezl);
    }
  }
}

/* Node field: E_d = -(phi[+1] - phi[-1]) / (2 d_d), the scale Escale of
 * src/particles.c:391-393 applied at the nodes. */
void orc_node_efield(const ch_params* p, const double* phi, double* Ex, double* Ey, double* Ez) {
  grid g = mkgrid(p);
  for (int k = 0; k < g.Nz; ++k)
    for (int j = 0; j < g.Ny; ++j)
      for (int i = 0; i < g.Nx; ++i) {
        int64_t c = nid(&g, i, j, k);
        Ex[c] = -(phi[nid(&g, i + 1, j, k)] - phi[nid(&g, i - 1, j, k)]) / (2.0 * g.dx);
        Ey[c] = -(phi[nid(&g, i, j + 1, k)] - phi[nid(&g, i, j - 1, k)]) / (2.0 * g.dy);
        Ez[c] = -(phi[nid(&g, i, j, k + 1)] - phi[nid(&g, i, j, k - 1)]) / (2.0 * g.dz);
      }
}

/* ------------------------------------------------------------------ */
/* Collisions (src/particles.c:471-624).
 *
 * The reference draws Nc accepted events: ion i uniformly, a Maxwellian
 * neutral V, acceptance with probability min(1, |v_i - V|/vrm); it repeats
 * until Nc events are accepted, so one ion may collide more than once.
 * Each accepted event lands on ion i with probability g_i / sum_j g_j,
 * g = E_V|v - V|, and carries a neutral drawn from the density proportional
 * to |v_i - V| N(V).  The per-ion form used here (collide_ion) runs each
 * ion's events as a Poisson process of rate Nc g(v) rho_n(x) / S over the
 * step, S = sum_j g_j over the velocities the ions carry into the step,
 * keyed by Philox(id, step), with the same neutral law and the reference's
 * centre-of-mass scatter and 10 vT refusal. */
double orc_gmean(double w, double sigma) {
  if (sigma <= 0.0) return w;
  double a = w / (sigma * sqrt(2.0));
  double c = sigma * sqrt(2.0 / PI);
  if (a < 1e-4) return 2.0 * c * (1.0 + a * a / 3.0);
  return c * exp(-a * a) + (w + sigma * sigma / w) * erf(a);
}

int64_t orc_collision_count(const ch_params* p, int64_t np) {
  double viTr = sqrt(p->viT[0] * p->viT[0] + p->viT[1] * p->viT[1] + p->viT[2] * p->viT[2]);
  double dvx = p->vi0[0] - p->vn0[0], dvy = p->vi0[1] - p->vn0[1], dvz = p->vi0[2] - p->vn0[2];
  double vrm = 4.0 * viTr + sqrt(dvx * dvx + dvy * dvy + dvz * dvz);
  double vn0r = sqrt(p->vn0[0] * p->vn0[0] + p->vn0[1] * p->vn0[1] + p->vn0[2] * p->vn0[2]);
  double den = (p->vnT + vn0r) * sqrt(p->mn / p->mi);
  double fc = p->nui * p->dt;
  if (!(den > 0.0)) return np;
  double v = ((double)np * fc * vrm) / den;
  if (v >= (double)np) return np;
  if (v < 0.0) return 0;
  return (int64_t)v;
}

double orc_sbar(const ch_params* p, const orc_particles* P) {
  double s = 0.0;
  for (int64_t i = 0; i < P->np; ++i) {
    double wx = P->vx[i] - p->vn0[0], wy = P->vy[i] - p->vn0[1], wz = P->vz[i] - p->vn0[2];
    s += orc_gmean(sqrt(wx * wx + wy * wy + wz * wz), p->vnT);
  }
  return s;
}

static double neutral_density(const ch_params* p, double x) {
  if (p->nn_profile != CH_NN_GAUSSIAN_X) return 1.0;
  double u = (x - p->nn_center) / p->nn_sigma;
  double v = exp(-0.5 * u * u);
  return v > p->nn_floor ? v : p->nn_floor;
}

/* Collisions of one ion over one step.  The ion's events form a Poisson
 * process in the step's unit time with the state-dependent rate
 *     lambda(v) = lscale * g(|v - vn0|),  lscale = Nc rho_n(x) / S,
 * which is the many-ion limit of the reference's sequential sampler (each
 * of its Nc accepted events picks ion i with probability g_i / sum_j g_j
 * at the current velocities, with replacement).  Exponential waiting times
 * come from Philox block (e << 8); the neutral of event e is drawn from the
 * density proportional to |v - V| N(V) by the speed-weighted proposal with
 * blocks (e << 8) | (1 + 2 it), (e << 8) | (2 + 2 it).  Refused events
 * (|v_f| > 10 vT, src/particles.c:597-606) leave v unchanged.
 * Returns the number of accepted collisions; *refused counts refusals. */
#define MAX_EVENTS 32
static int collide_ion(const ch_params* p, uint32_t id, uint32_t step, double lscale, double* vx, double* vy,
                       double* vz, int* refused) {
  const double sig = p->vnT;
  const double m1 = 2.0 * sig * sqrt(2.0 / PI);
  const double viTr = sqrt(p->viT[0] * p->viT[0] + p->viT[1] * p->viT[1] + p->viT[2] * p->viT[2]);
  const double mi = p->mi, mn = p->mn, M = mn + mi;
  double t = 0.0;
  int ncol = 0;
  for (uint32_t e = 0; e < MAX_EVENTS; ++e) {
    const double vix = *vx, viy = *vy, viz = *vz;
    const double wx = vix - p->vn0[0], wy = viy - p->vn0[1], wz = viz - p->vn0[2];
    const double w = sqrt(wx * wx + wy * wy + wz * wz);
    const double lam = lscale * orc_gmean(w, sig);
    if (!(lam > 0.0)) break;
    uint32_t r[4];
    draw(p, id, step, PURPOSE_COLLIDE, e << 8, r);
    t += -log(unit(r[0])) / lam;
    if (!(t < 1.0)) break;
    double Vx = 0, Vy = 0, Vz = 0, uz = 0, uphi = 0;
    int ok = 0;
    for (uint32_t it = 0; it < 64 && !ok; ++it) {
      uint32_t a[4], c[4];
      draw(p, id, step, PURPOSE_COLLIDE, (e << 8) | (1 + 2 * it), a);
      draw(p, id, step, PURPOSE_COLLIDE, (e << 8) | (2 + 2 * it), c);
      double nx, ny, nz;
      if (unit(a[0]) * (w + m1) < w) {
        double r1 = sqrt(-2.0 * log(unit(a[1]))), t1 = 2.0 * PI * unit(a[2]);
        double r2 = sqrt(-2.0 * log(unit(a[3]))), t2 = 2.0 * PI * unit(c[0]);
        nx = sig * (r1 * cos(t1)); ny = sig * (r1 * sin(t1)); nz = sig * (r2 * cos(t2));
      } else {
        double sp = sig * sqrt(-2.0 * log(unit(a[1]) * unit(a[2])));
        double ct = 2.0 * unit(a[3]) - 1.0, st = sqrt(fmax(0.0, 1.0 - ct * ct));
        double ph = 2.0 * PI * unit(c[0]);
        nx = sp * st * cos(ph); ny = sp * st * sin(ph); nz = sp * ct;
      }
      Vx = p->vn0[0] + nx; Vy = p->vn0[1] + ny; Vz = p->vn0[2] + nz;
      double dV = sqrt(nx * nx + ny * ny + nz * nz);
      double rx = vix - Vx, ry = viy - Vy, rz = viz - Vz;
      double D = sqrt(rx * rx + ry * ry + rz * rz);
      if (unit(c[1]) * (w + dV) < D) {
        ok = 1;
        uz = 2.0 * unit(c[2]) - 1.0;
        uphi = 2.0 * PI * unit(c[3]);
      }
    }
    if (!ok) { (*refused)++; continue; }
    /* centre-of-mass scatter (src/particles.c:552-591) */
    double vrx = vix - Vx, vry = viy - Vy, vrz = viz - Vz;
    double vrr = sqrt(vrx * vrx + vry * vry + vrz * vrz);
    double vcx = (vix * mi + Vx * mn) / M, vcy = (viy * mi + Vy * mn) / M, vcz = (viz * mi + Vz * mn) / M;
    double ax = vix - vcx, ay = viy - vcy, az = viz - vcz;
    double vcr = sqrt(ax * ax + ay * ay + az * az);
    double uperp = sqrt(fmax(0.0, 1.0 - uz * uz));
    double ux = uperp * cos(uphi), uy = uperp * sin(uphi);
    double costht = vrr > 0.0 ? vrz / vrr : 1.0;
    double sintht = sqrt(fmax(0.0, 1.0 - costht * costht));
    double cosphi = 1.0, sinphi = 0.0;
    if (vrr * sintht > 0.0) { cosphi = vrx / (vrr * sintht); sinphi = vry / (vrr * sintht); }
    double ux1 = uz * sintht + ux * costht, uy1 = uy, uz1 = uz * costht - ux * sintht;
    double ux2 = ux1 * cosphi - uy1 * sinphi, uy2 = ux1 * sinphi + uy1 * cosphi, uz2 = uz1;
    double vfx = vcx + vcr * ux2, vfy = vcy + vcr * uy2, vfz = vcz + vcr * uz2;
    double vfr = sqrt(vfx * vfx + vfy * vfy + vfz * vfz);
    if (vfr / viTr > 10.0) { (*refused)++; continue; }
    *vx = vfx; *vy = vfy; *vz = vfz;
    ncol++;
  }
  return ncol;
}

/* ------------------------------------------------------------------ */
int orc_update_velocities(const ch_params* p, const double* phi, orc_particles* P, int64_t step,
                          double sbar, double* sbar_next, orc_counters* cnt) {
  grid g = mkgrid(p);
  const int64_t N = g.N;
  double* E = (double*)malloc(sizeof(double) * 3 * N);
  if (!E) return CH_ERR_NOMEM;
  orc_node_efield(p, phi, E, E + N, E + 2 * N);
  const double tscale = 0.5 * (p->qi / p->mi) * p->dt;
  double t[3], s[3];
  for (int d = 0; d < 3; ++d) t[d] = tscale * p->B0[d];
  double tt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
  for (int d = 0; d < 3; ++d) s[d] = 2.0 * t[d] / (1.0 + tt);
  const int nocross = (p->faithful & CH_FAITHFUL_D2) != 0;
  const int gatherD3 = (p->faithful & (CH_FAITHFUL_D3 | CH_FAITHFUL_D4)) != 0;
  const int collide = p->mn > 0.0;
  int64_t Nc = collide ? orc_collision_count(p, P->np) : 0;
  int64_t ncol = 0, nref = 0;
  double expct = 0.0, snext = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : ncol, nref, expct, snext) schedule(static)
  for (int64_t ip = 0; ip < P->np; ++ip) {
    double X = (P->x[ip] - g.x0) / g.dx, Y = (P->y[ip] - g.y0) / g.dy, Z = (P->z[ip] - g.z0) / g.dz;
    double Ef[3];
    if (gatherD3) {
      /* the reference's numerators with Escale = -0.5 h tscale */
      double f[3];
      orc_difference_vector(p, phi, X, Y, Z, p->faithful, f);
      Ef[0] = -f[0] / (2.0 * g.dx); Ef[1] = -f[1] / (2.0 * g.dy); Ef[2] = -f[2] / (2.0 * g.dz);
    } else {
      int i = (int)floor(X), j = (int)floor(Y), k = (int)floor(Z);
      double wx = X - i, wy = Y - j, wz = Z - k;
      int64_t c000 = nid(&g, i, j, k), c100 = nid(&g, i + 1, j, k), c010 = nid(&g, i, j + 1, k),
              c110 = nid(&g, i + 1, j + 1, k), c001 = nid(&g, i, j, k + 1), c101 = nid(&g, i + 1, j, k + 1),
              c011 = nid(&g, i, j + 1, k + 1), c111 = nid(&g, i + 1, j + 1, k + 1);
      for (int d = 0; d < 3; ++d) {
        const double* e = E + d * N;
        /* y lerps, then x, then z: the corrected DifferenceVector order */
        double wll = e[c000] + wy * (e[c010] - e[c000]);
        double wlh = e[c100] + wy * (e[c110] - e[c100]);
        double whl = e[c001] + wy * (e[c011] - e[c001]);
        double whh = e[c101] + wy * (e[c111] - e[c101]);
        double ezl = wll + wx * (wlh - wll);
        double ezh = whl + wx * (whh - whl);
        Ef[d] = ezl + wz * (ezh - ezl);
      }
    }
    if (p->push_E0) { Ef[0] += p->E0[0]; Ef[1] += p->E0[1]; Ef[2] += p->E0[2]; }
    /* Boris (src/particles.c:374-447) with D1 resolved per component */
    double vm[3] = {P->vx[ip] + tscale * Ef[0], P->vy[ip] + tscale * Ef[1], P->vz[ip] + tscale * Ef[2]};
    double vp[3];
    if (nocross) {
      vp[0] = vm[0]; vp[1] = vm[1]; vp[2] = vm[2];
    } else {
      double c1[3] = {vm[1] * t[2] - vm[2] * t[1], vm[2] * t[0] - vm[0] * t[2], vm[0] * t[1] - vm[1] * t[0]};
      double vpr[3] = {vm[0] + c1[0], vm[1] + c1[1], vm[2] + c1[2]};
      double c2[3] = {vpr[1] * s[2] - vpr[2] * s[1], vpr[2] * s[0] - vpr[0] * s[2], vpr[0] * s[1] - vpr[1] * s[0]};
      vp[0] = vm[0] + c2[0]; vp[1] = vm[1] + c2[1]; vp[2] = vm[2] + c2[2];
    }
    double vx = vp[0] + tscale * Ef[0], vy = vp[1] + tscale * Ef[1], vz = vp[2] + tscale * Ef[2];
    if (collide) {
      double wx = vx - p->vn0[0], wy = vy - p->vn0[1], wz = vz - p->vn0[2];
      double gi = orc_gmean(sqrt(wx * wx + wy * wy + wz * wz), p->vnT);
      double lscale = sbar > 0.0 ? ((double)Nc * neutral_density(p, P->x[ip])) / sbar : 0.0;
      expct += lscale * gi;
      int nr = 0;
      ncol += collide_ion(p, (uint32_t)ip, (uint32_t)step, lscale, &vx, &vy, &vz, &nr);
      nref += nr;
      double qx = vx - p->vn0[0], qy = vy - p->vn0[1], qz = vz - p->vn0[2];
      snext += orc_gmean(sqrt(qx * qx + qy * qy + qz * qz), p->vnT);
    }
    P->vx[ip] = vx; P->vy[ip] = vy; P->vz[ip] = vz;
  }
  free(E);
  if (cnt) { cnt->Nc = Nc; cnt->collisions = ncol; cnt->refused = nref; cnt->expected = expct; }
  if (sbar_next) *sbar_next = snext;
  return nref >= 10 ? CH_ERR_COLLISION_LIMIT : 0;
}

/* Periodic move; x in [x0, x1).  The reference loops `while (x > x1)` and
 * leaves x == x1 in place (src/particles.c:681-704); the wrap here is half
 * open so that the deposit index stays inside the grid. */
static inline double wrap_pos(double x, double x0, double L) {
  double u = x - x0;
  if (u < 0.0 || u >= L) u -= L * floor(u / L);
  if (u >= L) u -= L;
  if (u < 0.0) u = 0.0;
  return x0 + u;
}

void orc_update_positions(const ch_params* p, orc_particles* P) {
  if (p->faithful & CH_FAITHFUL_D5) return; /* as written: results discarded */
  grid g = mkgrid(p);
  const double dt = p->dt;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t i = 0; i < P->np; ++i) {
    P->x[i] = wrap_pos(P->x[i] + P->vx[i] * dt, g.x0, g.Lx);
    P->y[i] = wrap_pos(P->y[i] + P->vy[i] * dt, g.y0, g.Ly);
    P->z[i] = wrap_pos(P->z[i] + P->vz[i] * dt, g.z0, g.Lz);
  }
}

/* ------------------------------------------------------------------ */
static void deposit_range(const grid* g, const orc_particles* P, int64_t a, int64_t b, double* nodes) {
  for (int64_t ip = a; ip < b; ++ip) {
    double x = (P->x[ip] - g->x0) / g->dx, y = (P->y[ip] - g->y0) / g->dy, z = (P->z[ip] - g->z0) / g->dz;
    int ixl = (int)floor(x), iyl = (int)floor(y), izl = (int)floor(z);
    double wxh = x - ixl, wxl = 1.0 - wxh;
    double wyh = y - iyl, wyl = 1.0 - wyh;
    double wzh = z - izl, wzl = 1.0 - wzh;
    /* weights of src/particles.c:204-211 */
    double w[8] = {wzh * wyh * wxh, wzl * wyh * wxh, wzh * wyl * wxh, wzl * wyl * wxh,
                   wzh * wyh * wxl, wzl * wyh * wxl, wzh * wyl * wxl, wzl * wyl * wxl};
    int64_t c[8] = {nid(g, ixl + 1, iyl + 1, izl + 1), nid(g, ixl + 1, iyl + 1, izl),
                    nid(g, ixl + 1, iyl, izl + 1),     nid(g, ixl + 1, iyl, izl),
                    nid(g, ixl, iyl + 1, izl + 1),     nid(g, ixl, iyl + 1, izl),
                    nid(g, ixl, iyl, izl + 1),         nid(g, ixl, iyl, izl)};
    double v[3] = {P->vx[ip], P->vy[ip], P->vz[ip]};
    for (int q = 0; q < 8; ++q) {
      double* o = nodes + 4 * c[q];
      o[0] += w[q];
      o[1] += v[0] * w[q];
      o[2] += v[1] * w[q];
      o[3] += v[2] * w[q];
    }
  }
}

void orc_collect(const ch_params* p, const orc_particles* P, double* nodes, int accumulate) {
  grid g = mkgrid(p);
  if (!accumulate) memset(nodes, 0, sizeof(double) * 4 * g.N);
  int nt = g_threads;
  if (nt <= 1) { deposit_range(&g, P, 0, P->np, nodes); return; }
  /* private grids summed in thread order: deterministic for a given nt */
  double* priv = (double*)calloc((size_t)nt * 4 * g.N, sizeof(double));
  if (!priv) { deposit_range(&g, P, 0, P->np, nodes); return; }
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#else
    int t = 0;
#endif
    int64_t a = P->np * t / nt, b = P->np * (t + 1) / nt;
    deposit_range(&g, P, a, b, priv + (size_t)t * 4 * g.N);
  }
  for (int t = 0; t < nt; ++t) {
    const double* q = priv + (size_t)t * 4 * g.N;
    for (int64_t c = 0; c < 4 * g.N; ++c) nodes[c] += q[c];
  }
  free(priv);
}

/* ------------------------------------------------------------------ */
static void kappa_tensor(const ch_params* p, double R[3][3], double* det) {
  double Kx = p->kappa_e[0], Ky = p->kappa_e[1], Kz = p->kappa_e[2];
  *det = 1 + Kx * Kx + Ky * Ky + Kz * Kz;
  R[0][0] = 1 + Kx * Kx; R[0][1] = Ky * Kx - Kz; R[0][2] = Kz * Kx + Ky;
  R[1][0] = Kx * Ky + Kz; R[1][1] = 1 + Ky * Ky; R[1][2] = Kz * Ky - Kx;
  R[2][0] = Kx * Kz - Ky; R[2][1] = Ky * Kz + Kx; R[2][2] = 1 + Kz * Kz;
}

static void remove_mean(double* b, int64_t N) {
  double s = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < N; ++i) s += b[i];
  s /= (double)N;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t i = 0; i < N; ++i) b[i] -= s;
}

void orc_rhs(const ch_params* p, const double* nodes, double* b) {
  grid g = mkgrid(p);
  const grid* G = &g;
  double R[3][3], det;
  kappa_tensor(p, R, &det);
  const double dx = g.dx, dy = g.dy, dz = g.dz;
  if (p->rhs_type == CH_RHS_CONSTANT) {
    /* ComputeConstantRHS (src/rhs.c:8-48) */
    double mean = 0.0;
    for (int64_t c = 0; c < g.N; ++c) mean += nodes[4 * c];
    mean /= (double)g.N;
    double val = mean * (2.0 * dx * dy * dz / det);
    for (int64_t c = 0; c < g.N; ++c) b[c] = val;
    return;
  }
  if (p->rhs_type == CH_RHS_SINUSOIDAL) {
    /* ComputeSinusoidalRHS (src/rhs.c:51-130) */
    double n0 = 0.0;
    for (int64_t c = 0; c < g.N; ++c) n0 += nodes[4 * c];
    n0 /= (double)g.N;
    for (int k = 0; k < g.Nz; ++k)
      for (int j = 0; j < g.Ny; ++j)
        for (int i = 0; i < g.Nx; ++i) {
          double x = ((double)i + 0.5) * dx, y = ((double)j + 0.5) * dy, z = ((double)k + 0.5) * dz;
          double val = cos(2 * PI * x) * cos(2 * PI * y) * cos(2 * PI * z);
          b[nid(G, i, j, k)] = n0 * val * (2.0 * dx * dy * dz / det);
        }
    remove_mean(b, g.N);
    return;
  }
  /* ComputeFullRHS (src/rhs.c:133-303), FD helpers of src/calculus.c */
  const double scale = 1.0 / det;
  const double E0x = p->E0[0], E0y = p->E0[1], E0z = p->E0[2];
  const int d8 = (p->faithful & CH_FAITHFUL_D8) != 0;
#define N_(i, j, k) nodes[4 * nid(G, i, j, k) + 0]
#define G_(d, i, j, k) nodes[4 * nid(G, i, j, k) + 1 + (d)]
#pragma omp parallel for num_threads(g_threads) collapse(2) schedule(static)
  for (int k = 0; k < g.Nz; ++k)
    for (int j = 0; j < g.Ny; ++j)
      for (int i = 0; i < g.Nx; ++i) {
        double dndx = (N_(i + 1, j, k) - N_(i - 1, j, k)) / (2.0 * dx);
        double dndy = (N_(i, j + 1, k) - N_(i, j - 1, k)) / (2.0 * dy);
        double dndz = (N_(i, j, k + 1) - N_(i, j, k - 1)) / (2.0 * dz);
        double dGxdx = (G_(0, i + 1, j, k) - G_(0, i - 1, j, k)) / (2.0 * dx);
        double dGydy = (G_(1, i, j + 1, k) - G_(1, i, j - 1, k)) / (2.0 * dy);
        double dGzdz = (G_(2, i, j, k + 1) - G_(2, i, j, k - 1)) / (2.0 * dz);
        double d2ndxx = (N_(i + 1, j, k) - 2.0 * N_(i, j, k) + N_(i - 1, j, k)) / (dx * dx);
        double d2ndyy = (N_(i, j + 1, k) - 2.0 * N_(i, j, k) + N_(i, j - 1, k)) / (dy * dy);
        double d2ndzz = (N_(i, j, k + 1) - 2.0 * N_(i, j, k) + N_(i, j, k - 1)) / (dz * dz);
        double d2ndxy = (N_(i + 1, j + 1, k) - N_(i - 1, j + 1, k) - N_(i + 1, j - 1, k) + N_(i - 1, j - 1, k)) /
                        (4.0 * dx * dy);
        double d2ndxz = (N_(i + 1, j, k + 1) - N_(i - 1, j, k + 1) - N_(i + 1, j, k - 1) + N_(i - 1, j, k - 1)) /
                        (4.0 * dx * dz);
        double vyz = d8 ? (N_(i + 1, j, k + 1) - N_(i - 1, j, k + 1) - N_(i + 1, j, k - 1) + N_(i - 1, j, k - 1))
                        : (N_(i, j + 1, k + 1) - N_(i, j - 1, k + 1) - N_(i, j + 1, k - 1) + N_(i, j - 1, k - 1));
        double d2ndyz = vyz / (4.0 * dy * dz);
        double d2ndyx = d2ndxy, d2ndzx = d2ndxz, d2ndzy = d2ndyz;
        double Eterm = (R[0][0] * E0x + R[0][1] * E0y + R[0][2] * E0z) * dndx +
                       (R[1][0] * E0x + R[1][1] * E0y + R[1][2] * E0z) * dndy +
                       (R[2][0] * E0x + R[2][1] * E0y + R[2][2] * E0z) * dndz;
        double Pterm = p->cth * (R[0][0] * d2ndxx + R[0][1] * d2ndxy + R[0][2] * d2ndxz + R[1][0] * d2ndyx +
                                 R[1][1] * d2ndyy + R[1][2] * d2ndyz + R[2][0] * d2ndzx + R[2][1] * d2ndzy +
                                 R[2][2] * d2ndzz);
        double Gterm = det * p->cG * (dGxdx + dGydy + dGzdz);
        b[nid(G, i, j, k)] = scale * (Eterm + Pterm + Gterm);
      }
#undef N_
#undef G_
  remove_mean(b, g.N);
}

/* ------------------------------------------------------------------ */
typedef struct coefs { double sxx, syy, szz, sxy, sxz, syz, syx, szx, szy; } coefs;

static coefs full_coefs(const ch_params* p, const grid* g) {
  /* src/lhs.c:404-447 */
  double R[3][3], det;
  kappa_tensor(p, R, &det);
  double hxx = 1.0 / (2.0 * g->dx * g->dx), hyy = 1.0 / (2.0 * g->dy * g->dy), hzz = 1.0 / (2.0 * g->dz * g->dz);
  double hxy = 1.0 / (8.0 * g->dy * g->dx), hxz = 1.0 / (8.0 * g->dz * g->dx), hyz = 1.0 / (8.0 * g->dy * g->dz);
  double scale = 1.0 / det;
  coefs c;
  c.sxx = scale * R[0][0] * hxx; c.syy = scale * R[1][1] * hyy; c.szz = scale * R[2][2] * hzz;
  c.sxy = scale * R[0][1] * hxy; c.sxz = scale * R[0][2] * hxz; c.syz = scale * R[1][2] * hyz;
  c.syx = scale * R[1][0] * hxy; c.szx = scale * R[2][0] * hxz; c.szy = scale * R[2][1] * hyz;
  return c;
}

static const int OFF[19][3] = {{1, 0, 0},  {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},  {0, 0, 1},
                               {0, 0, -1}, {1, 1, 0},  {1, -1, 0},  {-1, 1, 0},  {-1, -1, 0},
                               {1, 0, 1},  {1, 0, -1}, {-1, 0, 1},  {-1, 0, -1}, {0, 1, 1},
                               {0, 1, -1}, {0, -1, 1}, {0, -1, -1}, {0, 0, 0}};

static void row_values(const ch_params* p, const grid* g, const coefs* C, const double* n, int i, int j, int k,
                       double v[19]) {
  if (p->lhs_type == CH_LHS_IDENTITY) {
    for (int s = 0; s < 18; ++s) v[s] = 0.0;
    v[18] = 1.0;
    return;
  }
  if (p->lhs_type == CH_LHS_LAPLACIAN) {
    /* ComputeLaplacianLHS (src/lhs.c:204-218) */
    double sxx = g->dy * g->dz / g->dx, syy = g->dx * g->dz / g->dy, szz = g->dx * g->dy / g->dz;
    for (int s = 0; s < 19; ++s) v[s] = 0.0;
    v[0] = sxx; v[1] = sxx; v[2] = syy; v[3] = syy; v[4] = szz; v[5] = szz;
    v[18] = -(sxx + syy + szz + sxx + syy + szz);
    return;
  }
  /* ComputeFullLHS (src/lhs.c:479-511) */
  double nijk = n[nid(g, i, j, k)];
  double nmjk = n[nid(g, i - 1, j, k)], npjk = n[nid(g, i + 1, j, k)];
  double nimk = n[nid(g, i, j - 1, k)], nipk = n[nid(g, i, j + 1, k)];
  double nijm = n[nid(g, i, j, k - 1)], nijp = n[nid(g, i, j, k + 1)];
  const double sxx = C->sxx, syy = C->syy, szz = C->szz, sxy = C->sxy, sxz = C->sxz, syz = C->syz,
               syx = C->syx, szx = C->szx, szy = C->szy;
  v[6] = sxy * (npjk + nijk) + syx * (nipk + nijk);
  v[7] = -sxy * (npjk + nijk) - syx * (nijk + nimk);
  v[8] = -sxy * (nijk + nmjk) - syx * (nipk + nijk);
  v[9] = sxy * (nijk + nmjk) + syx * (nijk + nimk);
  v[10] = sxz * (npjk + nijk) + szx * (nijp + nijk);
  v[11] = -sxz * (npjk + nijk) - szx * (nijk + nijm);
  v[12] = -sxz * (nijk + nmjk) - szx * (nijp + nijk);
  v[13] = sxz * (nijk + nmjk) + szx * (nijk + nijm);
  v[14] = syz * (nipk + nijk) + szy * (nijp + nijk);
  v[15] = -syz * (nipk + nijk) - szy * (nijk + nijm);
  v[16] = -syz * (nijk + nimk) - szy * (nijp + nijk);
  v[17] = syz * (nijk + nimk) + szy * (nijk + nijm);
  v[0] = sxx * (npjk + nijk) + syx * (nipk - nimk) + szx * (nijp - nijm);
  v[1] = sxx * (nijk + nmjk) - syx * (nipk - nimk) - szx * (nijp - nijm);
  v[2] = syy * (nipk + nijk) + sxy * (npjk - nmjk) + szy * (nijp - nijm);
  v[3] = syy * (nijk + nimk) - sxy * (npjk - nmjk) - szy * (nijp - nijm);
  v[4] = szz * (nijp + nijk) + sxz * (npjk - nmjk) + syz * (nipk - nimk);
  v[5] = szz * (nijk + nijm) - sxz * (npjk - nmjk) - syz * (nipk - nimk);
  v[18] = -(sxx * (npjk + 2 * nijk + nmjk) + syy * (nipk + 2 * nijk + nimk) + szz * (nijp + 2 * nijk + nijm));
}

void orc_lhs_row(const ch_params* p, const double* n, int i, int j, int k, double vals[19], int64_t cols[19]) {
  grid g = mkgrid(p);
  coefs C = full_coefs(p, &g);
  row_values(p, &g, &C, n, i, j, k, vals);
  for (int s = 0; s < 19; ++s) cols[s] = nid(&g, i + OFF[s][0], j + OFF[s][1], k + OFF[s][2]);
}

void orc_apply(const ch_params* p, const double* n, const double* x, double* y) {
  grid g = mkgrid(p);
  coefs C = full_coefs(p, &g);
  const int64_t X = g.Nx, XY = (int64_t)g.Nx * g.Ny;
#pragma omp parallel for num_threads(g_threads) collapse(2) schedule(static)
  for (int k = 0; k < g.Nz; ++k)
    for (int j = 0; j < g.Ny; ++j) {
      const int kp = k + 1 == g.Nz ? 0 : k + 1, km = k == 0 ? g.Nz - 1 : k - 1;
      const int jp = j + 1 == g.Ny ? 0 : j + 1, jm = j == 0 ? g.Ny - 1 : j - 1;
      for (int i = 0; i < g.Nx; ++i) {
        const int ip = i + 1 == g.Nx ? 0 : i + 1, im = i == 0 ? g.Nx - 1 : i - 1;
        /* natural indices of the 19 stencil points in ComputeInteriorStencil order */
        const int64_t c[19] = {k * XY + j * X + ip,   k * XY + j * X + im,   k * XY + jp * X + i,
                               k * XY + jm * X + i,   kp * XY + j * X + i,   km * XY + j * X + i,
                               k * XY + jp * X + ip,  k * XY + jm * X + ip,  k * XY + jp * X + im,
                               k * XY + jm * X + im,  kp * XY + j * X + ip,  km * XY + j * X + ip,
                               kp * XY + j * X + im,  km * XY + j * X + im,  kp * XY + jp * X + i,
                               km * XY + jp * X + i,  kp * XY + jm * X + i,  km * XY + jm * X + i,
                               k * XY + j * X + i};
        double v[19];
        row_values(p, &g, &C, n, i, j, k, v);
        double acc = 0.0;
        for (int s2 = 0; s2 < 19; ++s2) acc += v[s2] * x[c[s2]];
        y[c[18]] = acc;
      }
    }
}

static double dot(const double* a, const double* b, int64_t N) {
  double s = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < N; ++i) s += a[i] * b[i];
  return s;
}

static void diag_of(const ch_params* p, const double* n, double* dinv, int64_t N) {
  grid g = mkgrid(p);
  coefs C = full_coefs(p, &g);
  for (int k = 0; k < g.Nz; ++k)
    for (int j = 0; j < g.Ny; ++j)
      for (int i = 0; i < g.Nx; ++i) {
        double v[19];
        row_values(p, &g, &C, n, i, j, k, v);
        dinv[nid(&g, i, j, k)] = v[18] != 0.0 ? 1.0 / v[18] : 1.0;
      }
  (void)N;
}

int orc_solve(const ch_params* p, const double* n, const double* b, double* phi, double rtol, int maxit, int* its,
              double* rnorm, double* bnorm) {
  grid g = mkgrid(p);
  const int64_t N = g.N;
  const int singular = p->lhs_type != CH_LHS_IDENTITY;
  double* w = (double*)calloc((size_t)N * 8, sizeof(double));
  if (!w) return CH_ERR_NOMEM;
  double *r = w, *z = w + N, *pp = w + 2 * N, *q = w + 3 * N, *rh = w + 4 * N, *sv = w + 5 * N, *tv = w + 6 * N,
         *dinv = w + 7 * N;
  const int jac = p->pc_type == CH_PC_JACOBI;
  if (jac) diag_of(p, n, dinv, N);
  double bn = sqrt(dot(b, b, N));
  double tol = fmax(rtol * bn, p->ksp_atol);
  if (singular) remove_mean(phi, N);
  orc_apply(p, n, phi, q);
  #pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t i = 0; i < N; ++i) r[i] = b[i] - q[i];
  double rn = sqrt(dot(r, r, N));
  int it = 0, rc = 0;
#define PREC(dst, src)                                            \
  do {                                                            \
    _Pragma("omp parallel for num_threads(g_threads) schedule(static)") \
    for (int64_t i_ = 0; i_ < N; ++i_) (dst)[i_] = jac ? (src)[i_] * dinv[i_] : (src)[i_]; \
    if (singular) remove_mean((dst), N);                          \
  } while (0)
  /* Krylov iterations; when the recurrence says converged but the true
   * residual b - A phi (checked below) is still above tol -- the recurrence
   * drifts near FP64's floor at tight rtol -- restart from the true residual */
  for (int restart = 0; restart < 8 && rn > tol && it < maxit; ++restart) {
    if (restart > 0) {
      orc_apply(p, n, phi, q);
      #pragma omp parallel for num_threads(g_threads) schedule(static)
      for (int64_t i = 0; i < N; ++i) r[i] = b[i] - q[i];
      rn = sqrt(dot(r, r, N));
      if (rn <= tol) break;
    }
    if (p->ksp_type == CH_KSP_CG) {
      PREC(z, r);
      #pragma omp parallel for num_threads(g_threads) schedule(static)
      for (int64_t i = 0; i < N; ++i) pp[i] = z[i];
      double rz = dot(r, z, N);
      while (it < maxit) {
        orc_apply(p, n, pp, q);
        double pq = dot(pp, q, N);
        double alpha = rz / pq;
        #pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int64_t i = 0; i < N; ++i) { phi[i] += alpha * pp[i]; r[i] -= alpha * q[i]; }
        ++it;
        rn = sqrt(dot(r, r, N));
        if (rn <= tol) break;
        PREC(z, r);
        double rz2 = dot(r, z, N);
        double beta = rz2 / rz;
        rz = rz2;
        #pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int64_t i = 0; i < N; ++i) pp[i] = z[i] + beta * pp[i];
      }
    } else {
      /* BiCGStab (van der Vorst 1992), right preconditioned */
      #pragma omp parallel for num_threads(g_threads) schedule(static)
      for (int64_t i = 0; i < N; ++i) { rh[i] = r[i]; pp[i] = 0.0; sv[i] = 0.0; }
      double rho = 1.0, alpha = 1.0, omega = 1.0;
      double* vv = sv; /* v vector */
      double* y = z;   /* preconditioned direction */
      double* s = tv;
      double* ts = q;  /* reused: t = A s_hat */
      double* sh = (double*)calloc((size_t)N * 2, sizeof(double));
      double* vvec = sh + N;
      (void)vv;
      while (it < maxit) {
        double rho1 = dot(rh, r, N);
        if (rho1 == 0.0) break;
        double beta = (rho1 / rho) * (alpha / omega);
        rho = rho1;
        #pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int64_t i = 0; i < N; ++i) pp[i] = r[i] + beta * (pp[i] - omega * vvec[i]);
        PREC(y, pp);
        orc_apply(p, n, y, vvec);
        alpha = rho / dot(rh, vvec, N);
        #pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int64_t i = 0; i < N; ++i) s[i] = r[i] - alpha * vvec[i];
        ++it;
        double sn = sqrt(dot(s, s, N));
        if (sn <= tol) {
          #pragma omp parallel for num_threads(g_threads) schedule(static)
          for (int64_t i = 0; i < N; ++i) phi[i] += alpha * y[i];
          #pragma omp parallel for num_threads(g_threads) schedule(static)
          for (int64_t i = 0; i < N; ++i) r[i] = s[i];
          rn = sn;
          break;
        }
        PREC(sh, s);
        orc_apply(p, n, sh, ts);
        omega = dot(ts, s, N) / dot(ts, ts, N);
        #pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int64_t i = 0; i < N; ++i) {
          phi[i] += alpha * y[i] + omega * sh[i];
          r[i] = s[i] - omega * ts[i];
        }
        rn = sqrt(dot(r, r, N));
        if (rn <= tol || omega == 0.0) break;
      }
      free(sh);
    }
    /* true residual of this pass */
    orc_apply(p, n, phi, q);
    #pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < N; ++i) r[i] = b[i] - q[i];
    rn = sqrt(dot(r, r, N));
  }
#undef PREC
  if (singular) remove_mean(phi, N);
  /* true residual */
  orc_apply(p, n, phi, q);
  #pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t i = 0; i < N; ++i) r[i] = b[i] - q[i];
  rn = sqrt(dot(r, r, N));
  if (rn > tol * 1.0000001 && rn > 0.0) rc = CH_ERR_NOT_CONVERGED;
  if (its) *its = it;
  if (rnorm) *rnorm = rn;
  if (bnorm) *bnorm = bn;
  free(w);
  return rc;
}

/* ------------------------------------------------------------------ */
static int potential(orc_state* s, int* its, double* rnorm, double* bnorm) {
  const ch_params* p = &s->p;
  int64_t N = (int64_t)p->Nx * p->Ny * p->Nz;
  orc_rhs(p, s->nodes, s->rhs);
  double* n = s->n_frozen;
  if (!(p->faithful & CH_FAITHFUL_D7) || !s->solved_once)
    for (int64_t c = 0; c < N; ++c) n[c] = s->nodes[4 * c];
  if (!s->solved_once) memset(s->phi, 0, sizeof(double) * N); /* ComputeInitialPhi */
  int rc = orc_solve(p, n, s->rhs, s->phi, p->ksp_rtol, p->ksp_max_it, its, rnorm, bnorm);
  s->solved_once = 1;
  return rc;
}

int orc_initialize(orc_state* s, int* its, double* rnorm, double* bnorm) {
  orc_collect(&s->p, &s->P, s->nodes, 0);
  s->sbar = s->p.mn > 0.0 ? orc_sbar(&s->p, &s->P) : 0.0;
  s->solved_once = 0;
  return potential(s, its, rnorm, bnorm);
}

int orc_step(orc_state* s, int64_t step, orc_counters* cnt, int* its, double* rnorm, double* bnorm) {
  double snext = 0.0;
  int rc = orc_update_velocities(&s->p, s->phi, &s->P, step, s->sbar, &snext, cnt);
  if (s->p.mn > 0.0) s->sbar = snext;
  if (rc) return rc;
  orc_update_positions(&s->p, &s->P);
  orc_collect(&s->p, &s->P, s->nodes, (s->p.faithful & CH_FAITHFUL_D6) != 0);
  return potential(s, its, rnorm, bnorm);
}

/* ------------------------------------------------------------------ */
/* Centre-of-mass scatter of one frozen event (src/particles.c:552-591,
 * the formula of collide_ion above) with the neutral velocity V given. */
static void scatter_event(double* vx, double* vy, double* vz, const double V[3], double uz, double uphi_frac,
                          double mi, double mn) {
  const double M = mi + mn;
  const double vix = *vx, viy = *vy, viz = *vz;
  const double uphi = 2.0 * PI * uphi_frac;
  double vrx = vix - V[0], vry = viy - V[1], vrz = viz - V[2];
  double vrr = sqrt(vrx * vrx + vry * vry + vrz * vrz);
  double vcx = (vix * mi + V[0] * mn) / M, vcy = (viy * mi + V[1] * mn) / M, vcz = (viz * mi + V[2] * mn) / M;
  double ax = vix - vcx, ay = viy - vcy, az = viz - vcz;
  double vcr = sqrt(ax * ax + ay * ay + az * az);
  double uperp = sqrt(fmax(0.0, 1.0 - uz * uz));
  double ux = uperp * cos(uphi), uy = uperp * sin(uphi);
  double costht = vrr > 0.0 ? vrz / vrr : 1.0;
  double sintht = sqrt(fmax(0.0, 1.0 - costht * costht));
  double cosphi = 1.0, sinphi = 0.0;
  if (vrr * sintht > 0.0) { cosphi = vrx / (vrr * sintht); sinphi = vry / (vrr * sintht); }
  double ux1 = uz * sintht + ux * costht, uy1 = uy, uz1 = uz * costht - ux * sintht;
  double ux2 = ux1 * cosphi - uy1 * sinphi, uy2 = ux1 * sinphi + uy1 * cosphi, uz2 = uz1;
  *vx = vcx + vcr * ux2; *vy = vcy + vcr * uy2; *vz = vcz + vcr * uz2;
}

int orc_adj_objective(const ch_params* p, const ch_loader* L, int64_t np, int nsteps, int window,
                      double flux_weight, double phi_weight, int64_t nev, const int32_t* ev_step,
                      const uint32_t* ev_ion, const int32_t* ev_flags, const double* ev_data, double rtol,
                      double* J) {
  grid g = mkgrid(p);
  const int64_t N = g.N;
  orc_particles P;
  P.np = np;
  double* buf = (double*)malloc(sizeof(double) * 6 * (size_t)np);
  double* nodes = (double*)calloc((size_t)N * 4, sizeof(double));
  double* b = (double*)malloc(sizeof(double) * N);
  double* phi = (double*)calloc((size_t)N, sizeof(double));
  double* n = (double*)malloc(sizeof(double) * N);
  double* E = (double*)malloc(sizeof(double) * 3 * N);
  int64_t* start = (int64_t*)malloc(sizeof(int64_t) * (size_t)np);
  if (!buf || !nodes || !b || !phi || !n || !E || !start) {
    free(buf); free(nodes); free(b); free(phi); free(n); free(E); free(start);
    return CH_ERR_NOMEM;
  }
  P.x = buf; P.y = buf + np; P.z = buf + 2 * np; P.vx = buf + 3 * np; P.vy = buf + 4 * np; P.vz = buf + 5 * np;
  orc_load(p, L, &P);
  int its, rc = 0;
  double rn, bn;
  orc_collect(p, &P, nodes, 0);
  orc_rhs(p, nodes, b);
  for (int64_t c = 0; c < N; ++c) n[c] = nodes[4 * c];
  rc = orc_solve(p, n, b, phi, rtol, p->ksp_max_it, &its, &rn, &bn);
  const double tscale = 0.5 * (p->qi / p->mi) * p->dt;
  double t[3], s[3];
  for (int d = 0; d < 3; ++d) t[d] = tscale * p->B0[d];
  const double tt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
  for (int d = 0; d < 3; ++d) s[d] = 2.0 * t[d] / (1.0 + tt);
  double Jsum = 0.0;
  int64_t e0 = 0;
  for (int st = 0; st < nsteps && rc == 0; ++st) {
    int64_t e1 = e0;
    while (e1 < nev && ev_step[e1] == st) ++e1;
    for (int64_t i = 0; i < np; ++i) start[i] = -1;
    for (int64_t e = e1 - 1; e >= e0; --e) start[ev_ion[e]] = e;  /* first event of each ion */
    orc_node_efield(p, phi, E, E + N, E + 2 * N);
    double sumvx = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : sumvx) schedule(static)
    for (int64_t ip = 0; ip < np; ++ip) {
      double X = (P.x[ip] - g.x0) / g.dx, Y = (P.y[ip] - g.y0) / g.dy, Z = (P.z[ip] - g.z0) / g.dz;
      int i = (int)floor(X), j = (int)floor(Y), k = (int)floor(Z);
      double wx = X - i, wy = Y - j, wz = Z - k;
      int64_t c000 = nid(&g, i, j, k), c100 = nid(&g, i + 1, j, k), c010 = nid(&g, i, j + 1, k),
              c110 = nid(&g, i + 1, j + 1, k), c001 = nid(&g, i, j, k + 1), c101 = nid(&g, i + 1, j, k + 1),
              c011 = nid(&g, i, j + 1, k + 1), c111 = nid(&g, i + 1, j + 1, k + 1);
      double Ef[3];
      for (int d = 0; d < 3; ++d) {
        const double* e = E + d * N;
        double wll = e[c000] + wy * (e[c010] - e[c000]);
        double wlh = e[c100] + wy * (e[c110] - e[c100]);
        double whl = e[c001] + wy * (e[c011] - e[c001]);
        double whh = e[c101] + wy * (e[c111] - e[c101]);
        double ezl = wll + wx * (wlh - wll);
        double ezh = whl + wx * (whh - whl);
        Ef[d] = ezl + wz * (ezh - ezl);
      }
      if (p->push_E0) { Ef[0] += p->E0[0]; Ef[1] += p->E0[1]; Ef[2] += p->E0[2]; }
      double vm[3] = {P.vx[ip] + tscale * Ef[0], P.vy[ip] + tscale * Ef[1], P.vz[ip] + tscale * Ef[2]};
      double c1[3] = {vm[1] * t[2] - vm[2] * t[1], vm[2] * t[0] - vm[0] * t[2], vm[0] * t[1] - vm[1] * t[0]};
      double vpr[3] = {vm[0] + c1[0], vm[1] + c1[1], vm[2] + c1[2]};
      double c2[3] = {vpr[1] * s[2] - vpr[2] * s[1], vpr[2] * s[0] - vpr[0] * s[2], vpr[0] * s[1] - vpr[1] * s[0]};
      double vx = vm[0] + c2[0] + tscale * Ef[0], vy = vm[1] + c2[1] + tscale * Ef[1],
             vz = vm[2] + c2[2] + tscale * Ef[2];
      if (p->mn > 0.0 && start[ip] >= 0)
        for (int64_t e = start[ip]; e < e1 && ev_ion[e] == (uint32_t)ip; ++e) {
          if (ev_flags[e] & 1) continue;
          const double* q = ev_data + 5 * e;
          const double V[3] = {p->vn0[0] + q[0], p->vn0[1] + q[1], p->vn0[2] + q[2]};
          scatter_event(&vx, &vy, &vz, V, q[3], q[4], p->mi, p->mn);
        }
      P.vx[ip] = vx; P.vy[ip] = vy; P.vz[ip] = vz;
      sumvx += vx;
    }
    e0 = e1;
    orc_update_positions(p, &P);
    orc_collect(p, &P, nodes, 0);
    orc_rhs(p, nodes, b);
    for (int64_t c = 0; c < N; ++c) n[c] = nodes[4 * c];
    rc = orc_solve(p, n, b, phi, rtol, p->ksp_max_it, &its, &rn, &bn);
    if (st >= nsteps - window) {
      double s2 = 0.0;
      for (int64_t c = 0; c < N; ++c) s2 += phi[c] * phi[c];
      Jsum += flux_weight / ((double)window * (double)N) * sumvx + phi_weight / ((double)window * (double)N) * s2;
    }
  }
  *J = Jsum;
  free(buf); free(nodes); free(b); free(phi); free(n); free(E); free(start);
  return rc;
}

/* sizeof(ch_params) as the C compiler lays it out, for the binding checks. */
int64_t orc_sizeof_params(void) { return (int64_t)sizeof(ch_params); }
