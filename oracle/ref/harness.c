/*
 * harness.c -- drives the reference's own hot-path functions, compiled
 * unmodified from its src/ directory against the PETSc stand-in, on plain
 * arrays.  TEST INFRASTRUCTURE ONLY: its outputs are the golden vectors
 * that pin the oracle (tests/golden/make_golden.py).
 *
 * Reference functions driven:
 *   CollectVlasovQuantities  src/particles.c:136-255
 *   UpdatePositions          src/particles.c:647-718
 *   ComputeCollisions        src/particles.c:471-624  (with src/random.c)
 *   DifferenceVector         src/vectors.c:12-138
 *   ComputeFullLHS / ComputeLaplacianLHS / ComputeIdentityLHS  src/lhs.c
 *   ComputeFullRHS / ComputeConstantRHS / ComputeSinusoidalRHS src/rhs.c
 *   dFdx ... d2Fdzy          src/calculus.c
 */
#include "hybrid.h"
#include "distributions.h"
#include "calculus.h"
#include "particles.h"
#include "random.h"
#include "vectors.h"
#include "standin.h"

/* InitializePositions (src/particles.c:9) names these loaders; the harness
 * never calls it, so they only need to link. */
PetscErrorCode SobolDistribution(Context* ctx) { (void)ctx; return PETSC_ERR_ARG_WRONG; }
PetscErrorCode UniformDistribution(Context* ctx) { (void)ctx; return PETSC_ERR_ARG_WRONG; }
PetscErrorCode SinusoidalDistribution(PetscReal x, PetscReal y, PetscReal z, PetscReal* v, Context* ctx) {
  (void)x; (void)y; (void)z; (void)v; (void)ctx;
  return PETSC_ERR_ARG_WRONG;
}
PetscErrorCode Rejection(DistributionFunction density, Context* ctx) { (void)density; (void)ctx; return PETSC_ERR_ARG_WRONG; }
const char* DensityTypes[] = {"flat-sobol", "flat-reverse", "flat-normal", "uniform", "sinusoidal", "gaussian", NULL};

extern DM ch_standin_matdm;

static const char* const VLASOV_NAMES[4] = {"density", "x flux", "y flux", "z flux"};

static void setup_grid(Context* ctx, int Nx, int Ny, int Nz, const double L[3]) {
  memset(ctx, 0, sizeof(*ctx));
  ctx->grid.N.x = Nx; ctx->grid.N.y = Ny; ctx->grid.N.z = Nz;
  ctx->grid.p0.x = 0.0; ctx->grid.p0.y = 0.0; ctx->grid.p0.z = 0.0;
  ctx->grid.p1.x = L[0]; ctx->grid.p1.y = L[1]; ctx->grid.p1.z = L[2];
  ctx->grid.L.x = L[0]; ctx->grid.L.y = L[1]; ctx->grid.L.z = L[2];
  ctx->grid.d.x = L[0] / Nx; ctx->grid.d.y = L[1] / Ny; ctx->grid.d.z = L[2] / Nz;
  ctx->vlasovDM = ch_standin_dmda(Nx, Ny, Nz, 4, VLASOV_NAMES);
  DMCreateGlobalVector(ctx->vlasovDM, &ctx->vlasov);
}

static void teardown(Context* ctx) {
  VecDestroy(&ctx->vlasov);
  DMDestroy(&ctx->vlasovDM);
  if (ctx->ionsDM) DMDestroy(&ctx->ionsDM);
}

/* CollectVlasovQuantities called ncalls times on the same ions (the global
 * vector is zeroed once, as SetUpVlasovDM does; src/setup.c:61). */
int ref_collect(int Nx, int Ny, int Nz, const double L[3], int np, const double* pos, const double* vel, int ncalls,
                double* out) {
  Context ctx;
  setup_grid(&ctx, Nx, Ny, Nz, L);
  ctx.ionsDM = ch_standin_swarm(ctx.vlasovDM, np);
  memcpy(ctx.ionsDM->position, pos, sizeof(double) * 4 * np);
  memcpy(ctx.ionsDM->velocity, vel, sizeof(double) * 4 * np);
  int rc = 0;
  for (int c = 0; c < ncalls && !rc; ++c) rc = CollectVlasovQuantities(&ctx);
  memcpy(out, ctx.vlasov->a, sizeof(double) * 4 * Nx * Ny * Nz);
  ctx.ionsDM->celldm = NULL;
  teardown(&ctx);
  return rc;
}

/* UpdatePositions on the given ions; positions are copied back out. */
int ref_update_positions(int Nx, int Ny, int Nz, const double L[3], double dt, int np, double* pos, const double* vel) {
  Context ctx;
  setup_grid(&ctx, Nx, Ny, Nz, L);
  ctx.dt = dt;
  ctx.ionsDM = ch_standin_swarm(ctx.vlasovDM, np);
  memcpy(ctx.ionsDM->position, pos, sizeof(double) * 4 * np);
  memcpy(ctx.ionsDM->velocity, vel, sizeof(double) * 4 * np);
  int rc = UpdatePositions(&ctx);
  memcpy(pos, ctx.ionsDM->position, sizeof(double) * 4 * np);
  ctx.ionsDM->celldm = NULL;
  teardown(&ctx);
  return rc;
}

/* DifferenceVector at cell-unit points (X, Y, Z) from phi in natural order. */
int ref_difference_vector(int Nx, int Ny, int Nz, const double* phi, int npts, const double* xyz, double* f) {
  DM dm = ch_standin_dmda(Nx, Ny, Nz, 1, NULL);
  Vec g, l;
  DMCreateGlobalVector(dm, &g);
  memcpy(g->a, phi, sizeof(double) * Nx * Ny * Nz);
  DMGetLocalVector(dm, &l);
  DMGlobalToLocal(dm, g, INSERT_VALUES, l);
  PetscReal*** F;
  DMDAVecGetArray(dm, l, &F);
  Grid grid;
  memset(&grid, 0, sizeof(grid));
  grid.N.x = Nx; grid.N.y = Ny; grid.N.z = Nz;
  int rc = 0;
  for (int q = 0; q < npts && !rc; ++q) rc = DifferenceVector(F, xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2], grid, f + 3 * q);
  DMDAVecRestoreArray(dm, l, &F);
  VecDestroy(&l);
  VecDestroy(&g);
  DMDestroy(&dm);
  return rc;
}

static void set_electrons(Context* ctx, const double kappa[3], double cth, double cG) {
  ctx->electrons.kappa.x = kappa[0]; ctx->electrons.kappa.y = kappa[1]; ctx->electrons.kappa.z = kappa[2];
  /* cth = gamma KB T / Q and cG = m nu / Q (src/rhs.c:190-191) */
  ctx->electrons.gamma = 1.0;
  ctx->electrons.T = cth * Q / KB;
  ctx->electrons.nu = 1.0;
  ctx->electrons.m = cG * Q;
}

/* LHS operator rows: cols/vals are N x 27 (row-major), ncols N. */
int ref_lhs(int Nx, int Ny, int Nz, const double L[3], const double kappa[3], int lhs_type, const double* nodes,
            int* ncols, int* cols, double* vals) {
  Context ctx;
  setup_grid(&ctx, Nx, Ny, Nz, L);
  set_electrons(&ctx, kappa, 1.0, 0.0);
  ctx.stencilFunc = ComputePeriodicStencil;
  int N = Nx * Ny * Nz;
  memcpy(ctx.vlasov->a, nodes, sizeof(double) * 4 * N);
  struct _p_KSP ksp;
  ksp.dm = ch_standin_dmda(Nx, Ny, Nz, 1, NULL);
  ksp.A = ch_standin_mat(N);
  DMCreateGlobalVector(ksp.dm, &ksp.sol);
  ch_standin_matdm = ksp.dm;
  int rc;
  if (lhs_type == 0) {
    for (int r = 0; r < N; ++r) { ksp.A->ncols[r] = 1; ksp.A->cols[r * 27] = r; }
    rc = ComputeIdentityLHS(&ksp, ksp.A, ksp.A, &ctx);
  } else if (lhs_type == 1) {
    rc = ComputeLaplacianLHS(&ksp, ksp.A, ksp.A, &ctx);
  } else {
    rc = ComputeFullLHS(&ksp, ksp.A, ksp.A, &ctx);
  }
  memcpy(ncols, ksp.A->ncols, sizeof(int) * N);
  memcpy(cols, ksp.A->cols, sizeof(int) * N * 27);
  memcpy(vals, ksp.A->vals, sizeof(double) * N * 27);
  ch_standin_mat_free(ksp.A);
  VecDestroy(&ksp.sol);
  DMDestroy(&ksp.dm);
  teardown(&ctx);
  return rc;
}

/* RHS vector b (natural order) from the dof-4 moments. */
int ref_rhs(int Nx, int Ny, int Nz, const double L[3], const double kappa[3], const double E0[3], double cth,
            double cG, int rhs_type, const double* nodes, double* b) {
  Context ctx;
  setup_grid(&ctx, Nx, Ny, Nz, L);
  set_electrons(&ctx, kappa, cth, cG);
  ctx.plasma.E0.x = E0[0]; ctx.plasma.E0.y = E0[1]; ctx.plasma.E0.z = E0[2];
  int N = Nx * Ny * Nz;
  memcpy(ctx.vlasov->a, nodes, sizeof(double) * 4 * N);
  struct _p_KSP ksp;
  ksp.dm = ch_standin_dmda(Nx, Ny, Nz, 1, NULL);
  ksp.A = NULL;
  DMCreateGlobalVector(ksp.dm, &ksp.sol);
  Vec bv;
  DMCreateGlobalVector(ksp.dm, &bv);
  int rc;
  if (rhs_type == 0) rc = ComputeConstantRHS(&ksp, bv, &ctx);
  else if (rhs_type == 1) rc = ComputeSinusoidalRHS(&ksp, bv, &ctx);
  else rc = ComputeFullRHS(&ksp, bv, &ctx);
  memcpy(b, bv->a, sizeof(double) * N);
  VecDestroy(&bv);
  VecDestroy(&ksp.sol);
  DMDestroy(&ksp.dm);
  teardown(&ctx);
  return rc;
}

/* ComputeCollisions on the given velocities (np x 4, in place).  Returns the
 * reference's status; *nc receives its collision count Nc. */
int ref_collisions(int np, double* vel, const double viT[3], const double vi0[3], double nu, double dt, double mi,
                   double mn, double vnT, const double vn0[3], long seed, int* nc) {
  Context ctx;
  double L[3] = {1, 1, 1};
  setup_grid(&ctx, 2, 2, 2, L);
  ctx.ionsDM = ch_standin_swarm(ctx.vlasovDM, np);
  memcpy(ctx.ionsDM->velocity, vel, sizeof(double) * 4 * np);
  ctx.plasma.Np = np;
  ctx.ions.nu = nu;
  ctx.dt = dt;
  ctx.ions.m = mi;
  ctx.ions.vT.x = viT[0]; ctx.ions.vT.y = viT[1]; ctx.ions.vT.z = viT[2];
  ctx.ions.vT.r = sqrt(viT[0] * viT[0] + viT[1] * viT[1] + viT[2] * viT[2]);
  ctx.ions.v0.x = vi0[0]; ctx.ions.v0.y = vi0[1]; ctx.ions.v0.z = vi0[2];
  ctx.neutrals.m = mn;
  ctx.neutrals.vT = vnT;
  ctx.neutrals.v0.x = vn0[0]; ctx.neutrals.v0.y = vn0[1]; ctx.neutrals.v0.z = vn0[2];
  ctx.neutrals.v0.r = sqrt(vn0[0] * vn0[0] + vn0[1] * vn0[1] + vn0[2] * vn0[2]);
  ctx.seed = seed;
  /* the count formula of src/particles.c:511-519, reported for the tests */
  double vrm = 4.0 * ctx.ions.vT.r + sqrt(PetscSqr(vi0[0] - vn0[0]) + PetscSqr(vi0[1] - vn0[1]) + PetscSqr(vi0[2] - vn0[2]));
  int Nc = (int)(((double)np * nu * dt * vrm) / ((vnT + ctx.neutrals.v0.r) * sqrt(mn / mi)));
  if (Nc > np) Nc = np;
  if (Nc < 0) Nc = 0;
  *nc = Nc;
  int rc = ComputeCollisions(&ctx);
  memcpy(vel, ctx.ionsDM->velocity, sizeof(double) * 4 * np);
  ctx.ionsDM->celldm = NULL;
  teardown(&ctx);
  return rc;
}

/* The calculus helpers at one interior node of a ghosted field, for the
 * FD-stencil pins: out[0..14] in the order ComputeFullRHS calls them. */
int ref_calculus(int Nx, int Ny, int Nz, const double L[3], const double* F, int i, int j, int k, double* out) {
  DM dm = ch_standin_dmda(Nx, Ny, Nz, 1, NULL);
  Vec g, l;
  DMCreateGlobalVector(dm, &g);
  memcpy(g->a, F, sizeof(double) * Nx * Ny * Nz);
  DMGetLocalVector(dm, &l);
  DMGlobalToLocal(dm, g, INSERT_VALUES, l);
  PetscReal*** A;
  DMDAVecGetArray(dm, l, &A);
  double dx = L[0] / Nx, dy = L[1] / Ny, dz = L[2] / Nz;
  int rc = 0;
  rc |= dFdx(A, dx, i, j, k, &out[0], CENTERED);
  rc |= dFdy(A, dy, i, j, k, &out[1], CENTERED);
  rc |= dFdz(A, dz, i, j, k, &out[2], CENTERED);
  rc |= d2Fdxx(A, dx, i, j, k, &out[3], CENTERED);
  rc |= d2Fdyy(A, dy, i, j, k, &out[4], CENTERED);
  rc |= d2Fdzz(A, dz, i, j, k, &out[5], CENTERED);
  rc |= d2Fdxy(A, dx, dy, i, j, k, &out[6], CENTERED, CENTERED);
  rc |= d2Fdyx(A, dy, dx, i, j, k, &out[7], CENTERED, CENTERED);
  rc |= d2Fdxz(A, dx, dz, i, j, k, &out[8], CENTERED, CENTERED);
  rc |= d2Fdzx(A, dz, dx, i, j, k, &out[9], CENTERED, CENTERED);
  rc |= d2Fdyz(A, dy, dz, i, j, k, &out[10], CENTERED, CENTERED);
  rc |= d2Fdzy(A, dz, dy, i, j, k, &out[11], CENTERED, CENTERED);
  DMDAVecRestoreArray(dm, l, &A);
  VecDestroy(&l);
  VecDestroy(&g);
  DMDestroy(&dm);
  return rc;
}
