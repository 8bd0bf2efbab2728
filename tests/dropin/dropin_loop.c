/* Runs the reference's loop order (src/hybrid.c:94-123) through the GPU
 * drop-in (petsc_dropin.c) on the PETSc stand-in, with the options given on
 * the command line, and prints what reached the C ABI (fake_chybrid.c).
 * TEST ONLY. */
#include <stdio.h>
#include <string.h>

#include "hybrid.h"
#include "particles.h"
#include "potential.h"
#include "standin.h"

void fake_report(FILE* f);

int main(int argc, char** argv) {
  ch_standin_options(argc - 1, (const char* const*)argv + 1);
  double kz = 0.0;
  PetscBool set = PETSC_FALSE;
  PetscOptionsGetReal(NULL, NULL, "-test_kappa_z", &kz, &set);
  Context ctx;
  memset(&ctx, 0, sizeof(ctx));
  ctx.grid.N.x = 8; ctx.grid.N.y = 8; ctx.grid.N.z = 8;
  ctx.grid.p1.x = 8.0; ctx.grid.p1.y = 8.0; ctx.grid.p1.z = 8.0;
  ctx.ions.q = 1.0; ctx.ions.m = 1.0; ctx.ions.nu = 0.1;
  ctx.ions.vT.x = ctx.ions.vT.y = ctx.ions.vT.z = 1.0;
  ctx.neutrals.m = 1.0; ctx.neutrals.vT = 1.0;
  ctx.plasma.B0.z = 1.0;
  ctx.electrons.kappa.z = kz;
  ctx.electrons.gamma = 1.0;
  ctx.lhsType = LHS_FULL;
  ctx.rhsType = RHS_FULL;
  ctx.dt = 0.05;
  ctx.seed = -12345;
  const char* names[4] = {"density", "x flux", "y flux", "z flux"};
  ctx.vlasovDM = ch_standin_dmda(8, 8, 8, 4, names);
  ctx.vlasov = ch_standin_global(ctx.vlasovDM);
  ctx.ionsDM = ch_standin_swarm(ctx.vlasovDM, 2048);
  DM phidm = ch_standin_dmda(8, 8, 8, 1, NULL);
  KSP ksp = ch_standin_ksp(phidm);
  int rc = CollectVlasovQuantities(&ctx);
  if (!rc) rc = ComputePotential(ksp, &ctx);
  for (int it = 0; it < 3 && !rc; ++it) {
    rc = UpdateVelocities(ksp, &ctx);
    if (!rc) rc = UpdatePositions(&ctx);
    if (!rc) rc = CollectVlasovQuantities(&ctx);
    if (!rc) rc = ComputePotential(ksp, &ctx);
  }
  printf("status %d\n", rc);
  fake_report(stdout);
  return rc ? 1 : 0;
}
