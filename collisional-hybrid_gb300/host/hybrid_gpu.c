/*
 * hybrid_gpu.c -- the reference's PIC driver (src/hybrid.c:18-144) on the
 * GPU through the C ABI, without PETSc: same option names, same step order
 *   UpdateVelocities -> UpdatePositions -> CollectVlasovQuantities ->
 *   ComputePotential
 * for Nt steps, printing one summary line per step.  Ions are placed on the
 * device by the reference's --density-type (default flat-sobol), or, with
 * -ch_amp* / -ch_phase*, by the inverse CDF of those density modes.
 *
 *   hybrid_gpu -Nx 32 -Ny 32 -Nz 32 -x1 32 -y1 32 -z1 32 -Np 524288 -viT 1
 *              -B0z 1 -E0x 0.5 -nui 0.1 -dt 0.05 -Nt 100 -ch_vnT 1 ...
 *
 * Exit status 0 on success, 1 on a reported error (message on stderr).
 */
#include <stdio.h>
#include <string.h>
#include <time.h>

#include "ch_options.h"

#define CHECK(call)                                                                 \
  do {                                                                              \
    ch_status rc_ = (call);                                                         \
    if (rc_ != CH_OK) {                                                             \
      fprintf(stderr, "%s failed (%d): %s\n", #call, (int)rc_, ch_last_error());    \
      if (ctx) ch_destroy(ctx);                                                     \
      return 1;                                                                     \
    }                                                                               \
  } while (0)

int main(int argc, char** argv) {
  ch_params p;
  ch_run_options r;
  char err[256] = "";
  ch_ctx* ctx = NULL;
  if (ch_parse_options(argc, argv, &p, &r, err, (int)sizeof(err)) != CH_OK) {
    fprintf(stderr, "options: %s\n", err);
    return 1;
  }
  time_t t0 = time(NULL);
  CHECK(ch_create(&p, -1, &ctx));
  ch_loader L;
  memset(&L, 0, sizeof(L));
  for (int m = 0; m < 3; ++m) {
    L.amp[m] = r.amp[m];
    L.phase[m] = r.phase[m];
    L.v0[m] = p.vi0[m];
    L.vT[m] = p.viT[m];
  }
  if (r.use_modes)
    CHECK(ch_particles_load(ctx, r.Np, &L));
  else
    CHECK(ch_particles_load_placed(ctx, r.Np, &L, r.density_type)); /* InitializePositions, src/hybrid.c:57 */
  ch_step_info info;
  ch_solve_info sinfo;
  CHECK(ch_collect_moments(ctx, NULL, &info));         /* src/hybrid.c:67 */
  CHECK(ch_compute_potential(ctx, NULL, &sinfo));      /* src/hybrid.c:81 */
  printf("initial: n_sum %.6e  ksp its %d  |r|/|b| %.3e\n", info.moment_sum[0], sinfo.iterations,
         sinfo.bnorm > 0 ? sinfo.rnorm / sinfo.bnorm : 0.0);
  for (int it = 0; it < r.Nt; ++it) {                  /* src/hybrid.c:101-123 */
    memset(&info, 0, sizeof(info));
    CHECK(ch_update_velocities(ctx, it, &info));
    CHECK(ch_update_positions(ctx));
    CHECK(ch_collect_moments(ctx, NULL, &info));
    CHECK(ch_compute_potential(ctx, NULL, &sinfo));
    printf("Time step %d: collisions %lld (Nc %lld)  n_sum %.6e  ksp its %d  |r|/|b| %.3e\n", it,
           (long long)info.collisions, (long long)info.Nc, info.moment_sum[0], sinfo.iterations,
           sinfo.bnorm > 0 ? sinfo.rnorm / sinfo.bnorm : 0.0);
  }
  CHECK(ch_destroy(ctx));
  ctx = NULL;
  printf("Elapsed time: %.0f s\n", difftime(time(NULL), t0)); /* src/hybrid.c:137 */
  return 0;
}
