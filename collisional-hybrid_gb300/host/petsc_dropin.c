/*
 * petsc_dropin.c -- GPU replacements of the reference's per-step entry
 * points for its own PETSc host (src/hybrid.c).  Link this file in place of
 * the hot-path functions of src/particles.c and src/potential.c:
 *
 *   UpdateVelocities(KSP, Context*)     src/particles.h:19  (src/particles.c:628)
 *   UpdatePositions(Context*)           src/particles.h:21  (src/particles.c:647)
 *   CollectVlasovQuantities(Context*)   src/particles.h:11  (src/particles.c:136)
 *   ComputePotential(KSP, Context*)     src/potential.h:7   (src/potential.c:6)
 *
 * Build against PETSc and the reference's headers:
 *   cc -DCH_WITH_PETSC -I$PETSC_DIR/include -I<reference>/src -I<this repo>/include \
 *      -c petsc_dropin.c
 * and link libchybrid.so.  One MPI rank drives one GPU (the replacement
 * rejects more ranks: the GPU path does not decompose the grid).
 *
 * Data flow: the DMSwarm "position"/"velocity" fields (RealVector AoS) are
 * copied to the device at the start of each particle call and back at its
 * end, so every host routine between calls sees current ions; the vlasov
 * global Vec (GridNode, dof 4) receives the moments; ctx->phi receives the
 * potential.  Reference option names map to ch_params through the Context
 * that ProcessOptions filled (src/parameters.c:28-562).
 */
#ifdef CH_WITH_PETSC

#include <petsc.h>
#include <string.h>

#include "chybrid.h"
#include "hybrid.h"

static ch_ctx* g_gpu = NULL;
static long long g_step = 0;

/* SI constants of the reference (src/constants.h) are folded into the
 * electron coefficients exactly as ComputeFullRHS forms them (src/rhs.c:190-191). */
static void params_from_context(const Context* ctx, ch_params* p) {
  ch_params_default(p);
  p->Nx = ctx->grid.N.x;
  p->Ny = ctx->grid.N.y;
  p->Nz = ctx->grid.N.z;
  p->x0 = ctx->grid.p0.x; p->y0 = ctx->grid.p0.y; p->z0 = ctx->grid.p0.z;
  p->x1 = ctx->grid.p1.x; p->y1 = ctx->grid.p1.y; p->z1 = ctx->grid.p1.z;
  p->qi = ctx->ions.q;
  p->mi = ctx->ions.m;
  p->nui = ctx->ions.nu;
  p->dt = ctx->dt;
  p->vi0[0] = ctx->ions.v0.x; p->vi0[1] = ctx->ions.v0.y; p->vi0[2] = ctx->ions.v0.z;
  p->viT[0] = ctx->ions.vT.x; p->viT[1] = ctx->ions.vT.y; p->viT[2] = ctx->ions.vT.z;
  p->mn = ctx->neutrals.m;
  p->vnT = ctx->neutrals.vT;
  p->vn0[0] = ctx->neutrals.v0.x; p->vn0[1] = ctx->neutrals.v0.y; p->vn0[2] = ctx->neutrals.v0.z;
  p->B0[0] = ctx->plasma.B0.x; p->B0[1] = ctx->plasma.B0.y; p->B0[2] = ctx->plasma.B0.z;
  p->E0[0] = ctx->plasma.E0.x; p->E0[1] = ctx->plasma.E0.y; p->E0[2] = ctx->plasma.E0.z;
  p->kappa_e[0] = ctx->electrons.kappa.x;
  p->kappa_e[1] = ctx->electrons.kappa.y;
  p->kappa_e[2] = ctx->electrons.kappa.z;
  p->cth = ctx->electrons.gamma * KB * ctx->electrons.T / Q;
  p->cG = ctx->electrons.m * ctx->electrons.nu / Q;
  p->lhs_type = (int32_t)ctx->lhsType;
  p->rhs_type = (int32_t)ctx->rhsType;
  p->seed = (uint64_t)(ctx->seed < 0 ? -ctx->seed : ctx->seed);
}

#define CH_PETSC(call)                                                                           \
  do {                                                                                           \
    ch_status rc_ = (call);                                                                      \
    if (rc_ == CH_ERR_COLLISION_LIMIT) SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_SIG, "%s", ch_last_error()); \
    if (rc_ != CH_OK) SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_LIB, "%s", ch_last_error());           \
  } while (0)

static PetscErrorCode ensure_gpu(Context* ctx) {
  PetscMPIInt size;
  PetscFunctionBeginUser;
  if (g_gpu) PetscFunctionReturn(PETSC_SUCCESS);
  PetscCallMPI(MPI_Comm_size(PETSC_COMM_WORLD, &size));
  if (size != 1) SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_SUP, "the GPU hot path runs on one rank (got %d)", size);
  ch_params p;
  params_from_context(ctx, &p);
  CH_PETSC(ch_create(&p, -1, &g_gpu));
  PetscFunctionReturn(PETSC_SUCCESS);
}

/* DMSwarm fields -> device */
static PetscErrorCode push_ions(Context* ctx) {
  PetscInt np;
  RealVector *pos, *vel;
  PetscFunctionBeginUser;
  PetscCall(DMSwarmGetLocalSize(ctx->ionsDM, &np));
  PetscCall(DMSwarmGetField(ctx->ionsDM, "position", NULL, NULL, (void**)&pos));
  PetscCall(DMSwarmGetField(ctx->ionsDM, "velocity", NULL, NULL, (void**)&vel));
  ch_status rc = ch_particles_upload(g_gpu, (const ch_real_vector*)pos, (const ch_real_vector*)vel, np);
  PetscCall(DMSwarmRestoreField(ctx->ionsDM, "velocity", NULL, NULL, (void**)&vel));
  PetscCall(DMSwarmRestoreField(ctx->ionsDM, "position", NULL, NULL, (void**)&pos));
  CH_PETSC(rc);
  PetscFunctionReturn(PETSC_SUCCESS);
}

/* device -> DMSwarm fields */
static PetscErrorCode pull_ions(Context* ctx) {
  RealVector *pos, *vel;
  PetscFunctionBeginUser;
  PetscCall(DMSwarmGetField(ctx->ionsDM, "position", NULL, NULL, (void**)&pos));
  PetscCall(DMSwarmGetField(ctx->ionsDM, "velocity", NULL, NULL, (void**)&vel));
  ch_status rc = ch_particles_download(g_gpu, (ch_real_vector*)pos, (ch_real_vector*)vel);
  PetscCall(DMSwarmRestoreField(ctx->ionsDM, "velocity", NULL, NULL, (void**)&vel));
  PetscCall(DMSwarmRestoreField(ctx->ionsDM, "position", NULL, NULL, (void**)&pos));
  CH_PETSC(rc);
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode UpdateVelocities(KSP ksp, Context* ctx) {
  PetscFunctionBeginUser;
  (void)ksp;  /* phi stays on the device from the last ComputePotential */
  PetscCall(ensure_gpu(ctx));
  PetscCall(push_ions(ctx));
  ch_step_info info;
  CH_PETSC(ch_update_velocities(g_gpu, g_step, &info));
  PetscCall(pull_ions(ctx));
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode UpdatePositions(Context* ctx) {
  PetscFunctionBeginUser;
  PetscCall(ensure_gpu(ctx));
  PetscCall(push_ions(ctx));
  CH_PETSC(ch_update_positions(g_gpu));
  PetscCall(pull_ions(ctx));
  PetscCall(DMSwarmMigrate(ctx->ionsDM, PETSC_TRUE)); /* src/particles.c:714 */
  g_step++;
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode CollectVlasovQuantities(Context* ctx) {
  PetscScalar* a;
  PetscFunctionBeginUser;
  PetscCall(ensure_gpu(ctx));
  PetscCall(push_ions(ctx));
  PetscCall(VecGetArray(ctx->vlasov, &a)); /* GridNode, natural order on one rank */
  ch_status rc = ch_collect_moments(g_gpu, (ch_grid_node*)a, NULL);
  PetscCall(VecRestoreArray(ctx->vlasov, &a));
  CH_PETSC(rc);
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode ComputePotential(KSP ksp, Context* ctx) {
  PetscScalar* a;
  DM dm;
  PetscFunctionBeginUser;
  PetscCall(ensure_gpu(ctx));
  /* the host may have replaced the moments (LoadVlasovQuantities, src/fileio.c:6-70) */
  PetscCall(VecGetArray(ctx->vlasov, &a));
  ch_status rc = ch_set_moments(g_gpu, (const ch_grid_node*)a);
  PetscCall(VecRestoreArray(ctx->vlasov, &a));
  CH_PETSC(rc);
  if (!ctx->phi) {
    PetscCall(KSPGetDM(ksp, &dm));
    PetscCall(DMCreateGlobalVector(dm, &ctx->phi));
  }
  PetscCall(VecGetArray(ctx->phi, &a));
  ch_solve_info info;
  rc = ch_compute_potential(g_gpu, a, &info);
  PetscCall(VecRestoreArray(ctx->phi, &a));
  CH_PETSC(rc);
  PetscFunctionReturn(PETSC_SUCCESS);
}

#endif /* CH_WITH_PETSC */
