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
 * Data flow: the ions stay on the device between the particle calls of a
 * step.  UpdateVelocities uploads the DMSwarm "position"/"velocity" fields
 * (RealVector AoS) only when the host holds newer ions than the device: on
 * the first call, when the fields' base address or local size changed (a
 * DMSwarm reallocation or migration), or after the host called
 * HybridGPUIonsChanged().  UpdatePositions downloads the step's ions once,
 * so the DMSwarm holds them for DMSwarmMigrate and any host routine after
 * it; CollectVlasovQuantities then deposits from the device copy.  One
 * upload and one download per step instead of one of each per call.  The
 * vlasov global Vec (GridNode, dof 4) receives the moments; ctx->phi
 * receives the potential.
 *
 * Options: the Context fields that ProcessOptions filled
 * (src/parameters.c:28-562) give the physics; the KSP gives the solver as
 * KSPSetFromOptions set it (src/hybrid.c:75): -ksp_type cg | bcgs (PETSc's
 * default gmres, which has no GPU form here, maps to CG for a symmetric
 * operator and to BiCGStab otherwise), -ksp_rtol, -ksp_atol, -ksp_max_it;
 * the options database gives -ch_precision fp64|mixed, -ch_pc
 * none|jacobi|mg, -ch_sort_period n and -ch_faithful bits.
 */
#ifdef CH_WITH_PETSC

#include <petsc.h>
#include <string.h>

#include "chybrid.h"
#include "hybrid.h"

static ch_ctx* g_gpu = NULL;
static long long g_step = 0;
/* Which copy of the ions is current (see the data flow above). */
static const void* g_pos_seen = NULL;
static const void* g_vel_seen = NULL;
static PetscInt g_np_seen = -1;
static int g_host_newer = 1;
static int g_device_newer = 0;

#define CH_PETSC(call)                                                                           \
  do {                                                                                           \
    ch_status rc_ = (call);                                                                      \
    if (rc_ == CH_ERR_COLLISION_LIMIT) SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_SIG, "%s", ch_last_error()); \
    if (rc_ != CH_OK) SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_LIB, "%s", ch_last_error());           \
  } while (0)

/* -name value from the options database, as an index into names[] (-1 when
 * the option is absent; -2 when its value is not one of names[]). */
static int option_enum(const char* name, const char* const* names, int n) {
  char buf[64];
  PetscBool set = PETSC_FALSE;
  if (PetscOptionsGetString(NULL, NULL, name, buf, sizeof buf, &set) || !set) return -1;
  for (int i = 0; i < n; ++i)
    if (!strcmp(buf, names[i])) return i;
  return -2;
}

/* SI constants of the reference (src/constants.h) are folded into the
 * electron coefficients exactly as ComputeFullRHS forms them (src/rhs.c:190-191). */
static PetscErrorCode params_from_context(const Context* ctx, ch_params* p) {
  static const char* const prec_names[] = {"fp64", "mixed"};
  static const char* const pc_names[] = {"none", "jacobi", "mg"};
  PetscFunctionBeginUser;
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
  int e = option_enum("-ch_precision", prec_names, 2);
  if (e == -2) SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_ARG_OUTOFRANGE, "-ch_precision: fp64 or mixed");
  if (e >= 0) p->precision = e;
  e = option_enum("-ch_pc", pc_names, 3);
  if (e == -2) SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_ARG_OUTOFRANGE, "-ch_pc: none, jacobi or mg");
  if (e >= 0) p->pc_type = e;
  PetscInt iv;
  PetscBool set = PETSC_FALSE;
  PetscCall(PetscOptionsGetInt(NULL, NULL, "-ch_sort_period", &iv, &set));
  if (set) p->sort_period = (int32_t)iv;
  set = PETSC_FALSE;
  PetscCall(PetscOptionsGetInt(NULL, NULL, "-ch_faithful", &iv, &set));
  if (set) p->faithful = (uint32_t)iv;
  PetscFunctionReturn(PETSC_SUCCESS);
}

/* The KSP's method and tolerances, as KSPSetFromOptions left them. */
static PetscErrorCode solver_from_ksp(KSP ksp, const Context* ctx) {
  PetscReal rtol, atol, dtol;
  PetscInt maxits;
  KSPType type;
  ch_params p;
  PetscFunctionBeginUser;
  PetscCall(KSPGetTolerances(ksp, &rtol, &atol, &dtol, &maxits));
  PetscCall(KSPGetType(ksp, &type));
  PetscCall(params_from_context(ctx, &p));
  const int symmetric = p.lhs_type != CH_LHS_FULL ||
                        (p.kappa_e[0] == 0.0 && p.kappa_e[1] == 0.0 && p.kappa_e[2] == 0.0);
  int32_t kt;
  if (type && !strcmp(type, "cg"))
    kt = CH_KSP_CG;  /* the library refuses it for a non-symmetric operator */
  else if (type && !strcmp(type, "bcgs"))
    kt = CH_KSP_BCGS;
  else if (!type || !strcmp(type, "gmres") || !strcmp(type, "fgmres") || !strcmp(type, "lgmres"))
    kt = symmetric ? CH_KSP_CG : CH_KSP_BCGS;
  else
    SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_SUP, "-ksp_type %s: the GPU solve offers cg and bcgs", type);
  CH_PETSC(ch_set_solver(g_gpu, kt, p.pc_type, rtol, atol, (int32_t)maxits));
  PetscFunctionReturn(PETSC_SUCCESS);
}

static PetscErrorCode ensure_gpu(Context* ctx) {
  PetscMPIInt size;
  PetscFunctionBeginUser;
  if (g_gpu) PetscFunctionReturn(PETSC_SUCCESS);
  PetscCallMPI(MPI_Comm_size(PETSC_COMM_WORLD, &size));
  if (size != 1) SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_SUP, "the GPU hot path runs on one rank (got %d)", size);
  ch_params p;
  PetscCall(params_from_context(ctx, &p));
  CH_PETSC(ch_create(&p, -1, &g_gpu));
  g_host_newer = 1;
  g_device_newer = 0;
  PetscFunctionReturn(PETSC_SUCCESS);
}

/* DMSwarm fields -> device, when the host holds the newer ions */
static PetscErrorCode sync_to_device(Context* ctx) {
  PetscInt np;
  RealVector *pos, *vel;
  PetscFunctionBeginUser;
  PetscCall(DMSwarmGetLocalSize(ctx->ionsDM, &np));
  PetscCall(DMSwarmGetField(ctx->ionsDM, "position", NULL, NULL, (void**)&pos));
  PetscCall(DMSwarmGetField(ctx->ionsDM, "velocity", NULL, NULL, (void**)&vel));
  ch_status rc = CH_OK;
  const int moved = (const void*)pos != g_pos_seen || (const void*)vel != g_vel_seen || np != g_np_seen;
  if (g_host_newer || moved) {
    if (g_device_newer && !g_host_newer && moved)
      rc = CH_ERR_STATE;  /* the fields moved while the device held newer ions */
    else
      rc = ch_particles_upload(g_gpu, (const ch_real_vector*)pos, (const ch_real_vector*)vel, np);
    if (rc == CH_OK) {
      g_pos_seen = pos;
      g_vel_seen = vel;
      g_np_seen = np;
      g_host_newer = 0;
      g_device_newer = 0;
    }
  }
  PetscCall(DMSwarmRestoreField(ctx->ionsDM, "velocity", NULL, NULL, (void**)&vel));
  PetscCall(DMSwarmRestoreField(ctx->ionsDM, "position", NULL, NULL, (void**)&pos));
  if (rc == CH_ERR_STATE)
    SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_ORDER, "the DMSwarm fields changed while the device held newer ions");
  CH_PETSC(rc);
  PetscFunctionReturn(PETSC_SUCCESS);
}

/* device -> DMSwarm fields, when the device holds the newer ions */
static PetscErrorCode sync_to_host(Context* ctx) {
  RealVector *pos, *vel;
  PetscFunctionBeginUser;
  if (!g_device_newer) PetscFunctionReturn(PETSC_SUCCESS);
  PetscCall(DMSwarmGetField(ctx->ionsDM, "position", NULL, NULL, (void**)&pos));
  PetscCall(DMSwarmGetField(ctx->ionsDM, "velocity", NULL, NULL, (void**)&vel));
  ch_status rc = ch_particles_download(g_gpu, (ch_real_vector*)pos, (ch_real_vector*)vel);
  if (rc == CH_OK) {
    g_pos_seen = pos;
    g_vel_seen = vel;
    g_device_newer = 0;
  }
  PetscCall(DMSwarmRestoreField(ctx->ionsDM, "velocity", NULL, NULL, (void**)&vel));
  PetscCall(DMSwarmRestoreField(ctx->ionsDM, "position", NULL, NULL, (void**)&pos));
  CH_PETSC(rc);
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode HybridGPUIonsChanged(void) {
  PetscFunctionBeginUser;
  if (g_device_newer)
    SETERRQ(PETSC_COMM_WORLD, PETSC_ERR_ORDER, "the device holds newer ions: call HybridGPUSyncIons first");
  g_host_newer = 1;
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode HybridGPUSyncIons(Context* ctx) {
  PetscFunctionBeginUser;
  if (g_gpu) PetscCall(sync_to_host(ctx));
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode UpdateVelocities(KSP ksp, Context* ctx) {
  PetscFunctionBeginUser;
  (void)ksp;  /* phi stays on the device from the last ComputePotential */
  PetscCall(ensure_gpu(ctx));
  PetscCall(sync_to_device(ctx));
  ch_step_info info;
  CH_PETSC(ch_update_velocities(g_gpu, g_step, &info));
  g_device_newer = 1;
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode UpdatePositions(Context* ctx) {
  PetscFunctionBeginUser;
  PetscCall(ensure_gpu(ctx));
  PetscCall(sync_to_device(ctx));
  CH_PETSC(ch_update_positions(g_gpu));
  g_device_newer = 1;
  PetscCall(sync_to_host(ctx));                       /* the step's ions, once */
  PetscCall(DMSwarmMigrate(ctx->ionsDM, PETSC_TRUE)); /* src/particles.c:714 */
  g_step++;
  PetscFunctionReturn(PETSC_SUCCESS);
}

PetscErrorCode CollectVlasovQuantities(Context* ctx) {
  PetscScalar* a;
  PetscFunctionBeginUser;
  PetscCall(ensure_gpu(ctx));
  PetscCall(sync_to_device(ctx));
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
  PetscCall(solver_from_ksp(ksp, ctx));
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
