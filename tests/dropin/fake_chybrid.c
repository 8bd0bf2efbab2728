/* A recording stand-in of the C ABI (include/chybrid.h) for the drop-in's
 * CPU test: it keeps the parameters, solver settings and transfer counts
 * that petsc_dropin.c passes down, and computes nothing.  TEST ONLY. */
#include <stdio.h>
#include <string.h>

#include "chybrid.h"

static ch_params g_created;
static int g_ncreate = 0, g_uploads = 0, g_downloads = 0, g_solves = 0, g_set_solver = 0;
static int32_t g_ksp = -1, g_pc = -1, g_maxit = -1;
static double g_rtol = -1.0, g_atol = -1.0;
static int g_dummy;

const char* ch_last_error(void) { return "recording stand-in"; }
ch_status ch_params_default(ch_params* p) {
  memset(p, 0, sizeof(*p));
  p->ksp_type = CH_KSP_CG;
  p->pc_type = CH_PC_JACOBI;
  p->ksp_rtol = 1e-5;
  p->ksp_atol = 1e-50;
  p->ksp_max_it = 10000;
  p->sort_period = 8;
  return CH_OK;
}
ch_status ch_create(const ch_params* p, int32_t device, ch_ctx** out) {
  (void)device;
  g_created = *p;
  ++g_ncreate;
  *out = (ch_ctx*)&g_dummy;
  return CH_OK;
}
ch_status ch_particles_upload(ch_ctx* c, const ch_real_vector* pos, const ch_real_vector* vel, int64_t np) {
  (void)c; (void)pos; (void)vel; (void)np;
  ++g_uploads;
  return CH_OK;
}
ch_status ch_particles_download(ch_ctx* c, ch_real_vector* pos, ch_real_vector* vel) {
  (void)c; (void)pos; (void)vel;
  ++g_downloads;
  return CH_OK;
}
ch_status ch_update_velocities(ch_ctx* c, int64_t step, ch_step_info* info) {
  (void)c; (void)step;
  if (info) memset(info, 0, sizeof(*info));
  return CH_OK;
}
ch_status ch_update_positions(ch_ctx* c) { (void)c; return CH_OK; }
ch_status ch_collect_moments(ch_ctx* c, ch_grid_node* out, ch_step_info* info) {
  (void)c; (void)out; (void)info;
  return CH_OK;
}
ch_status ch_set_moments(ch_ctx* c, const ch_grid_node* in) { (void)c; (void)in; return CH_OK; }
ch_status ch_set_solver(ch_ctx* c, int32_t ksp_type, int32_t pc_type, double rtol, double atol, int32_t max_it) {
  (void)c;
  ++g_set_solver;
  g_ksp = ksp_type; g_pc = pc_type; g_rtol = rtol; g_atol = atol; g_maxit = max_it;
  return CH_OK;
}
ch_status ch_compute_potential(ch_ctx* c, double* phi, ch_solve_info* info) {
  (void)c; (void)phi;
  if (info) memset(info, 0, sizeof(*info));
  ++g_solves;
  return CH_OK;
}

void fake_report(FILE* f) {
  const ch_params* p = &g_created;
  fprintf(f, "creates %d\nuploads %d\ndownloads %d\nsolves %d\nset_solver %d\n", g_ncreate, g_uploads, g_downloads,
          g_solves, g_set_solver);
  fprintf(f, "precision %d\ncreate_pc %d\nsort_period %d\nfaithful %u\n", p->precision, p->pc_type, p->sort_period,
          p->faithful);
  fprintf(f, "kappa %.17g %.17g %.17g\n", p->kappa_e[0], p->kappa_e[1], p->kappa_e[2]);
  fprintf(f, "grid %d %d %d\nnui %.17g\ndt %.17g\n", p->Nx, p->Ny, p->Nz, p->nui, p->dt);
  fprintf(f, "ksp %d\npc %d\nrtol %.17g\natol %.17g\nmaxit %d\n", g_ksp, g_pc, g_rtol, g_atol, g_maxit);
}
