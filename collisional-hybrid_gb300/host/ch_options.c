/*
 * ch_options.c -- ProcessOptions (src/parameters.c:28-562) for the GPU host.
 *
 * Option names, defaults and derived quantities follow the reference; the
 * SI constants Q, ME, KB (src/constants.h:5-8) become normalised units
 * e = kB = 1 with masses in ion-mass units (-ch_me sets the electron mass).
 */
#include "ch_options.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static const char* const RHS_NAMES[] = {"constant", "sinusoidal", "full", NULL};
static const char* const LHS_NAMES[] = {"identity", "laplacian", "full", NULL};
static const char* const DENSITY_NAMES[] = {"flat-sobol", "flat-reverse", "flat-normal", "uniform",
                                            "sinusoidal", "gaussian", NULL};
/* -ksp_type: cg, bcgs, or PETSc's default gmres, which has no GPU form
 * here and maps to CG for a symmetric operator, BiCGStab otherwise */
static const char* const KSP_NAMES[] = {"cg", "bcgs", "gmres", NULL};
static const char* const PC_NAMES[] = {"none", "jacobi", "mg", NULL};
static const char* const PREC_NAMES[] = {"fp64", "mixed", NULL};

typedef struct {
  int argc;
  char** argv;
} args_t;

static const char* find(const args_t* a, const char* name) {
  /* last occurrence wins, like the options database */
  const char* v = NULL;
  for (int i = 1; i < a->argc; ++i)
    if (!strcmp(a->argv[i], name)) v = (i + 1 < a->argc) ? a->argv[i + 1] : "";
  return v;
}

static int has(const args_t* a, const char* name) {
  for (int i = 1; i < a->argc; ++i)
    if (!strcmp(a->argv[i], name)) return 1;
  return 0;
}

static int get_real(const args_t* a, const char* name, double* out) {
  const char* v = find(a, name);
  if (!v || !*v) return 0;
  char* end = NULL;
  double d = strtod(v, &end);
  if (end == v) return -1;
  *out = d;
  return 1;
}

static int get_int(const args_t* a, const char* name, long long* out) {
  const char* v = find(a, name);
  if (!v || !*v) return 0;
  char* end = NULL;
  long long d = strtoll(v, &end, 10);
  if (end == v) return -1;
  *out = d;
  return 1;
}

static int get_enum(const args_t* a, const char* name, const char* const* names, int* out) {
  const char* v = find(a, name);
  if (!v) return 0;
  for (int i = 0; names[i]; ++i)
    if (!strcmp(v, names[i])) { *out = i; return 1; }
  return -1;
}

#define FAIL(...) do { if (err) snprintf(err, (size_t)err_len, __VA_ARGS__); return CH_ERR_ARG; } while (0)

ch_status ch_parse_options(int argc, char** argv, ch_params* p, ch_run_options* r, char* err, int err_len) {
  args_t a = {argc, argv};
  double d;
  long long n;
  int e;
  ch_params_default(p);
  memset(r, 0, sizeof(*r));
  r->Nt = 1;
  r->Np = -1;
  r->density_type = 0;
  double me = 1.0 / 1836.15267343; /* ME/MP */
  if (get_real(&a, "-ch_me", &d) > 0) me = d;

  /* grid (src/parameters.c:110-153, src/setup.c:8-12) */
  p->x0 = p->y0 = p->z0 = 0.0;
  p->x1 = p->y1 = p->z1 = 1.0;
  if (get_real(&a, "-x0", &d) > 0) p->x0 = d;
  if (get_real(&a, "-y0", &d) > 0) p->y0 = d;
  if (get_real(&a, "-z0", &d) > 0) p->z0 = d;
  if (get_real(&a, "-x1", &d) > 0) p->x1 = d;
  if (get_real(&a, "-y1", &d) > 0) p->y1 = d;
  if (get_real(&a, "-z1", &d) > 0) p->z1 = d;
  if (get_int(&a, "-Nx", &n) > 0) p->Nx = (int32_t)n;
  if (get_int(&a, "-Ny", &n) > 0) p->Ny = (int32_t)n;
  if (get_int(&a, "-Nz", &n) > 0) p->Nz = (int32_t)n;
  if ((e = get_enum(&a, "--rhs-type", RHS_NAMES, &p->rhs_type)) < 0) FAIL("bad --rhs-type");
  if ((e = get_enum(&a, "--lhs-type", LHS_NAMES, &p->lhs_type)) < 0) FAIL("bad --lhs-type");
  if ((e = get_enum(&a, "--density-type", DENSITY_NAMES, &r->density_type)) < 0) FAIL("bad --density-type");
  for (int s = 0; s < 6; ++s) {
    static const char* const bc[6] = {"--x0-bc", "--x1-bc", "--y0-bc", "--y1-bc", "--z0-bc", "--z1-bc"};
    const char* v = find(&a, bc[s]);
    if (v && strcmp(v, "periodic")) FAIL("%s %s: only periodic boundaries are supported (src/parameters.c:499-502)",
                                         bc[s], v);
  }
  if (get_int(&a, "-Np", &n) > 0) r->Np = n;
  /* species (src/parameters.c:197-345) */
  if (get_real(&a, "-qi", &d) > 0) p->qi = d;
  if (get_real(&a, "-mi", &d) > 0) p->mi = d;
  double nue = 1.0;
  if (get_real(&a, "-nue", &d) > 0) nue = d;
  if (get_real(&a, "-nui", &d) > 0) p->nui = d;
  if (get_real(&a, "-vi0", &d) > 0) p->vi0[0] = p->vi0[1] = p->vi0[2] = d;
  if (get_real(&a, "-vi0x", &d) > 0) p->vi0[0] = d;
  if (get_real(&a, "-vi0y", &d) > 0) p->vi0[1] = d;
  if (get_real(&a, "-vi0z", &d) > 0) p->vi0[2] = d;
  double viT[3] = {0, 0, 0}, veT[3] = {0, 0, 0}, Ti = 0.0, Te = 0.0;
  if (get_real(&a, "-viT", &d) > 0) viT[0] = viT[1] = viT[2] = d;
  if (get_real(&a, "-viTx", &d) > 0) viT[0] = d;
  if (get_real(&a, "-viTy", &d) > 0) viT[1] = d;
  if (get_real(&a, "-viTz", &d) > 0) viT[2] = d;
  if (get_real(&a, "-veT", &d) > 0) veT[0] = veT[1] = veT[2] = d;
  if (get_real(&a, "-veTx", &d) > 0) veT[0] = d;
  if (get_real(&a, "-veTy", &d) > 0) veT[1] = d;
  if (get_real(&a, "-veTz", &d) > 0) veT[2] = d;
  if (get_real(&a, "-Ti", &d) > 0) Ti = d;
  if (get_real(&a, "-Te", &d) > 0) Te = d;
  p->mn = p->mi;
  if (get_real(&a, "-mn", &d) > 0) p->mn = d;
  double Tn = -1.0;
  if (get_real(&a, "-Tn", &d) > 0) Tn = d;
  if (get_real(&a, "-vn0", &d) > 0) p->vn0[0] = p->vn0[1] = p->vn0[2] = d;
  if (get_real(&a, "-vn0x", &d) > 0) p->vn0[0] = d;
  if (get_real(&a, "-vn0y", &d) > 0) p->vn0[1] = d;
  if (get_real(&a, "-vn0z", &d) > 0) p->vn0[2] = d;
  if (get_real(&a, "-B0x", &d) > 0) p->B0[0] = d;
  if (get_real(&a, "-B0y", &d) > 0) p->B0[1] = d;
  if (get_real(&a, "-B0z", &d) > 0) p->B0[2] = d;
  if (get_real(&a, "-E0x", &d) > 0) p->E0[0] = d;
  if (get_real(&a, "-E0y", &d) > 0) p->E0[1] = d;
  if (get_real(&a, "-E0z", &d) > 0) p->E0[2] = d;
  if (get_int(&a, "-Nt", &n) > 0) r->Nt = (int32_t)n;
  p->dt = 1.0 / p->nui; /* src/parameters.c:417 */
  if (get_real(&a, "-dt", &d) > 0) p->dt = d;
  /* derived (src/parameters.c:507-556) */
  const double B[3] = {p->B0[0], p->B0[1], p->B0[2]};
  for (int c = 0; c < 3; ++c) p->kappa_e[c] = fabs(-1.0 * B[c] / me) / nue;
  if (viT[0] != 0.0 || viT[1] != 0.0 || viT[2] != 0.0) {
    double r2 = viT[0] * viT[0] + viT[1] * viT[1] + viT[2] * viT[2];
    Ti = 0.5 * p->mi * r2;
  } else {
    double t = sqrt(2.0 * Ti / p->mi) / 3.0;
    viT[0] = viT[1] = viT[2] = t;
  }
  if (veT[0] != 0.0 || veT[1] != 0.0 || veT[2] != 0.0) {
    double r2 = veT[0] * veT[0] + veT[1] * veT[1] + veT[2] * veT[2];
    Te = 0.5 * me * r2;
  }
  for (int c = 0; c < 3; ++c) p->viT[c] = viT[c];
  if (Tn == -1.0) Tn = Ti;
  p->vnT = p->mn > 0.0 ? sqrt(2.0 * Tn / p->mn) : 0.0;
  if (get_real(&a, "-ch_vnT", &d) > 0) p->vnT = d;
  p->cth = 1.0 * Te;   /* gamma = 1 (src/parameters.c:552), kB/e = 1 */
  p->cG = me * nue;    /* me nue / e */
  if (get_real(&a, "-ch_cth", &d) > 0) p->cth = d;
  if (get_real(&a, "-ch_cG", &d) > 0) p->cG = d;
  if (get_real(&a, "-ch_kappa_ex", &d) > 0) p->kappa_e[0] = d;
  if (get_real(&a, "-ch_kappa_ey", &d) > 0) p->kappa_e[1] = d;
  if (get_real(&a, "-ch_kappa_ez", &d) > 0) p->kappa_e[2] = d;
  /* solver */
  int kt = 2;  /* absent: PETSc's default, gmres */
  if (get_enum(&a, "-ksp_type", KSP_NAMES, &kt) < 0) FAIL("-ksp_type: cg, bcgs or gmres");
  if (kt == 2) {
    const int sym = p->lhs_type != CH_LHS_FULL ||
                    (p->kappa_e[0] == 0.0 && p->kappa_e[1] == 0.0 && p->kappa_e[2] == 0.0);
    kt = sym ? CH_KSP_CG : CH_KSP_BCGS;
  }
  p->ksp_type = kt;
  if (get_enum(&a, "-ch_pc", PC_NAMES, &p->pc_type) < 0) FAIL("-ch_pc: none, jacobi or mg");
  if (get_real(&a, "-ksp_rtol", &d) > 0) p->ksp_rtol = d;
  if (get_real(&a, "-ksp_atol", &d) > 0) p->ksp_atol = d;
  if (get_int(&a, "-ksp_max_it", &n) > 0) p->ksp_max_it = (int32_t)n;
  if (get_enum(&a, "-ch_precision", PREC_NAMES, &p->precision) < 0) FAIL("-ch_precision: fp64 or mixed");
  /* -ch_ extensions */
  if (get_int(&a, "-ch_seed", &n) > 0) p->seed = (uint64_t)n;
  if (get_int(&a, "-ch_faithful", &n) > 0) p->faithful = (uint32_t)n;
  if (has(&a, "-ch_push_E0")) p->push_E0 = 1;
  if (get_int(&a, "-ch_sort_period", &n) > 0) p->sort_period = (int32_t)n;
  if (get_real(&a, "-ch_nn_sigma", &d) > 0) {
    p->nn_profile = CH_NN_GAUSSIAN_X;
    p->nn_sigma = d;
    p->nn_center = 0.5 * (p->x0 + p->x1);
    p->nn_floor = 0.1;
    if (get_real(&a, "-ch_nn_floor", &d) > 0) p->nn_floor = d;
  }
  r->use_modes = 0;
  if (get_real(&a, "-ch_amp1", &d) > 0) { r->amp[0] = d; r->use_modes = 1; }
  if (get_real(&a, "-ch_amp2", &d) > 0) { r->amp[1] = d; r->use_modes = 1; }
  if (get_real(&a, "-ch_amp3", &d) > 0) { r->amp[2] = d; r->use_modes = 1; }
  if (get_real(&a, "-ch_phase1", &d) > 0) { r->phase[0] = d; r->use_modes = 1; }
  if (get_real(&a, "-ch_phase2", &d) > 0) { r->phase[1] = d; r->use_modes = 1; }
  if (get_real(&a, "-ch_phase3", &d) > 0) { r->phase[2] = d; r->use_modes = 1; }
  r->random_phases = has(&a, "-ch_random_phases");
  if (r->random_phases) r->use_modes = 1;
  r->verbose = has(&a, "-ch_verbose");
  if (r->Np < 0) r->Np = (int64_t)p->Nx * p->Ny * p->Nz; /* src/setup.c:44-46 */
  (void)e;
  return CH_OK;
}
