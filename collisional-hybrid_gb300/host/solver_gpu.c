/*
 * solver_gpu.c -- the reference's stand-alone potential solver
 * (src/solver.c:18-102) on the GPU through the C ABI, without PETSc or
 * HDF5: same option names, same order of work.
 *
 *   ProcessOptions                 -> ch_parse_options (grid, physics, -ksp_*)
 *   LoadVlasovQuantities           -> --input <file>: the density ("density-kji")
 *     (src/fileio.c:6-70)             as raw little-endian FP64 in DMDA natural
 *                                     order, Nx*Ny*Nz values (the layout that
 *                                     ch_output writes); each flux is
 *                                     --flux-scale (or --x/y/z-flux-scale,
 *                                     default 1) times the density, as the
 *                                     reference forms them
 *   ComputePotential               -> ch_set_moments + ch_compute_potential,
 *                                     from phi = 0 (ComputeInitialPhi)
 *   OutputHDF5("")                 -> ch_output_open(--output, default
 *                                     "results") + ch_output("")
 *
 * Without --input the reference falls back to the sinusoidal RHS
 * (src/fileio.c:20-24); its density vector then holds zeros, which leave the
 * full operator without coefficients, so here the density is 1 instead.
 * -ch_repeat k solves k times, each from phi = 0, and prints the mean solve
 * time and solves/s (the solve micro-benchmark).
 *
 *   solver_gpu -Nx 128 -Ny 128 -Nz 128 -x1 128 -y1 128 -z1 128 --input n.f64 \
 *              -ksp_rtol 1e-10 -ch_precision mixed -ch_pc mg -ch_repeat 20
 *
 * Exit status 0 on success, 1 on a reported error (message on stderr).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "ch_options.h"

static const char* arg_str(int argc, char** argv, const char* name) {
  for (int i = 1; i + 1 < argc; ++i)
    if (!strcmp(argv[i], name)) return argv[i + 1];
  return NULL;
}

static double arg_real(int argc, char** argv, const char* name, double dflt) {
  const char* v = arg_str(argc, argv, name);
  return v ? strtod(v, NULL) : dflt;
}

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

int main(int argc, char** argv) {
  ch_params p;
  ch_run_options r;
  char err[256] = "";
  ch_ctx* ctx = NULL;
  ch_grid_node* nodes = NULL;
  double* phi = NULL;
  int rc = 1;
  if (ch_parse_options(argc, argv, &p, &r, err, (int)sizeof(err)) != CH_OK) {
    fprintf(stderr, "options: %s\n", err);
    return 1;
  }
  const char* input = arg_str(argc, argv, "--input");
  const char* output = arg_str(argc, argv, "--output");
  const int repeat = (int)arg_real(argc, argv, "-ch_repeat", 1.0);
  const double fs = arg_real(argc, argv, "--flux-scale", 1.0);  /* src/parameters.c:419-439 */
  const double fsc[3] = {arg_real(argc, argv, "--x-flux-scale", fs), arg_real(argc, argv, "--y-flux-scale", fs),
                         arg_real(argc, argv, "--z-flux-scale", fs)};
  p.mn = 0.0;  /* a solve has no ions: no neutrals, no collision setup */
  const int64_t N = (int64_t)p.Nx * p.Ny * p.Nz;
  nodes = (ch_grid_node*)calloc((size_t)N, sizeof(ch_grid_node));
  phi = (double*)calloc((size_t)N, sizeof(double));
  if (!nodes || !phi || repeat < 1) {
    fprintf(stderr, "bad -ch_repeat or out of memory\n");
    goto done;
  }
  if (input) {
    FILE* f = fopen(input, "rb");
    if (!f) {
      fprintf(stderr, "--input %s: cannot open\n", input);
      goto done;
    }
    double* n = (double*)malloc(sizeof(double) * (size_t)N);
    const size_t got = n ? fread(n, sizeof(double), (size_t)N, f) : 0;
    fclose(f);
    if (got != (size_t)N) {
      fprintf(stderr, "--input %s: expected %lld FP64 values, read %zu\n", input, (long long)N, got);
      free(n);
      goto done;
    }
    for (int64_t c = 0; c < N; ++c) {
      nodes[c].n = n[c];
      for (int d = 0; d < 3; ++d) nodes[c].flux[d] = fsc[d] * n[c];
    }
    free(n);
  } else {
    printf("Warning: no --input; using the sinusoidal RHS on a unit density.\n");
    p.rhs_type = CH_RHS_SINUSOIDAL;
    for (int64_t c = 0; c < N; ++c) nodes[c].n = 1.0;
  }
  ch_status s = ch_create(&p, -1, &ctx);
  if (s == CH_OK) s = ch_set_moments(ctx, nodes);
  ch_solve_info info;
  memset(&info, 0, sizeof(info));
  double best = 1e30, total = 0.0;
  int its_sum = 0;
  for (int k = 0; k < repeat && s == CH_OK; ++k) {
    memset(phi, 0, sizeof(double) * (size_t)N);
    s = ch_set_phi(ctx, phi);  /* ComputeInitialPhi: phi = 0 (src/potential.c:20-30) */
    if (s != CH_OK) break;
    const double t0 = now_s();
    s = ch_compute_potential(ctx, k + 1 == repeat ? phi : NULL, &info);
    const double dt = now_s() - t0;
    total += dt;
    if (dt < best) best = dt;
    its_sum += info.iterations;
  }
  if (s == CH_OK) {  /* OutputHDF5("", &ctx) (src/solver.c:73) */
    s = ch_output_open(ctx, output ? output : "results");
    if (s == CH_OK) s = ch_output(ctx, "");
    if (s == CH_OK) s = ch_output_wait(ctx, NULL);
  }
  if (s != CH_OK) {
    fprintf(stderr, "solve failed (%d): %s\n", (int)s, ch_last_error());
    goto done;
  }
  printf("KSP iterations %d  refinements %d  |r|/|b| %.3e  (rtol %.1e)\n", info.iterations, info.refinements,
         info.bnorm > 0 ? info.rnorm / info.bnorm : 0.0, p.ksp_rtol);
  printf("solves %d  mean %.3f ms  best %.3f ms  solves/s %.1f  iterations/solve %.1f\n", repeat,
         1e3 * total / repeat, 1e3 * best, repeat / total, (double)its_sum / repeat);
  rc = 0;
done:
  if (ctx) ch_destroy(ctx);
  free(nodes);
  free(phi);
  return rc;
}
