/*
 * ch_options.h -- the reference's command-line options mapped to ch_params.
 *
 * ch_parse_options reads the option names of ProcessOptions
 * (src/parameters.c:28-562) from argv and derives the same quantities
 * (thermal speeds from temperatures, electron magnetisation, dt = 1/nu),
 * in normalised units (e = kB = 1, ion mass unit).  Options the reference
 * does not have carry a -ch_ prefix.
 */
#ifndef CH_OPTIONS_H
#define CH_OPTIONS_H

#include "chybrid.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ch_run_options {
  int32_t Nt;            /* -Nt (src/parameters.c:406-411)                    */
  int64_t Np;            /* -Np, -1 = one ion per cell (src/setup.c:44-46)    */
  int32_t density_type;  /* --density-type index in DensityTypes               */
  double amp[3];         /* -ch_amp1..3: density perturbation amplitudes       */
  double phase[3];       /* -ch_phase1..3 (-ch_random_phases draws them)       */
  int32_t random_phases; /* -ch_random_phases                                  */
  int32_t verbose;       /* -ch_verbose                                        */
  int32_t use_modes;     /* a -ch_amp / -ch_phase option was given: load by the
                            inverse CDF of the density modes (ch_particles_load)
                            instead of the --density-type placement          */
} ch_run_options;

/* Parses argv (unknown options are ignored, like PETSc's options database)
 * into *p and *r.  Returns CH_OK or CH_ERR_ARG with ch_last_error-style text
 * in err (err_len bytes). */
ch_status ch_parse_options(int argc, char** argv, ch_params* p, ch_run_options* r, char* err, int err_len);

#ifdef __cplusplus
}
#endif
#endif
