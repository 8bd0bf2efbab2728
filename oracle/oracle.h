/*
 * oracle.h -- FP64 CPU restatement of the hybrid-PIC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * GPU path and the timed CPU baseline; the product never links it.
 *
 * Each function names the reference file:line it restates.  Where the
 * reference's as-written code is defective the default is the corrected
 * algorithm and the CH_FAITHFUL_Dn bit selects the as-written behaviour.
 * Parity pins: golden vectors produced by the reference's own sources
 * (compiled here against a PETSc stand-in), analytic identities, and
 * Philox4x32-10 known-answer vectors.
 */
#ifndef CH_ORACLE_H
#define CH_ORACLE_H

#include <stdint.h>
#include "../include/chybrid.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Particle state in the FP64 plain form: SoA, index = ion id. */
typedef struct orc_particles {
  int64_t np;
  double *x, *y, *z, *vx, *vy, *vz;
} orc_particles;

/* Seeded loader shared with the GPU loader (same Philox counters). */
int orc_load(const ch_params* p, const ch_loader* L, orc_particles* P);
/* the reference's --density-type placements 0 (flat-sobol), 3 (uniform),
 * 4 (sinusoidal rejection), as ch_particles_load_placed places them */
int orc_load_placed(const ch_params* p, const ch_loader* L, int type, orc_particles* P);

/* DifferenceVector (src/vectors.c:12-138): numerators of the central
 * differences of phi interpolated to the cell-unit point (X, Y, Z).
 * CH_FAITHFUL_D3 / D4 select the as-written interpolation / boundary rule. */
void orc_difference_vector(const ch_params* p, const double* phi,
                           double X, double Y, double Z, uint32_t faithful, double f[3]);

/* Node electric field E = -grad phi by periodic central differences. */
void orc_node_efield(const ch_params* p, const double* phi, double* Ex, double* Ey, double* Ez);

/* Mean relative speed E|w - V| of a fixed velocity against a Maxwellian of
 * per-component std sigma, w = |v - vn0|. */
double orc_gmean(double w, double sigma);

/* Collision count of the reference (src/particles.c:510-519). */
int64_t orc_collision_count(const ch_params* p, int64_t np);

/* Sum over ions of orc_gmean(|v - vn0|, vnT): the normaliser of the
 * per-ion collision probability. */
double orc_sbar(const ch_params* p, const orc_particles* P);

/* UpdateVelocities (src/particles.c:628-643): Boris push (:348-464) with E
 * gathered at each ion, then the per-ion Philox collision if mn > 0.
 * sbar: the normaliser for this step; returns the next step's in *sbar_next. */
typedef struct orc_counters {
  int64_t Nc, collisions, refused;
  double expected;
} orc_counters;
int orc_update_velocities(const ch_params* p, const double* phi, orc_particles* P,
                          int64_t step, double sbar, double* sbar_next, orc_counters* cnt);

/* UpdatePositions (src/particles.c:647-718). */
void orc_update_positions(const ch_params* p, orc_particles* P);

/* CollectVlasovQuantities (src/particles.c:136-255): CIC deposit into
 * `nodes` (N x {n, Gx, Gy, Gz} interleaved).  accumulate != 0 adds to the
 * existing values (the as-written behaviour, CH_FAITHFUL_D6). */
void orc_collect(const ch_params* p, const orc_particles* P, double* nodes, int accumulate);

/* ComputeFullRHS (src/rhs.c:133-303) and the alternatives (:8, :51). */
void orc_rhs(const ch_params* p, const double* nodes, double* b);

/* The 19 stencil values of one row of ComputeFullLHS (src/lhs.c:467-516),
 * in ComputeInteriorStencil order (src/lhs.c:7-106); cols receive natural
 * indices with periodic wrap.  lhs_type selects identity/laplacian/full. */
void orc_lhs_row(const ch_params* p, const double* n, int i, int j, int k,
                 double vals[19], int64_t cols[19]);

/* y = A(n) x, matrix free. */
void orc_apply(const ch_params* p, const double* n, const double* x, double* y);

/* Krylov solve of A(n) phi = b (CG or BiCGStab, optional Jacobi), constant
 * null space projected out, warm start from phi.  Converged when
 * ||b - A phi||_2 <= max(rtol ||b||_2, atol).  Returns 0 or CH_ERR_NOT_CONVERGED. */
int orc_solve(const ch_params* p, const double* n, const double* b, double* phi,
              double rtol, int maxit, int* its, double* rnorm, double* bnorm);

/* One time step of the reference loop (src/hybrid.c:107-117). */
typedef struct orc_state {
  ch_params p;
  orc_particles P;
  double* phi;      /* N */
  double* nodes;    /* 4N */
  double* rhs;      /* N */
  double* n_frozen; /* N, operator density for CH_FAITHFUL_D7 */
  double sbar;
  int solved_once;
} orc_state;
int orc_step(orc_state* s, int64_t step, orc_counters* cnt, int* its, double* rnorm, double* bnorm);
/* Initial moments and first solve (src/hybrid.c:67,81); also sets sbar. */
int orc_initialize(orc_state* s, int* its, double* rnorm, double* bnorm);

/* The differentiable model of the GPU adjoint with frozen collision events
 * (the FP64 step: gather, Boris, the given events, move, deposit, solve),
 * replayed at the parameters in p (E0, vn0) and L (amp[0]).  Events in
 * (step, ion, event) order: ev_step, ev_ion, ev_flags (1 = refused) and 5
 * doubles each (V - vn0, uz, uphi as a fraction of a turn).  Returns J, the
 * objective over the states after the last `window` steps:
 * flux_weight/(window N) sum_i v_x + phi_weight/(window N) sum phi^2. */
int orc_adj_objective(const ch_params* p, const ch_loader* L, int64_t np, int nsteps, int window,
                      double flux_weight, double phi_weight, int64_t nev, const int32_t* ev_step,
                      const uint32_t* ev_ion, const int32_t* ev_flags, const double* ev_data, double rtol,
                      double* J);

int64_t orc_sizeof_params(void);

/* Threads used by the loops (1 = serial, as the reference's per-rank loops). */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
