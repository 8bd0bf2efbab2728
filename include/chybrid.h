/*
 * chybrid.h -- C ABI of the GB300 (sm_103a) hybrid-PIC hot path.
 *
 * One step of the collisional hybrid particle-in-cell method on one GPU:
 *   UpdateVelocities   Boris push with E = -grad(phi) + ion-neutral collisions
 *   UpdatePositions    x += v dt with periodic wrap
 *   CollectVlasovQuantities  cloud-in-cell deposit of n and Gamma = n v
 *   ComputePotential   19-point quasineutral potential solve (matrix free)
 *
 * Every entry point returns ch_status (0 = CH_OK, negative = error); the
 * message of the last error on the calling thread is ch_last_error().
 * Host buffers are owned by the caller and copied in or out; device buffers
 * are owned by the ch_ctx.  Calls are synchronous at return.  One host
 * thread drives one ch_ctx at a time.
 *
 * Layouts follow the reference so that a PETSc host can pass its borrowed
 * arrays straight through:
 *   ch_real_vector == RealVector {x, y, z, r}  (src/hybrid.h:40-45), the
 *                     DMSwarm "position"/"velocity" field (src/setup.c:130-132)
 *   ch_grid_node   == GridNode {n, flux[3]}     (src/hybrid.h:140-143), the
 *                     dof-4 DMDA "vlasov" vector (src/setup.c:15-16)
 *   grid vectors are in DMDA natural order idx = (k*Ny + j)*Nx + i.
 */
#ifndef CHYBRID_H
#define CHYBRID_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CH_ABI_VERSION 1

typedef int32_t ch_status;
enum {
  CH_OK = 0,
  CH_ERR_ARG = -1,            /* bad argument or option value            */
  CH_ERR_CUDA = -2,           /* CUDA runtime error                      */
  CH_ERR_NOMEM = -3,          /* device or host allocation failed        */
  CH_ERR_NOT_CONVERGED = -4,  /* Krylov solve missed rtol within max_it  */
  CH_ERR_COLLISION_LIMIT = -5,/* >= 10 collisions refused in one step
                                 (src/particles.c:597-606)               */
  CH_ERR_NAN = -6,            /* non-finite value in a moment or phi     */
  CH_ERR_RANGE = -7,          /* fixed-point deposit range exceeded      */
  CH_ERR_TIMEOUT = -8,        /* a bounded device wait ran out           */
  CH_ERR_STATE = -9,          /* call out of order (e.g. no particles)   */
  CH_ERR_UNSUPPORTED = -10    /* option combination not implemented      */
};

/* RealVector (src/hybrid.h:40-45): the r slot is carried, never read. */
typedef struct ch_real_vector { double x, y, z, r; } ch_real_vector;
/* GridNode (src/hybrid.h:140-143). */
typedef struct ch_grid_node { double n, flux[3]; } ch_grid_node;

/* --lhs-type (src/lhs.h:8-12) */
enum { CH_LHS_IDENTITY = 0, CH_LHS_LAPLACIAN = 1, CH_LHS_FULL = 2 };
/* --rhs-type (src/rhs.h:8-12) */
enum { CH_RHS_CONSTANT = 0, CH_RHS_SINUSOIDAL = 1, CH_RHS_FULL = 2 };
/* -ksp_type / -pc_type subset */
enum { CH_KSP_CG = 0, CH_KSP_BCGS = 1 };
enum { CH_PC_NONE = 0, CH_PC_JACOBI = 1, CH_PC_MG = 2 };
/* -ch_precision */
enum { CH_FP64 = 0, CH_MIXED = 1 };
/* neutral-density profile (scales the local collision rate) */
enum { CH_NN_UNIFORM = 0, CH_NN_GAUSSIAN_X = 1 };

/* Reference-faithful switches, one bit per documented defect of the
 * reference's as-written code.  All off = the corrected algorithm. */
enum {
  CH_FAITHFUL_D2 = 1u << 2,  /* CrossProduct returns 0 (src/vectors.c:157-159) */
  CH_FAITHFUL_D3 = 1u << 3,  /* degenerate z lerp in DifferenceVector (src/vectors.c:61-67) */
  CH_FAITHFUL_D4 = 1u << 4,  /* one-sided difference at ixh==N (src/vectors.c:48-60) */
  CH_FAITHFUL_D5 = 1u << 5,  /* UpdatePositions discards x (src/particles.c:677-706) */
  CH_FAITHFUL_D6 = 1u << 6,  /* moments accumulate across steps (src/particles.c:242) */
  CH_FAITHFUL_D7 = 1u << 7,  /* operator A(n) frozen at the first solve */
  CH_FAITHFUL_D8 = 1u << 8   /* d2Fdyz uses the x-z stencil (src/calculus.c:464) */
};

/* Run parameters: the Context fields that the hot path reads
 * (src/hybrid.h:106-138) after ProcessOptions (src/parameters.c:28-562)
 * has derived them.  Option names in the comments are the reference's. */
typedef struct ch_params {
  int32_t Nx, Ny, Nz;        /* -Nx -Ny -Nz                                   */
  int32_t precision;         /* CH_FP64 | CH_MIXED  (-ch_precision)           */
  double x0, y0, z0;         /* -x0 -y0 -z0                                   */
  double x1, y1, z1;         /* -x1 -y1 -z1   (L = x1-x0, d = L/N, src/setup.c:47-49) */
  double qi, mi;             /* -qi -mi                                       */
  double nui;                /* -nui  ion-neutral collision frequency         */
  double dt;                 /* -dt                                           */
  double vi0[3];             /* -vi0x -vi0y -vi0z  ion drift (enters vrm)     */
  double viT[3];             /* -viTx -viTy -viTz  ion per-component thermal speed */
  double mn;                 /* -mn   neutral mass; <= 0 disables collisions  */
  double vnT;                /* neutral thermal speed (std of each component) */
  double vn0[3];             /* -vn0x -vn0y -vn0z neutral drift               */
  double B0[3];              /* -B0x -B0y -B0z                                */
  double E0[3];              /* -E0x -E0y -E0z  (enters the RHS only)         */
  double kappa_e[3];         /* electron magnetization Omega_e/nu_e           */
  double cth;                /* gamma kB Te / e  (src/rhs.c:190)              */
  double cG;                 /* me nue / e       (src/rhs.c:191)              */
  int32_t lhs_type;          /* --lhs-type  CH_LHS_*                          */
  int32_t rhs_type;          /* --rhs-type  CH_RHS_*                          */
  int32_t ksp_type;          /* -ksp_type cg|bcgs                             */
  int32_t pc_type;           /* -ch_pc none|jacobi|mg                         */
  double ksp_rtol;           /* -ksp_rtol                                     */
  double ksp_atol;           /* -ksp_atol                                     */
  int32_t ksp_max_it;        /* -ksp_max_it                                   */
  int32_t nn_profile;        /* CH_NN_*                                       */
  double nn_center, nn_sigma, nn_floor;  /* Gaussian neutral-density profile  */
  uint64_t seed;             /* -ch_seed  Philox key                          */
  uint32_t run;              /* ensemble member index (Philox counter word 3) */
  uint32_t faithful;         /* CH_FAITHFUL_* bits                            */
  int32_t push_E0;           /* -ch_push_E0: add E0 to the ion push           */
  int32_t sort_period;       /* steps between counting sorts (0 = never)      */
  double deposit_scale_log2; /* fixed-point deposit scale 2^s (0 = default:  
                                2^48 in the FP64 form, 2^40 in the mixed form) */
} ch_params;

/* Fills *p with the reference defaults (src/parameters.c:28-562) in
 * normalised units: e = kB = 1.  Grid, species and solver fields that the
 * reference derives are set for a 7^3 unit box, periodic. */
ch_status ch_params_default(ch_params* p);

/* Per-solve report (KSPGetIterationNumber / KSPGetResidualNorm). */
typedef struct ch_solve_info {
  int32_t iterations;        /* Krylov iterations (outer + inner for mixed)   */
  int32_t refinements;       /* FP64 refinement passes (mixed form)           */
  double rnorm;              /* ||b - A phi||_2, FP64, unpreconditioned       */
  double bnorm;              /* ||b||_2                                       */
} ch_solve_info;

/* Per-step counters. */
typedef struct ch_step_info {
  int64_t Nc;                /* collisions the reference would attempt (src/particles.c:514) */
  int64_t collisions;        /* accepted ion-neutral collisions               */
  int64_t refused;           /* collisions refused for |v_f| > 10 vT          */
  double expected;           /* sum of per-ion collision probabilities        */
  double moment_sum[4];      /* FP64 global sums of n, Gx, Gy, Gz             */
  ch_solve_info solve;       /* last potential solve of the call              */
} ch_step_info;

/* Opaque per-run state: device particles, grid fields, solver workspace. */
typedef struct ch_ctx ch_ctx;

const char* ch_last_error(void);
int32_t ch_abi_version(void);

/* Creates the device state for one run (SetUpVlasovDM, SetUpPotentialDM,
 * SetUpIonsDM; src/setup.c:6,71,105).  Selects device `device` (-1: current). */
ch_status ch_create(const ch_params* p, int32_t device, ch_ctx** out);
ch_status ch_destroy(ch_ctx* c);

/* Copies np ions in (DMSwarm "position"/"velocity", AoS 32 B each).  Ion id
 * = array index; ids key the Philox streams. */
ch_status ch_particles_upload(ch_ctx* c, const ch_real_vector* pos,
                              const ch_real_vector* vel, int64_t np);
/* Copies the ions out in id order (the order they were uploaded). */
ch_status ch_particles_download(ch_ctx* c, ch_real_vector* pos, ch_real_vector* vel);

/* Seeded synthetic plasma on the device (replaces InitializePositions /
 * InitializeVelocities, src/particles.c:9-132): x by inverse CDF of
 * n(x) = 1 + sum_m amp[m] sin(2 pi m x/Lx + phase[m]), m = 1..3; y, z uniform;
 * v = v0 + vT * N(0,1) per component, Philox-keyed by (id, seed). */
typedef struct ch_loader {
  double amp[3];
  double phase[3];
  double v0[3];
  double vT[3];
} ch_loader;
ch_status ch_particles_load(ch_ctx* c, int64_t np, const ch_loader* L);

/* --density-type (DensityTypes, src/parameters.c:18-20, default flat-sobol) */
enum {
  CH_DENSITY_FLAT_SOBOL = 0,   /* SobolDistribution (src/distributions.c:96-128) */
  CH_DENSITY_FLAT_REVERSE = 1, /* not implemented in the reference either      */
  CH_DENSITY_FLAT_NORMAL = 2,  /* not implemented in the reference either      */
  CH_DENSITY_UNIFORM = 3,      /* UniformDistribution (src/distributions.c:33-94) */
  CH_DENSITY_SINUSOIDAL = 4,   /* Rejection of SinusoidalDistribution (:131-232) */
  CH_DENSITY_GAUSSIAN = 5      /* not implemented in the reference either      */
};
/* InitializePositions (src/particles.c:9-132) with the reference's
 * --density-type placements, and Maxwellian velocities v0 + vT N(0,1) from
 * L (InitializeVelocities, :136-165; Philox-keyed by ion id and seed; L's
 * density modes are not used):
 *   flat-sobol  point id + 1 of a 3-D Sobol sequence in Gray-code order
 *               (direction numbers of Joe & Kuo for the first three
 *               dimensions), v = r (L + d) - d/2 per axis, clamped to
 *               [p0 + 0.01 d, p1 - 0.01 d] as the reference clamps;
 *   uniform     np / (Nx Ny Nz) ions at the centre of every cell (np must be
 *               a multiple of the cell count; the reference fills all but
 *               the last cell of each axis and leaves the rest at the origin);
 *   sinusoidal  rejection sampling of n = 1 + 0.25 sin(2 pi x) over the box,
 *               with the bound 1.25 (the reference evaluates its bound at
 *               integer points, where the sine vanishes).
 * flat-reverse, flat-normal and gaussian return CH_ERR_UNSUPPORTED, as the
 * reference's InitializePositions does (src/particles.c:28-45). */
ch_status ch_particles_load_placed(ch_ctx* c, int64_t np, const ch_loader* L, int32_t density_type);

/* UpdateVelocities (src/particles.c:628-643): BorisMover (:348-464) with E
 * gathered from the current phi, then ComputeCollisions (:471-624) if mn > 0.
 * `step` keys the Philox streams of this step. */
ch_status ch_update_velocities(ch_ctx* c, int64_t step, ch_step_info* info);
/* UpdatePositions (src/particles.c:647-718). */
ch_status ch_update_positions(ch_ctx* c);
/* CollectVlasovQuantities (src/particles.c:136-255).  host_out (nullable)
 * receives Nx*Ny*Nz GridNode in natural order. */
ch_status ch_collect_moments(ch_ctx* c, ch_grid_node* host_out, ch_step_info* info);
/* ComputePotential (src/potential.c:6-15): RHS (rhs.c), operator (lhs.c),
 * Krylov solve warm-started from the previous phi.  phi_out nullable. */
ch_status ch_compute_potential(ch_ctx* c, double* phi_out, ch_solve_info* info);
/* KSPSetType / KSPSetTolerances as KSPSetFromOptions applies them
 * (src/hybrid.c:75): the Krylov method (CH_KSP_CG | CH_KSP_BCGS), the
 * preconditioner (CH_PC_*), rtol, atol and max_it of the following solves.
 * A solve with CG while kappa_e != 0 and the full LHS returns
 * CH_ERR_UNSUPPORTED: that operator is not symmetric (src/lhs.c:412-420). */
ch_status ch_set_solver(ch_ctx* c, int32_t ksp_type, int32_t pc_type, double rtol, double atol, int32_t max_it);
/* The reference time-loop body (src/hybrid.c:101-123) without output,
 * nsteps times, steps numbered first_step, first_step+1, ... */
ch_status ch_step(ch_ctx* c, int64_t first_step, int32_t nsteps, ch_step_info* info);
/* The same steps with the ions held by the host, as DMSwarm keeps them in
 * the reference's loop (src/hybrid.c:101-123): uploads pos / vel (the ions
 * last uploaded or downloaded, same count), runs nsteps >= 1 steps and
 * downloads the ions into pos / vel in id order.  With registered arrays
 * (ch_host_register, ch_host_alloc) in the mixed form, once the arrays hold
 * the ions in the id order of a previous transfer, the first step's push
 * reads them straight from the host arrays and the last step's push writes
 * its result back in the same launch, so the upload and the download share
 * the host link (nearly duplex); it uses the collision-rate sum S of the
 * previous step and runs the step again the ordinary way if the host
 * changed velocities since (the result is the same either way).  Otherwise
 * the download of the last step starts once its push has moved the ions and
 * overlaps its deposit and potential solve, or follows the steps. */
ch_status ch_step_host(ch_ctx* c, int64_t first_step, int32_t nsteps, ch_real_vector* pos,
                       ch_real_vector* vel, ch_step_info* info);

/* Grid-vector access for hosts and tests (natural order, FP64). */
ch_status ch_set_moments(ch_ctx* c, const ch_grid_node* host_in);  /* LoadVlasovQuantities, src/fileio.c:6-70 */
ch_status ch_get_phi(ch_ctx* c, double* out);
ch_status ch_set_phi(ch_ctx* c, const double* in);
ch_status ch_get_rhs(ch_ctx* c, double* out);   /* ctx->rhs after the last RHS build */
/* y = A(n) x with the current operator (matrix-free ComputeFullLHS). */
ch_status ch_apply_operator(ch_ctx* c, const double* x, double* y);

/* Per-phase device timing (CUDA events on the context's stream) and the
 * number of kernels this library launched, for profiling hosts.  No
 * counterpart in the reference (its only timing is src/hybrid.c:133-137). */
typedef struct ch_profile {
  double pass_ms;      /* ion passes (push / move / deposit, fused or not) */
  int64_t pass_calls;
  double solve_ms;     /* RHS + Krylov solve */
  int64_t solve_calls;
  double sort_ms;      /* counting sort by cell */
  int64_t sort_calls;
  double moments_ms;   /* fixed-point -> FP64 moment conversion */
  int64_t moments_calls;
  int64_t launches;    /* kernels launched by this library, all contexts */
  double deposit_ms;   /* the deposit-only passes among pass_ms */
  int64_t deposit_calls;
  int64_t host_push_calls;   /* ch_step_host pushes that streamed the host arrays */
  int64_t host_push_reruns;  /* of those, steps run again because the host had
                                changed velocities since the last transfer */
} ch_profile;
ch_status ch_set_profiling(ch_ctx* c, int32_t enable);
ch_status ch_get_profile(ch_ctx* c, ch_profile* out);
ch_status ch_reset_profile(ch_ctx* c);
/* The cudaStream_t every call of this context is ordered on. */
ch_status ch_get_stream(ch_ctx* c, void** stream);

/* OutputHDF5 (src/fileio.c:73-126) without HDF5.  ch_output_open sets the
 * file stem (the reference's ctx->outstem); ch_output then writes the current
 * density, x/y/z flux, rhs and potential -- the reference's dataset names --
 * as <stem><insert>.<field>.f64 (raw little-endian FP64, DMDA natural order;
 * spaces in names become '_') with a manifest <stem><insert>.json.  The fields
 * are snapshot on the device at once; the copy to the host and the file
 * writes run beside the following steps (a second stream and a host thread,
 * two slots in flight).  ch_output_wait returns when every queued output is
 * on disk (written: files-sets written so far; nullable). */
ch_status ch_output_open(ch_ctx* c, const char* stem);
ch_status ch_output(ch_ctx* c, const char* insert);
ch_status ch_output_wait(ch_ctx* c, int64_t* written);

/* CollectVlasovQuantities for callers that cannot allocate device memory
 * (no counterpart in the reference).  Hosts whose device memory belongs to
 * their own pool allocator (a framework that reserves the GPU's memory up
 * front and hands out sub-blocks) and time-critical loops that cannot absorb
 * the device-wide synchronisation of cudaMalloc/cudaFree cannot create a
 * ch_ctx; this call needs none.  It allocates nothing: the caller passes
 * device pointers to the ions (FP64 SoA positions and velocities, np of
 * each) and to the output `moments` (4 * Nx*Ny*Nz doubles: n, then Gx, Gy,
 * Gz, each in DMDA natural order), and the deposit's fixed-point scratch
 * lives in a static device array of 4 * 2^18 * 8 bytes = 8 MiB, so grids of
 * at most 2^18 nodes (64^3) are accepted; larger grids return CH_ERR_ARG.
 * Every GPU that loads the library holds that array until the process
 * exits.  The work is queued on `stream` (a cudaStream_t; NULL = the legacy
 * default stream) and the call returns without waiting.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) in that
 * device's primary context, so make that first call before any stream
 * capture; callers on a non-primary driver context, or that reset the device
 * between calls, are not supported.  All calls share the one array, and each
 * call clears it before depositing: calls that may overlap on the GPU
 * (different streams, or different host threads) race and must be
 * serialised by the caller.  For finite ions the moments equal those of
 * ch_collect_moments in the FP64 form bit for bit (same fixed-point sums,
 * default scale 2^48).
 * An ion with a non-finite position or velocity, or one so far out that no
 * cell index or fixed-point contribution fits, or a density sum beyond the
 * fixed-point range, makes every output value NaN: the asynchronous form of
 * the CH_ERR_NAN / CH_ERR_RANGE that ch_collect_moments returns. */
ch_status ch_collect_moments_noalloc(const ch_params* p, const double* x, const double* y, const double* z,
                                     const double* vx, const double* vy, const double* vz, int64_t np,
                                     double* moments, void* stream);

/* ---------------------------------------------------------------------
 * Ensembles (no counterpart in the reference, whose run-batch script starts
 * one process per parameter set).  A ch_batch advances nruns independent
 * runs -- each with its own grid, ion count, parameters and seed -- together:
 * every phase of a step is one launch over all runs (one persistent pass over
 * every run's bricks; one potential solve with a thread-block cluster per
 * run), and a step is replayed from a captured CUDA graph.  Mixed precision,
 * full LHS and RHS, CG with the multigrid preconditioner; the physics of
 * each run is that of ch_step on a ch_ctx with the same parameters.
 * --------------------------------------------------------------------- */
typedef struct ch_batch ch_batch;

/* Per-run report of the last step of a ch_batch_step call. */
typedef struct ch_run_info {
  int64_t Nc;                /* collisions the reference would attempt        */
  int64_t collisions;        /* accepted ion-neutral collisions               */
  int64_t refused;           /* refused (|v_f| > 10 vT)                       */
  double expected;           /* sum of per-ion collision probabilities        */
  ch_solve_info solve;       /* the run's potential solve                     */
  int32_t status;            /* CH_OK or the run's error                      */
  int32_t flags;             /* 1 bad density, 2 not converged, 4 non-finite residual,
                                8 refused >= 10, 16 non-finite ion, 32 deposit range */
} ch_run_info;

/* Launch shape of the ensemble step; ch_batch_autotune picks it by timing. */
typedef struct ch_batch_tuning {
  int32_t cluster;           /* CTAs per run in the potential solve: 1, 2, 4, 8 */
  int32_t pass_ctas_per_sm;  /* persistent CTAs per SM of the deposit: 1 to 3 */
  double pass_ms;            /* measured for the chosen shape (autotune)      */
  double solve_ms;
  int32_t cluster_big;       /* CTAs per large run (node count >= twice the
                                mean) solved in a launch of their own beside
                                the others: 0 (no such launch), 8 or 16      */
} ch_batch_tuning;

/* Creates the device state of nruns runs (all CH_MIXED, lhs/rhs full,
 * ksp cg, pc mg, sort_period equal across runs).  Ion counts are fixed here:
 * np[r] ions for run r. */
ch_status ch_batch_create(const ch_params* runs, const int64_t* np, int32_t nruns, int32_t device,
                          ch_batch** out);
ch_status ch_batch_destroy(ch_batch* b);
/* Seeded synthetic plasma of every run (loaders[r], the run's seed and run
 * index), as ch_particles_load. */
ch_status ch_batch_load(ch_batch* b, const ch_loader* loaders);
/* Ions of run r from host AoS arrays (np[r] each), as ch_particles_upload. */
ch_status ch_batch_upload(ch_batch* b, int32_t run, const ch_real_vector* pos, const ch_real_vector* vel);
ch_status ch_batch_download(ch_batch* b, int32_t run, ch_real_vector* pos, ch_real_vector* vel);
/* Sorts every run's ions, deposits the moments and solves the initial
 * potential of every run (CollectVlasovQuantities + ComputePotential before
 * the time loop, src/hybrid.c:94-99).  Call after load/upload. */
ch_status ch_batch_initialize(ch_batch* b);
/* nsteps steps of every run, numbered first_step, first_step + 1, ...
 * info (nullable) receives nruns reports of the last step.  Errors of any
 * run are reported when the call returns. */
ch_status ch_batch_step(ch_batch* b, int64_t first_step, int32_t nsteps, ch_run_info* info);
ch_status ch_batch_get_phi(ch_batch* b, int32_t run, double* out);
ch_status ch_batch_get_moments(ch_batch* b, int32_t run, ch_grid_node* out);
ch_status ch_batch_set_phi(ch_batch* b, int32_t run, const double* in);
/* Times every launch shape on the current state (which is restored) and
 * keeps the fastest; out (nullable) receives the choice. */
ch_status ch_batch_autotune(ch_batch* b, ch_batch_tuning* out);
ch_status ch_batch_set_tuning(ch_batch* b, const ch_batch_tuning* t);
/* ch_batch_autotune with a cache file of JSON lines, kept across processes:
 * a batch of the same class (device name and SM count, run count, and the
 * power-of-two buckets of its total nodes, total ions and largest run)
 * takes the stored launch shape without timing (*hit = 1); otherwise it is
 * tuned and a line is appended (*hit = 0).  hit and out are nullable. */
ch_status ch_batch_autotune_cached(ch_batch* b, const char* path, ch_batch_tuning* out, int32_t* hit);
ch_status ch_batch_get_tuning(ch_batch* b, ch_batch_tuning* out);
/* Per-phase timing of ch_batch_step (events; graphs are not used while
 * profiling is on) and the stream of the batch. */
ch_status ch_batch_set_profiling(ch_batch* b, int32_t enable);
ch_status ch_batch_get_profile(ch_batch* b, ch_profile* out);
ch_status ch_batch_get_stream(ch_batch* b, void** stream);

/* ---------------------------------------------------------------------
 * Differentiation (no counterpart in the reference).  A discrete adjoint of
 * the FP64 step with the collision events and scattering draws of a
 * recorded run frozen.  Parameters theta = (E0x, E0y, E0z, vn0x, vn0y, vn0z,
 * amp), amp = loader amp[0] (the first density mode).  Objective, summed
 * over the states after the last `window` steps:
 *   J = sum_k [ flux_weight/(window N) sum_i v_x,i + phi_weight/(window N) sum_c phi_c^2 ]
 * (sum_i v_x,i is the sum over nodes of Gamma_x: the mean x-directed ion flux
 * times N).  kappa_e = 0, full LHS/RHS, uniform neutrals.
 * --------------------------------------------------------------------- */
typedef struct ch_adjoint ch_adjoint;
#define CH_ADJ_NTHETA 7
typedef struct ch_adjoint_config {
  int32_t nsteps;            /* steps of the run                              */
  int32_t checkpoint_every;  /* ion-state checkpoints every k steps           */
  int32_t window;            /* the objective covers the final `window` steps */
  int32_t pad;
  double flux_weight;        /* weight of the mean x flux                     */
  double phi_weight;         /* weight of the mean square potential           */
} ch_adjoint_config;
typedef struct ch_adjoint_timing {
  double forward_ms;         /* last ch_adjoint_forward                       */
  double gradient_ms;        /* last ch_adjoint_gradient (recompute included) */
  double recompute_ms;       /* its segment recomputation                     */
  int64_t events;            /* frozen collision events of the recorded run   */
} ch_adjoint_timing;
ch_status ch_adjoint_create(const ch_params* p, int64_t np, const ch_loader* L, const ch_adjoint_config* cfg,
                            int32_t device, ch_adjoint** out);
ch_status ch_adjoint_destroy(ch_adjoint* a);
/* The forward model at theta (CH_ADJ_NTHETA values).  record = 1 draws the
 * collision events (Philox, as the FP64 step) and freezes them, stores the
 * checkpoints and makes theta the point of the next gradient; record = 0
 * replays the frozen events at this theta (finite differences). */
ch_status ch_adjoint_forward(ch_adjoint* a, const double* theta, int32_t record, double* J);
/* dJ/dtheta at the recorded point; J (nullable) receives J there. */
ch_status ch_adjoint_gradient(ch_adjoint* a, double* grad, double* J);
/* The frozen events, for an independent replay: with null arrays *count
 * receives the number; otherwise `count` events in (step, ion, event) order:
 * step, ion, flags (1 = refused) and 5 doubles each (V - vn0 (3), uz, uphi
 * as a fraction of a turn). */
ch_status ch_adjoint_events(ch_adjoint* a, int64_t* count, int32_t* step, uint32_t* ion, int32_t* flags,
                            double* data);
ch_status ch_adjoint_get_timing(ch_adjoint* a, ch_adjoint_timing* out);

/* Page-locks caller memory so that the copies of upload/download run at
 * full link speed (no counterpart in the reference: its arrays never leave
 * the host). */
ch_status ch_host_register(void* ptr, uint64_t bytes);
ch_status ch_host_unregister(void* ptr);
/* Page-locked host memory for hosts that own their particle arrays: an
 * anonymous mapping backed by transparent huge pages where the kernel offers
 * them, touched, page-locked and mapped for the GPU.  The GPU streams it at
 * the full host-link rate however fragmented free memory has become, where
 * registered base pages of an ordinary allocation can come many times
 * slower.  Free with ch_host_free.  (No counterpart in the reference.) */
ch_status ch_host_alloc(uint64_t bytes, void** out);
ch_status ch_host_free(void* ptr);

#ifdef __cplusplus
}
#endif
#endif /* CHYBRID_H */
