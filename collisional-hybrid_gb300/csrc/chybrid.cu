// chybrid.cu -- the C ABI (include/chybrid.h) over the sm_103a kernels.
//
// Mirrors the reference's per-step entry points (src/particles.h:11-21,
// src/potential.h:7-13): one ch_ctx holds what Context + the DMDA/DMSwarm/KSP
// objects hold in the reference, all resident in HBM.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <sys/mman.h>
#include <unistd.h>
#include <new>
#include <string>
#include <vector>
#include <thread>
#include <vector>

#include "particles.cuh"
#include "solver.cuh"

using namespace ch;

static thread_local char g_err[512] = "";

// Host ranges page-locked through ch_host_register, with the device address
// of each mapping.  A transfer whose whole host range lies inside one of
// them is done by the conversion kernels reading (or a copy kernel writing)
// host memory directly over the C2C link instead of a staging copy.
struct HostRange {
  char* p;
  uint64_t n;
  char* d;
};
static std::mutex g_hr_mu;
static std::vector<HostRange> g_hr;

static void* device_view(const void* ptr, uint64_t bytes, uint64_t align) {
  if (!ptr || ((uintptr_t)ptr % align) != 0) return nullptr;
  const char* q = static_cast<const char*>(ptr);
  std::lock_guard<std::mutex> lk(g_hr_mu);
  for (const auto& r : g_hr)
    if (r.d && q >= r.p && q + bytes <= r.p + r.n) return r.d + (q - r.p);
  return nullptr;
}

ch_status ch_fail(ch_status code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

ch_status ch_cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  return ch_fail(e == cudaErrorMemoryAllocation ? CH_ERR_NOMEM : CH_ERR_CUDA, "%s failed: %s (%s:%d)", what,
                 cudaGetErrorString(e), file, line);
}

static std::atomic<unsigned long long> g_launches{0};
void ch::note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void ch::note_launch_n(long long n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
unsigned long long ch::launches_now() { return g_launches.load(); }

struct ChOutput;

struct ch_ctx {
  ChOutput* out = nullptr;  // asynchronous output (ch_output_*), created on demand
  ch_params p;
  GridDesc g;
  int device = 0;
  int sms = 1;
  bool mixed = false;
  cudaStream_t stream = nullptr;
  int64_t np = 0;
  // ions (ping-pong buffers for the counting sort)
  F64Particles P{}, Q{};
  MixParticles M{}, MQ{};
  uint32_t* keys = nullptr;
  // grid
  uint32_t *counts = nullptr, *starts = nullptr, *cursor = nullptr, *block_sums = nullptr;
  uint32_t* starts_next = nullptr;  // the order a step's fused deposit + scatter writes (mixed form)
  double *phi = nullptr, *E64 = nullptr, *mom = nullptr, *rhs = nullptr, *nfz = nullptr;
  float4* E32 = nullptr;
  unsigned long long* acc = nullptr;
  // reductions
  DevCounters* cnt = nullptr;
  DevCounters* hcnt = nullptr;
  double* part = nullptr;
  int part_cap = 0;
  double* red = nullptr;
  double* hred = nullptr;
  // staging for AoS transfers
  double4_32a *stage_pos = nullptr, *stage_vel = nullptr;
  // slot of each ion id in the current order (mixed form), made by a download
  // into mapped host arrays; valid until the order changes (sort, load)
  uint32_t* slot_of_id = nullptr;
  bool slot_map_valid = false;
  // the ions as a host-streaming push read them (k_host_push), kept so that
  // the step can be run again the ordinary way if their S differs
  MixParticles HB{};
  // download of registered arrays: conversion chunks on `stream`, their
  // downloads: id-order conversion on conv_stream, copies to the host on
  // copy_stream (chunk_ev[k]: chunk k converted)
  cudaStream_t copy_stream = nullptr, conv_stream = nullptr;
  cudaEvent_t chunk_ev[8] = {};
  // state
  double sbar = 0.0;
  double dep_scale = 0.0;
  bool solved_once = false;
  bool moments_valid = false;
  int64_t since_sort = 0;
  PotentialSolver solver;
  // profiling: each phase's pair of events is resolved when the profile is
  // read or a step returns, so timing adds no host round trip inside a step
  struct ProfPhase {
    cudaEvent_t a, b;
    double *ms, *ms2;
  };
  bool prof = false;
  std::vector<cudaEvent_t> ev_free;
  std::vector<ProfPhase> ev_pending;
  cudaEvent_t ev_open = nullptr;
  ch_profile pr{};
};

// Times [begin, end) of one phase on the context stream when profiling.
// The events are read later (prof_flush), so the stream keeps running; the
// call counts are taken at once.
static cudaEvent_t prof_event(ch_ctx* c) {
  cudaEvent_t e = nullptr;
  if (!c->ev_free.empty()) {
    e = c->ev_free.back();
    c->ev_free.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    e = nullptr;
  }
  return e;
}
// Adds the elapsed times of the recorded phases (waiting for their ends).
static void prof_flush(ch_ctx* c) {
  for (const auto& q : c->ev_pending) {
    float t = 0.0f;
    if (cudaEventSynchronize(q.b) == cudaSuccess && cudaEventElapsedTime(&t, q.a, q.b) == cudaSuccess) {
      *q.ms += t;
      if (q.ms2) *q.ms2 += t;
    }
    c->ev_free.push_back(q.a);
    c->ev_free.push_back(q.b);
  }
  c->ev_pending.clear();
}
static void prof_begin(ch_ctx* c) {
  if (!c->prof) return;
  if (!c->ev_open) c->ev_open = prof_event(c);
  if (c->ev_open) cudaEventRecord(c->ev_open, c->stream);
}
// ms2 / calls2 (nullable): a second tally the phase also counts towards.
static void prof_end(ch_ctx* c, double* ms, int64_t* calls, double* ms2 = nullptr, int64_t* calls2 = nullptr) {
  if (!c->prof) return;
  *calls += 1;
  if (calls2) *calls2 += 1;
  cudaEvent_t e = c->ev_open ? prof_event(c) : nullptr;
  if (!e) return;
  cudaEventRecord(e, c->stream);
  c->ev_pending.push_back(ch_ctx::ProfPhase{c->ev_open, e, ms, ms2});
  c->ev_open = nullptr;
  if (c->ev_pending.size() >= 256) prof_flush(c);  // bounded
}

extern "C" const char* ch_last_error(void) { return g_err; }
extern "C" int32_t ch_abi_version(void) { return CH_ABI_VERSION; }

extern "C" ch_status ch_params_default(ch_params* p) {
  if (!p) return ch_fail(CH_ERR_ARG, "ch_params_default: null");
  memset(p, 0, sizeof(*p));
  // src/parameters.c:28-562 defaults in normalised units (e = kB = 1, mi = 1)
  p->Nx = p->Ny = p->Nz = 7;  // src/setup.c:10-12
  p->x1 = p->y1 = p->z1 = 1.0;
  p->qi = 1.0;
  p->mi = 1.0;
  p->nui = 1.0;
  p->dt = 1.0 / p->nui;  // src/parameters.c:417
  p->mn = p->mi;         // src/parameters.c:337
  p->vnT = 0.0;          // sqrt(2 kB Tn/mn) with Tn = Ti = 0
  p->cth = 0.0;          // Te = 0
  p->cG = 1.0 / 1836.15267343;  // me nue / e with nue = 1, me/mi
  p->lhs_type = CH_LHS_FULL;
  p->rhs_type = CH_RHS_FULL;
  p->ksp_type = CH_KSP_CG;
  p->pc_type = CH_PC_JACOBI;
  p->ksp_rtol = 1e-5;  // PETSc KSP defaults
  p->ksp_atol = 1e-50;
  p->ksp_max_it = 10000;
  p->precision = CH_FP64;
  p->seed = 12345;     // |-(rank+1)*12345| for rank 0 (src/hybrid.c:49)
  p->nn_profile = CH_NN_UNIFORM;
  p->nn_sigma = 1.0;
  p->sort_period = 8;
  return CH_OK;
}

static ch_status validate(const ch_params* p) {
  if (p->Nx < 3 || p->Ny < 3 || p->Nz < 3)
    return ch_fail(CH_ERR_ARG, "grid %dx%dx%d: each axis needs at least 3 nodes for the 19-point stencil", p->Nx,
                   p->Ny, p->Nz);
  if ((int64_t)p->Nx * p->Ny * p->Nz >= (1LL << 31))
    return ch_fail(CH_ERR_ARG, "grid %dx%dx%d: at most 2^31-1 nodes", p->Nx, p->Ny, p->Nz);
  if (p->Nx > CH_MAX_NX || p->Ny > CH_MAX_NY || p->Nz > CH_MAX_NZ)
    return ch_fail(CH_ERR_ARG, "grid %dx%dx%d exceeds %dx%dx%d", p->Nx, p->Ny, p->Nz, CH_MAX_NX, CH_MAX_NY,
                   CH_MAX_NZ);
  if (!(p->x1 > p->x0) || !(p->y1 > p->y0) || !(p->z1 > p->z0)) return ch_fail(CH_ERR_ARG, "empty domain");
  if (!(p->mi > 0.0)) return ch_fail(CH_ERR_ARG, "ion mass must be positive");
  if (!(p->dt > 0.0) || !isfinite(p->dt)) return ch_fail(CH_ERR_ARG, "dt must be positive");
  if (p->precision != CH_FP64 && p->precision != CH_MIXED) return ch_fail(CH_ERR_ARG, "unknown precision");
  if (p->ksp_type != CH_KSP_CG && p->ksp_type != CH_KSP_BCGS) return ch_fail(CH_ERR_ARG, "unknown ksp_type");
  if (p->pc_type != CH_PC_NONE && p->pc_type != CH_PC_JACOBI && p->pc_type != CH_PC_MG)
    return ch_fail(CH_ERR_ARG, "unknown pc_type");
  if (p->lhs_type < 0 || p->lhs_type > 2 || p->rhs_type < 0 || p->rhs_type > 2)
    return ch_fail(CH_ERR_ARG, "unknown lhs/rhs type");
  if (p->precision == CH_MIXED && (p->faithful & (CH_FAITHFUL_D3 | CH_FAITHFUL_D4)))
    return ch_fail(CH_ERR_UNSUPPORTED, "the as-written DifferenceVector (D3/D4) runs in the FP64 form only");
  if (!(p->ksp_rtol > 0.0) || p->ksp_max_it < 1) return ch_fail(CH_ERR_ARG, "bad ksp tolerance / max_it");
  if (p->mn > 0.0 && !(p->viT[0] > 0.0 || p->viT[1] > 0.0 || p->viT[2] > 0.0))
    return ch_fail(CH_ERR_ARG, "collisions need a positive ion thermal speed (vrm, src/particles.c:511)");
  if (p->deposit_scale_log2 != 0.0 &&
      !(p->deposit_scale_log2 >= (p->precision == CH_MIXED ? 22.0 : 1.0) && p->deposit_scale_log2 <= 62.0))
    return ch_fail(CH_ERR_ARG, "deposit_scale_log2 %g outside [%d, 62]", p->deposit_scale_log2,
                   p->precision == CH_MIXED ? 22 : 1);
  return CH_OK;
}

static GridDesc make_grid(const ch_params& p) {
  GridDesc g;
  g.Nx = p.Nx; g.Ny = p.Ny; g.Nz = p.Nz;
  ch_grid_finish(g);
  g.x0 = p.x0; g.y0 = p.y0; g.z0 = p.z0;
  g.Lx = p.x1 - p.x0; g.Ly = p.y1 - p.y0; g.Lz = p.z1 - p.z0;
  g.dx = g.Lx / p.Nx; g.dy = g.Ly / p.Ny; g.dz = g.Lz / p.Nz;
  return g;
}

static void free_particles(ch_ctx* c) {
  void* v[] = {c->P.x, c->P.y, c->P.z, c->P.vx, c->P.vy, c->P.vz, c->P.id, c->Q.x, c->Q.y, c->Q.z, c->Q.vx,
               c->Q.vy, c->Q.vz, c->Q.id, c->M.pos, c->M.vel, c->MQ.pos, c->MQ.vel, c->keys, c->stage_pos,
               c->stage_vel, c->part, c->slot_of_id, c->HB.pos, c->HB.vel};
  for (void* q : v)
    if (q) cudaFree(q);
  c->HB = MixParticles{};
  c->slot_of_id = nullptr;
  c->slot_map_valid = false;
  c->P = F64Particles{};
  c->Q = F64Particles{};
  c->M = MixParticles{};
  c->MQ = MixParticles{};
  c->keys = nullptr;
  c->stage_pos = c->stage_vel = nullptr;
  c->part = nullptr;
  c->part_cap = 0;
  c->np = 0;
}

static void output_close(ch_ctx* c);

extern "C" ch_status ch_destroy(ch_ctx* c) {
  if (!c) return CH_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  output_close(c);
  free_particles(c);
  void* v[] = {c->counts, c->starts, c->starts_next, c->cursor, c->block_sums, c->phi, c->E64, c->mom, c->rhs, c->nfz,
               c->E32, c->acc, c->cnt, c->red};
  for (void* q : v)
    if (q) cudaFree(q);
  if (c->hcnt) cudaFreeHost(c->hcnt);
  if (c->hred) cudaFreeHost(c->hred);
  c->solver.release();
  prof_flush(c);
  for (cudaEvent_t e : c->ev_free) cudaEventDestroy(e);
  if (c->ev_open) cudaEventDestroy(c->ev_open);
  for (cudaEvent_t e : c->chunk_ev)
    if (e) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->conv_stream) cudaStreamDestroy(c->conv_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return CH_OK;
}

extern "C" ch_status ch_create(const ch_params* p, int32_t device, ch_ctx** out) {
  if (!p || !out) return ch_fail(CH_ERR_ARG, "ch_create: null argument");
  *out = nullptr;
  ch_status rc = validate(p);
  if (rc) return rc;
  int ndev = 0;
  CH_CUDA_OK(cudaGetDeviceCount(&ndev));
  if (ndev < 1) return ch_fail(CH_ERR_CUDA, "no CUDA device");
  if (device >= 0) CH_CUDA_OK(cudaSetDevice(device));
  ch_ctx* c = new (std::nothrow) ch_ctx();
  if (!c) return ch_fail(CH_ERR_NOMEM, "ch_create: host allocation");
  c->p = *p;
  c->g = make_grid(*p);
  c->mixed = p->precision == CH_MIXED;
  CH_CUDA_OK(cudaGetDevice(&c->device));
  CH_CUDA_OK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device));
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { ch_destroy(c); return ch_cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__); }
  const int64_t N = c->g.N;
  const int nsb = (int)((N + 1023) / 1024) + 1;
  struct { void** p; size_t b; } allocs[] = {
      {(void**)&c->counts, sizeof(uint32_t) * N},       {(void**)&c->starts, sizeof(uint32_t) * (N + 1)},
      {(void**)&c->starts_next, sizeof(uint32_t) * (N + 1)},
      {(void**)&c->cursor, sizeof(uint32_t) * N},       {(void**)&c->block_sums, sizeof(uint32_t) * nsb},
      {(void**)&c->phi, sizeof(double) * N},            {(void**)&c->mom, sizeof(double) * 4 * N},
      {(void**)&c->rhs, sizeof(double) * N},            {(void**)&c->nfz, sizeof(double) * N},
      {(void**)&c->acc, sizeof(unsigned long long) * 4 * N}, {(void**)&c->cnt, sizeof(DevCounters)},
      {(void**)&c->red, sizeof(double) * 8}};
  for (auto& a : allocs) {
    e = cudaMalloc(a.p, a.b);
    if (e != cudaSuccess) { ch_destroy(c); return ch_cuda_fail(e, "cudaMalloc(grid)", __FILE__, __LINE__); }
  }
  e = c->mixed ? cudaMalloc(&c->E32, sizeof(float4) * N) : cudaMalloc(&c->E64, sizeof(double) * 3 * N);
  if (e != cudaSuccess) { ch_destroy(c); return ch_cuda_fail(e, "cudaMalloc(E)", __FILE__, __LINE__); }
  if (cudaMallocHost(&c->hcnt, sizeof(DevCounters)) != cudaSuccess ||
      cudaMallocHost(&c->hred, sizeof(double) * 8) != cudaSuccess) {
    ch_destroy(c);
    return ch_fail(CH_ERR_NOMEM, "pinned host allocation");
  }
  cudaMemsetAsync(c->phi, 0, sizeof(double) * N, c->stream);
  cudaMemsetAsync(c->acc, 0, sizeof(unsigned long long) * 4 * N, c->stream);
  cudaMemsetAsync(c->mom, 0, sizeof(double) * 4 * N, c->stream);
  rc = c->solver.init(*p, c->g, c->sms);
  if (rc) { ch_destroy(c); return rc; }
  // fixed-point deposit scale 2^s
  // default fixed-point scale: 2^-48 per unit weight keeps the FP64 form's
  // moments within 1e-15 of an FP64 sum (2^40 left 5e-13, which the RHS
  // differences lift to 1.5e-12 in phi) while a node still holds 8192 ion
  // weights and |sum v w| up to 32768; the mixed form's tiles flush at 2^40
  const double s_default = p->precision == CH_MIXED ? 40.0 : 48.0;
  c->dep_scale = ldexp(1.0, (int)(p->deposit_scale_log2 > 0.0 ? p->deposit_scale_log2 : s_default));
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) { ch_destroy(c); return ch_cuda_fail(e, "ch_create", __FILE__, __LINE__); }
  *out = c;
  return CH_OK;
}

static StepConsts consts(const ch_ctx* c, int64_t step) {
  const ch_params& p = c->p;
  StepConsts k;
  memset(&k, 0, sizeof(k));
  k.g = c->g;
  k.tscale = 0.5 * (p.qi / p.mi) * p.dt;
  double tt = 0.0;
  for (int d = 0; d < 3; ++d) { k.t[d] = k.tscale * p.B0[d]; tt += k.t[d] * k.t[d]; }
  for (int d = 0; d < 3; ++d) k.s[d] = 2.0 * k.t[d] / (1.0 + tt);
  for (int d = 0; d < 3; ++d) k.E0[d] = p.E0[d];
  k.push_E0 = p.push_E0;
  k.faithful = p.faithful;
  k.dt = p.dt;
  k.collide = p.mn > 0.0;
  k.vnT = p.vnT;
  for (int d = 0; d < 3; ++d) k.vn0[d] = p.vn0[d];
  k.mi = p.mi;
  k.mn = p.mn;
  k.viTr = sqrt(p.viT[0] * p.viT[0] + p.viT[1] * p.viT[1] + p.viT[2] * p.viT[2]);
  k.m1 = 2.0 * p.vnT * sqrt(2.0 / CH_PI);
  k.nn_profile = p.nn_profile;
  k.nn_center = p.nn_center;
  k.nn_sigma = p.nn_sigma;
  k.nn_floor = p.nn_floor;
  k.seed_lo = (uint32_t)p.seed;
  k.seed_hi = (uint32_t)(p.seed >> 32);
  k.run = p.run;
  k.step = (uint32_t)step;
  k.dep_scale = c->dep_scale;
  ch_consts_finish(k);
  return k;
}

// src/particles.c:510-519
static int64_t collision_count(const ch_params& p, int64_t np) {
  const double viTr = sqrt(p.viT[0] * p.viT[0] + p.viT[1] * p.viT[1] + p.viT[2] * p.viT[2]);
  const double dvx = p.vi0[0] - p.vn0[0], dvy = p.vi0[1] - p.vn0[1], dvz = p.vi0[2] - p.vn0[2];
  const double vrm = 4.0 * viTr + sqrt(dvx * dvx + dvy * dvy + dvz * dvz);
  const double vn0r = sqrt(p.vn0[0] * p.vn0[0] + p.vn0[1] * p.vn0[1] + p.vn0[2] * p.vn0[2]);
  const double den = (p.vnT + vn0r) * sqrt(p.mn / p.mi);
  const double fc = p.nui * p.dt;
  if (!(den > 0.0)) return np;
  const double v = ((double)np * fc * vrm) / den;
  if (v >= (double)np) return np;
  if (v < 0.0) return 0;
  return (int64_t)v;
}

static ch_status ensure_particles(ch_ctx* c, int64_t np) {
  if (np <= 0) return ch_fail(CH_ERR_ARG, "number of ions must be positive");
  if (np > 0xFFFFFFFFll) return ch_fail(CH_ERR_ARG, "at most 2^32-1 ions (32-bit ids)");
  if (c->np == np) return CH_OK;
  free_particles(c);
  cudaError_t e = cudaSuccess;
  if (c->mixed) {
    e = cudaMalloc(&c->M.pos, sizeof(float4) * np);
    if (e == cudaSuccess) e = cudaMalloc(&c->M.vel, sizeof(float4) * np);
    if (e == cudaSuccess) e = cudaMalloc(&c->MQ.pos, sizeof(float4) * np);
    if (e == cudaSuccess) e = cudaMalloc(&c->MQ.vel, sizeof(float4) * np);
    c->M.np = c->MQ.np = np;
  } else {
    double** a[] = {&c->P.x, &c->P.y, &c->P.z, &c->P.vx, &c->P.vy, &c->P.vz,
                    &c->Q.x, &c->Q.y, &c->Q.z, &c->Q.vx, &c->Q.vy, &c->Q.vz};
    for (double** q : a)
      if (e == cudaSuccess) e = cudaMalloc(q, sizeof(double) * np);
    if (e == cudaSuccess) e = cudaMalloc(&c->P.id, sizeof(uint32_t) * np);
    if (e == cudaSuccess) e = cudaMalloc(&c->Q.id, sizeof(uint32_t) * np);
    c->P.np = c->Q.np = np;
  }
  if (e == cudaSuccess) e = cudaMalloc(&c->keys, sizeof(uint32_t) * np);
  if (c->mixed) c->M.rank = c->MQ.rank = c->keys;  // in-cell ranks of the pass before a sort
  const int cap = grid_for(np > c->g.N ? np : c->g.N, 256, c->sms, 8);
  if (e == cudaSuccess) e = cudaMalloc(&c->part, sizeof(double) * 4 * cap);
  if (e != cudaSuccess) {
    free_particles(c);
    return ch_cuda_fail(e, "cudaMalloc(ions)", __FILE__, __LINE__);
  }
  c->part_cap = cap;
  c->np = np;
  return CH_OK;
}

static ch_status ensure_staging(ch_ctx* c) {
  if (c->stage_pos) return CH_OK;
  cudaError_t e = cudaMalloc(&c->stage_pos, sizeof(double4_32a) * c->np);
  if (e == cudaSuccess) e = cudaMalloc(&c->stage_vel, sizeof(double4_32a) * c->np);
  if (e != cudaSuccess) return ch_cuda_fail(e, "cudaMalloc(staging)", __FILE__, __LINE__);
  return CH_OK;
}

static void do_sort(ch_ctx* c) {
  c->slot_map_valid = false;
  prof_begin(c);
  launch_sort(c->mixed, c->g, c->P, c->Q, c->M, c->MQ, c->counts, c->starts, c->cursor, c->keys, c->block_sums,
              c->sms, c->stream);
  prof_end(c, &c->pr.sort_ms, &c->pr.sort_calls);
  std::swap(c->P, c->Q);
  std::swap(c->M, c->MQ);
  c->since_sort = 0;
}

// keep_order: the ions were put back into the slots of the current order,
// whose brick ranges stay valid, so no sort is needed.
static ch_status after_load(ch_ctx* c, bool keep_order = false) {
  if (!keep_order) do_sort(c);
  if (c->p.mn > 0.0) {
    StepConsts k = consts(c, 0);
    const int nb = launch_sbar(c->mixed, k, c->P, c->M, c->part, c->sms, c->stream);
    launch_reduce_partials(c->part, nb, 1, c->red, c->stream);
    CH_CUDA_OK(cudaMemcpyAsync(c->hred, c->red, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  c->sbar = c->p.mn > 0.0 ? c->hred[0] : 0.0;
  c->moments_valid = false;  // phi stays: a host that re-uploads its ions keeps the warm start
  return CH_OK;
}

extern "C" ch_status ch_particles_upload(ch_ctx* c, const ch_real_vector* pos, const ch_real_vector* vel,
                                         int64_t np) {
  if (!c || !pos || !vel) return ch_fail(CH_ERR_ARG, "ch_particles_upload: null argument");
  ch_status rc = ensure_particles(c, np);
  if (rc) return rc;
  const uint64_t bytes = sizeof(double4_32a) * (uint64_t)np;
  const void* dp = device_view(pos, bytes, 16);
  const void* dv = device_view(vel, bytes, 16);
  if (dp && dv && c->mixed && c->slot_map_valid) {
    // registered host arrays in the id order of the last download: every ion
    // goes back into its slot (one pass over the link, no sort)
    launch_host_to_mixed(c->g, dp, dv, c->slot_of_id, c->M, c->sms, c->stream);
    return after_load(c, true);
  }
  if (dp && dv) {
    // registered host arrays: the conversion reads them directly
    launch_aos_in_u16(c->mixed, c->g, dp, dv, c->P, c->M, c->sms, c->stream);
  } else {
    rc = ensure_staging(c);
    if (rc) return rc;
    CH_CUDA_OK(cudaMemcpyAsync(c->stage_pos, pos, bytes, cudaMemcpyHostToDevice, c->stream));
    CH_CUDA_OK(cudaMemcpyAsync(c->stage_vel, vel, bytes, cudaMemcpyHostToDevice, c->stream));
    launch_aos_in(c->mixed, c->g, c->stage_pos, c->stage_vel, c->P, c->M, c->sms, c->stream);
  }
  return after_load(c);
}

extern "C" ch_status ch_particles_load(ch_ctx* c, int64_t np, const ch_loader* L) {
  if (!c || !L) return ch_fail(CH_ERR_ARG, "ch_particles_load: null argument");
  double s = fabs(L->amp[0]) + fabs(L->amp[1]) + fabs(L->amp[2]);
  if (!(s < 1.0)) return ch_fail(CH_ERR_ARG, "density perturbation amplitudes must sum below 1");
  ch_status rc = ensure_particles(c, np);
  if (rc) return rc;
  launch_load(c->mixed, c->g, *L, c->p.seed, c->p.run, c->P, c->M, c->sms, c->stream);
  return after_load(c);
}

extern "C" ch_status ch_particles_load_placed(ch_ctx* c, int64_t np, const ch_loader* L, int32_t density_type) {
  static const char* const names[] = {"flat-sobol", "flat-reverse", "flat-normal", "uniform", "sinusoidal",
                                      "gaussian"};
  if (!c || !L) return ch_fail(CH_ERR_ARG, "ch_particles_load_placed: null argument");
  if (density_type < 0 || density_type > CH_DENSITY_GAUSSIAN)
    return ch_fail(CH_ERR_ARG, "unknown --density-type %d", density_type);
  if (density_type == CH_DENSITY_FLAT_REVERSE || density_type == CH_DENSITY_FLAT_NORMAL ||
      density_type == CH_DENSITY_GAUSSIAN)
    return ch_fail(CH_ERR_UNSUPPORTED, "Not implemented: %s density (src/particles.c:28-45)", names[density_type]);
  if (np < 1) return ch_fail(CH_ERR_ARG, "np < 1");
  if (density_type == CH_DENSITY_UNIFORM && np % c->g.N != 0)
    return ch_fail(CH_ERR_ARG,
                   "uniform placement puts the same number of ions in every cell: np = %lld is not a multiple of "
                   "%lld cells",
                   (long long)np, (long long)c->g.N);
  if (np > (int64_t)UINT32_MAX) return ch_fail(CH_ERR_ARG, "np beyond 32-bit ion ids");
  ch_status rc = ensure_particles(c, np);
  if (rc) return rc;
  launch_load_placed(c->mixed, c->g, *L, density_type, c->p.seed, c->p.run, c->P, c->M, c->sms, c->stream);
  return after_load(c);
}

// Registered host arrays, mixed form: the ions of src (the buffers of the
// current order, or of the order a sort step's deposit has just written),
// converted chunk by chunk into the staging arrays in id order on
// conv_stream, each chunk copied out over the host link on copy_stream while
// the next converts, so the link runs without gaps.  remap rebuilds the
// id -> slot map from src first (after a sort; the map also lets the next
// upload keep the order).  The map and the first chunk are converted on
// c->stream itself, so the link starts at once even when the kernels that
// follow there (a deposit's persistent CTAs) fill the GPU; the other chunks
// convert on conv_stream.  Returns without waiting: the caller
// synchronises copy_stream.
static ch_status download_enqueue(ch_ctx* c, MixParticles src, bool remap, ch_real_vector* pos,
                                  ch_real_vector* vel) {
  if (!c->slot_of_id) {
    CH_CUDA_OK(cudaMalloc(&c->slot_of_id, sizeof(uint32_t) * c->np));
    remap = true;
  }
  ch_status rs = ensure_staging(c);
  if (rs) return rs;
  if (!c->copy_stream) {
    CH_CUDA_OK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    CH_CUDA_OK(cudaStreamCreateWithFlags(&c->conv_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : c->chunk_ev) CH_CUDA_OK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  if (remap) launch_slot_map(src, c->slot_of_id, c->sms, c->stream);
  const int64_t chunks = 8, per = ((c->np + chunks - 1) / chunks + 31) / 32 * 32;
  int k = 0;
  for (int64_t a = 0; a < c->np; a += per, ++k) {
    const int64_t b = a + per < c->np ? a + per : c->np;
    cudaStream_t cs = k == 0 ? c->stream : c->conv_stream;
    launch_mixed_to_host(c->g, src, c->slot_of_id, c->stage_pos, c->stage_vel, a, b, c->sms, cs);
    CH_CUDA_OK(cudaEventRecord(c->chunk_ev[k], cs));
    if (k == 0) CH_CUDA_OK(cudaStreamWaitEvent(c->conv_stream, c->chunk_ev[0], 0));
    CH_CUDA_OK(cudaStreamWaitEvent(c->copy_stream, c->chunk_ev[k], 0));
    const size_t off = sizeof(double4_32a) * (size_t)a, len = sizeof(double4_32a) * (size_t)(b - a);
    CH_CUDA_OK(cudaMemcpyAsync(reinterpret_cast<char*>(pos) + off, reinterpret_cast<char*>(c->stage_pos) + off, len,
                               cudaMemcpyDeviceToHost, c->copy_stream));
    CH_CUDA_OK(cudaMemcpyAsync(reinterpret_cast<char*>(vel) + off, reinterpret_cast<char*>(c->stage_vel) + off, len,
                               cudaMemcpyDeviceToHost, c->copy_stream));
  }
  return CH_OK;
}

extern "C" ch_status ch_particles_download(ch_ctx* c, ch_real_vector* pos, ch_real_vector* vel) {
  if (!c || !pos || !vel) return ch_fail(CH_ERR_ARG, "ch_particles_download: null argument");
  if (c->np == 0) return ch_fail(CH_ERR_STATE, "no ions");
  const uint64_t bytes = sizeof(double4_32a) * (uint64_t)c->np;
  void* dp = device_view(pos, bytes, 16);
  void* dv = device_view(vel, bytes, 16);
  if (dp && dv && c->mixed) {
    ch_status rs = download_enqueue(c, c->M, !c->slot_map_valid, pos, vel);
    if (rs) return rs;
    CH_CUDA_OK(cudaStreamSynchronize(c->copy_stream));
    c->slot_map_valid = true;
    return CH_OK;
  }
  ch_status rc = ensure_staging(c);
  if (rc) return rc;
  launch_aos_out(c->mixed, c->g, c->P, c->M, c->stage_pos, c->stage_vel, c->sms, c->stream);
  if (dp && dv) {
    // registered host arrays: a copy kernel streams the staging out
    launch_stream_copy(dp, c->stage_pos, bytes, c->sms, c->stream);
    launch_stream_copy(dv, c->stage_vel, bytes, c->sms, c->stream);
  } else {
    CH_CUDA_OK(cudaMemcpyAsync(pos, c->stage_pos, bytes, cudaMemcpyDeviceToHost, c->stream));
    CH_CUDA_OK(cudaMemcpyAsync(vel, c->stage_vel, bytes, cudaMemcpyDeviceToHost, c->stream));
  }
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  return CH_OK;
}

// ------------------------------------------------------------------ phases
static ch_status run_pass(ch_ctx* c, int phases, int64_t step, ch_step_info* info, bool count_cells = false) {
  StepConsts k = consts(c, step);
  const bool push = (phases & PH_PUSH) != 0;
  int64_t Nc = 0;
  if (push) {
    launch_node_efield(c->mixed, c->g, k.tscale, c->phi, c->E64, c->E32, c->sms, c->stream);
    CH_CUDA_OK(cudaMemsetAsync(c->cnt, 0, sizeof(DevCounters), c->stream));
    if (k.collide) Nc = collision_count(c->p, c->np);
  }
  if (phases & PH_DEPOSIT) CH_CUDA_OK(cudaMemsetAsync(&c->cnt->range_error, 0, sizeof(int), c->stream));
  prof_begin(c);
  uint32_t* hist = nullptr;
  if (count_cells && c->mixed) {
    CH_CUDA_OK(cudaMemsetAsync(c->counts, 0, sizeof(uint32_t) * c->g.N, c->stream));
    hist = c->counts;
  }
  const int nb = launch_pass(c->mixed, phases, k, c->P, c->M, c->E64, c->E32, c->phi, c->acc, (double)Nc, c->sbar,
                             c->cnt, c->part, c->starts, hist, c->sms, c->stream);
  if (phases == PH_DEPOSIT)
    prof_end(c, &c->pr.pass_ms, &c->pr.pass_calls, &c->pr.deposit_ms, &c->pr.deposit_calls);
  else
    prof_end(c, &c->pr.pass_ms, &c->pr.pass_calls);
  if (push) {
    launch_reduce_partials(c->part, nb, 2, c->red, c->stream);
    CH_CUDA_OK(cudaMemcpyAsync(c->hred, c->red, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
    CH_CUDA_OK(cudaMemcpyAsync(c->hcnt, c->cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, c->stream));
    CH_CUDA_OK(cudaStreamSynchronize(c->stream));
    if (k.collide) c->sbar = c->hred[1];
    if (info) {
      info->Nc = Nc;
      info->collisions = (int64_t)c->hcnt->collisions;
      info->refused = (int64_t)c->hcnt->refused;
      info->expected = c->hred[0];
    }
    if (c->hcnt->refused >= 10)
      return ch_fail(CH_ERR_COLLISION_LIMIT, "%llu collisions refused in step %lld (src/particles.c:603-605)",
                     (unsigned long long)c->hcnt->refused, (long long)step);
  }
  if (phases & PH_MOVE) c->since_sort++;
  return CH_OK;
}

static ch_status finalize_moments(ch_ctx* c, ch_step_info* info) {
  const int reset = (c->p.faithful & CH_FAITHFUL_D6) ? 0 : 1;
  prof_begin(c);
  const int nb = launch_finalize(c->g.N, c->acc, 1.0 / c->dep_scale, reset, c->mom, c->part, c->cnt, c->sms,
                                 c->stream);
  prof_end(c, &c->pr.moments_ms, &c->pr.moments_calls);
  launch_reduce_partials(c->part, nb, 4, c->red + 4, c->stream);
  CH_CUDA_OK(cudaMemcpyAsync(c->hred + 4, c->red + 4, sizeof(double) * 4, cudaMemcpyDeviceToHost, c->stream));
  CH_CUDA_OK(cudaMemcpyAsync(&c->hcnt->range_error, &c->cnt->range_error, sizeof(int), cudaMemcpyDeviceToHost,
                             c->stream));
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  c->moments_valid = true;
  if (info)
    for (int q = 0; q < 4; ++q) info->moment_sum[q] = c->hred[4 + q];
  if (c->hcnt->range_error & 2) return ch_fail(CH_ERR_NAN, "non-finite ion position or velocity");
  if (c->hcnt->range_error)
    return ch_fail(CH_ERR_RANGE, "deposit exceeded the fixed-point range 2^%d; lower deposit_scale_log2",
                   63 - (int)log2(c->dep_scale));
  for (int q = 0; q < 4; ++q)
    if (!isfinite(c->hred[4 + q])) return ch_fail(CH_ERR_NAN, "non-finite moment sum");
  return CH_OK;
}

extern "C" ch_status ch_update_velocities(ch_ctx* c, int64_t step, ch_step_info* info) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  if (c->np == 0) return ch_fail(CH_ERR_STATE, "no ions");
  return run_pass(c, PH_PUSH, step, info);
}

extern "C" ch_status ch_update_positions(ch_ctx* c) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  if (c->np == 0) return ch_fail(CH_ERR_STATE, "no ions");
  ch_status rc = run_pass(c, PH_MOVE, 0, nullptr);
  if (rc) return rc;
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  return CH_OK;
}

static ch_status copy_moments_out(ch_ctx* c, ch_grid_node* host_out) {
  // SoA device -> interleaved GridNode on the host
  const int64_t N = c->g.N;
  CH_CUDA_OK(cudaMemcpy2DAsync(host_out, sizeof(ch_grid_node), c->mom, sizeof(double), sizeof(double), N,
                               cudaMemcpyDeviceToHost, c->stream));
  for (int q = 1; q < 4; ++q)
    CH_CUDA_OK(cudaMemcpy2DAsync((char*)host_out + q * sizeof(double), sizeof(ch_grid_node), c->mom + q * N,
                                 sizeof(double), sizeof(double), N, cudaMemcpyDeviceToHost, c->stream));
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  return CH_OK;
}

extern "C" ch_status ch_collect_moments(ch_ctx* c, ch_grid_node* host_out, ch_step_info* info) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  if (c->np == 0) return ch_fail(CH_ERR_STATE, "no ions");
  ch_status rc = run_pass(c, PH_DEPOSIT, 0, nullptr);
  if (rc) return rc;
  rc = finalize_moments(c, info);
  if (rc) return rc;
  if (host_out) return copy_moments_out(c, host_out);
  return CH_OK;
}

// CG needs a symmetric operator.  With kappa_e != 0 the full operator's
// tensor R = I + kk^T + [k]x has an antisymmetric part (src/lhs.c:412-420),
// so only BiCGStab applies.
static bool cg_unsound(const ch_params& p) {
  return p.ksp_type == CH_KSP_CG && p.lhs_type == CH_LHS_FULL &&
         (p.kappa_e[0] != 0.0 || p.kappa_e[1] != 0.0 || p.kappa_e[2] != 0.0);
}

static ch_status potential(ch_ctx* c, ch_solve_info* info) {
  if (!c->moments_valid) return ch_fail(CH_ERR_STATE, "no moments: call ch_collect_moments first");
  if (cg_unsound(c->p))
    return ch_fail(CH_ERR_UNSUPPORTED,
                   "-ksp_type cg with kappa_e = (%g, %g, %g): the full operator is not symmetric "
                   "(src/lhs.c:412-420); use -ksp_type bcgs",
                   c->p.kappa_e[0], c->p.kappa_e[1], c->p.kappa_e[2]);
  const int64_t N = c->g.N;
  prof_begin(c);
  c->solver.build_rhs(c->mom, c->rhs, c->stream);
  const double* n = c->mom;
  if (c->p.faithful & CH_FAITHFUL_D7) {
    if (!c->solved_once) CH_CUDA_OK(cudaMemcpyAsync(c->nfz, c->mom, sizeof(double) * N, cudaMemcpyDeviceToDevice,
                                                    c->stream));
    n = c->nfz;
  }
  if (!c->solved_once) CH_CUDA_OK(cudaMemsetAsync(c->phi, 0, sizeof(double) * N, c->stream));  // ComputeInitialPhi
  SolveStats st{};
  ch_status rc = c->solver.solve(n, c->rhs, c->phi, &st, c->stream);
  prof_end(c, &c->pr.solve_ms, &c->pr.solve_calls);
  c->solved_once = true;
  if (info) {
    info->iterations = st.iterations;
    info->refinements = st.refinements;
    info->rnorm = st.rnorm;
    info->bnorm = st.bnorm;
  }
  if (rc == CH_ERR_NOT_CONVERGED)
    return ch_fail(rc, "potential solve: ||r|| = %.3e > rtol ||b|| = %.3e after %d iterations", st.rnorm,
                   c->p.ksp_rtol * st.bnorm, st.iterations);
  if (rc) return rc;
  if (!isfinite(st.rnorm)) return ch_fail(CH_ERR_NAN, "non-finite potential residual");
  return CH_OK;
}

extern "C" ch_status ch_set_solver(ch_ctx* c, int32_t ksp_type, int32_t pc_type, double rtol, double atol,
                                   int32_t max_it) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  if (ksp_type != CH_KSP_CG && ksp_type != CH_KSP_BCGS) return ch_fail(CH_ERR_ARG, "unknown ksp_type %d", ksp_type);
  if (pc_type != CH_PC_NONE && pc_type != CH_PC_JACOBI && pc_type != CH_PC_MG)
    return ch_fail(CH_ERR_ARG, "unknown pc_type %d", pc_type);
  if (!(rtol > 0.0) || !(atol >= 0.0) || max_it < 1)
    return ch_fail(CH_ERR_ARG, "bad ksp tolerances: rtol %g, atol %g, max_it %d", rtol, atol, max_it);
  c->p.ksp_type = ksp_type;
  c->p.pc_type = pc_type;
  c->p.ksp_rtol = rtol;
  c->p.ksp_atol = atol;
  c->p.ksp_max_it = max_it;
  c->solver.set_options(ksp_type, pc_type, rtol, atol, max_it);
  return CH_OK;
}

extern "C" ch_status ch_compute_potential(ch_ctx* c, double* phi_out, ch_solve_info* info) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  ch_status rc = potential(c, info);
  if (rc) return rc;
  if (phi_out) {
    CH_CUDA_OK(cudaMemcpyAsync(phi_out, c->phi, sizeof(double) * c->g.N, cudaMemcpyDeviceToHost, c->stream));
    CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  }
  return CH_OK;
}

// Scan of the push's cell count into starts_next, then the deposit fused
// with the scatter of M into MQ in that order (mixed form).
static ch_status run_deposit_sort(ch_ctx* c) {
  StepConsts k = consts(c, 0);
  CH_CUDA_OK(cudaMemsetAsync(&c->cnt->range_error, 0, sizeof(int), c->stream));
  prof_begin(c);
  launch_scan(c->g.N, c->counts, c->starts_next, c->cursor, c->block_sums, c->stream);
  prof_end(c, &c->pr.sort_ms, &c->pr.sort_calls);
  prof_begin(c);
  launch_deposit_sort(k, c->M, c->MQ, c->starts, c->starts_next, c->acc, c->cnt, c->sms, c->stream);
  prof_end(c, &c->pr.pass_ms, &c->pr.pass_calls, &c->pr.deposit_ms, &c->pr.deposit_calls);
  return CH_OK;
}

// nsteps steps.  With dpos / dvel (registered host arrays, mixed form) the
// last step also downloads its ions: they are final once the push has moved
// them, so the download starts then and overlaps the deposit and the
// potential solve; on a sort step it starts after the deposit, from the new
// order, so the id -> slot map stays valid for the next upload.
static ch_status run_steps(ch_ctx* c, int64_t first_step, int32_t nsteps, ch_step_info* info,
                           ch_real_vector* dpos = nullptr, ch_real_vector* dvel = nullptr) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  if (c->np == 0) return ch_fail(CH_ERR_STATE, "no ions");
  if (!c->solved_once) return ch_fail(CH_ERR_STATE, "initial potential not computed");
  if (nsteps < 0) return ch_fail(CH_ERR_ARG, "nsteps < 0");
  ch_step_info local;
  for (int32_t s = 0; s < nsteps; ++s) {
    memset(&local, 0, sizeof(local));
    const bool sort_due = c->p.sort_period > 0 && c->since_sort + 1 >= c->p.sort_period;
    const bool download = dpos && s + 1 == nsteps;
    // Two launches: push + collide + move (with the new-cell histogram when
    // a sort is due) at 4 CTAs per SM in a small shared footprint, then the
    // deposit.  The pair is faster than one fused launch, whose shared
    // memory and registers allow only 2 CTAs per SM; the results are the
    // same bit for bit.
    ch_status rc = run_pass(c, PH_PUSH | PH_MOVE, first_step + s, &local, sort_due);
    if (!rc && download && !sort_due) rc = download_enqueue(c, c->M, !c->slot_map_valid, dpos, dvel);
    // Mixed form, sort due: the push counted every ion's new cell and rank;
    // the scan gives the new order, and the deposit, which reads every ion
    // anyway, also writes it there (the counting sort's scatter).
    const bool fused_sort = sort_due && c->mixed;
    if (!rc && fused_sort) rc = run_deposit_sort(c);
    else if (!rc) rc = run_pass(c, PH_DEPOSIT, 0, nullptr);
    if (!rc && download && fused_sort) rc = download_enqueue(c, c->MQ, true, dpos, dvel);
    if (rc) return rc;
    rc = finalize_moments(c, &local);
    if (rc) return rc;
    rc = potential(c, &local.solve);
    if (rc) return rc;
    if (fused_sort) {
      std::swap(c->M, c->MQ);
      std::swap(c->starts, c->starts_next);
      c->since_sort = 0;
      c->slot_map_valid = false;
    } else if (sort_due) {
      do_sort(c);  // FP64 form (the mixed form sorts inside its deposit)
    }
  }
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  prof_flush(c);  // the events have completed
  if (dpos) {
    CH_CUDA_OK(cudaStreamSynchronize(c->copy_stream));
    c->slot_map_valid = true;  // rebuilt from the order the ions now have, or still valid
  }
  if (info) *info = local;
  return CH_OK;
}

// The push launch of a step of ch_step_host whose ions the host holds
// (registered arrays, mixed form, ions in the id order of the last
// transfer): k_host_push reads them (read) and/or writes the step's result
// back (write) over the host link while it pushes, both directions at once.
// It uses S of the previous step.  When the ions it read give another S (the
// host changed velocities since the last transfer), it puts the uploaded ions
// back into M, takes their S and sets *redo: the caller then runs the push
// the ordinary way.
static ch_status run_host_push(ch_ctx* c, int64_t step, ch_step_info* info, bool count_cells, bool read, bool write,
                               void* dp, void* dv, bool* redo) {
  *redo = false;
  StepConsts k = consts(c, step);
  launch_node_efield(true, c->g, k.tscale, c->phi, c->E64, c->E32, c->sms, c->stream);
  CH_CUDA_OK(cudaMemsetAsync(c->cnt, 0, sizeof(DevCounters), c->stream));
  const int64_t Nc = k.collide ? collision_count(c->p, c->np) : 0;
  if (read && !c->HB.pos) {
    CH_CUDA_OK(cudaMalloc(&c->HB.pos, sizeof(float4) * c->np));
    CH_CUDA_OK(cudaMalloc(&c->HB.vel, sizeof(float4) * c->np));
    c->HB.np = c->np;
  }
  if (!read && !c->slot_map_valid) {  // a sort earlier in the call changed the order
    launch_slot_map(c->M, c->slot_of_id, c->sms, c->stream);
    c->slot_map_valid = true;
  }
  uint32_t* hist = nullptr;
  if (count_cells) {
    CH_CUDA_OK(cudaMemsetAsync(c->counts, 0, sizeof(uint32_t) * c->g.N, c->stream));
    hist = c->counts;
  }
  prof_begin(c);
  const int nb = launch_host_push(k, dp, dv, c->slot_of_id, c->M, c->HB, c->E32, (double)Nc, c->sbar, hist, read,
                                  write, c->cnt, c->part, c->sms, c->stream);
  prof_end(c, &c->pr.pass_ms, &c->pr.pass_calls);
  launch_reduce_partials(c->part, nb, 3, c->red, c->stream);
  CH_CUDA_OK(cudaMemcpyAsync(c->hred, c->red, sizeof(double) * 3, cudaMemcpyDeviceToHost, c->stream));
  CH_CUDA_OK(cudaMemcpyAsync(c->hcnt, c->cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, c->stream));
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  c->pr.host_push_calls++;
  if (read && k.collide && c->hred[2] != c->sbar) {
    c->pr.host_push_reruns++;
    CH_CUDA_OK(cudaMemcpyAsync(c->M.pos, c->HB.pos, sizeof(float4) * c->np, cudaMemcpyDeviceToDevice, c->stream));
    CH_CUDA_OK(cudaMemcpyAsync(c->M.vel, c->HB.vel, sizeof(float4) * c->np, cudaMemcpyDeviceToDevice, c->stream));
    c->sbar = c->hred[2];
    *redo = true;
    return CH_OK;
  }
  if (k.collide) c->sbar = c->hred[1];
  if (info) {
    info->Nc = Nc;
    info->collisions = (int64_t)c->hcnt->collisions;
    info->refused = (int64_t)c->hcnt->refused;
    info->expected = c->hred[0];
  }
  if (k.collide && c->hcnt->refused >= 10)
    return ch_fail(CH_ERR_COLLISION_LIMIT, "%llu collisions refused in step %lld (src/particles.c:603-605)",
                   (unsigned long long)c->hcnt->refused, (long long)step);
  c->since_sort++;
  return CH_OK;
}

// ch_step_host's steps when the ions the host holds are in the id order of
// the last transfer through registered arrays (mixed form): the first step's
// push reads them straight from the host arrays and the last step's push
// writes the result back, so the upload and the download share the link
// instead of following each other.
static ch_status run_steps_host(ch_ctx* c, int64_t first_step, int32_t nsteps, ch_step_info* info, void* dp,
                                void* dv, ch_real_vector* pos, ch_real_vector* vel) {
  ch_step_info local;
  bool enqueued = false;
  for (int32_t s = 0; s < nsteps; ++s) {
    memset(&local, 0, sizeof(local));
    const bool sort_due = c->p.sort_period > 0 && c->since_sort + 1 >= c->p.sort_period;
    const bool read = s == 0, write = s + 1 == nsteps;
    bool redo = false, written = false;
    ch_status rc = CH_OK;
    if (read || write) {
      rc = run_host_push(c, first_step + s, &local, sort_due, read, write, dp, dv, &redo);
      written = write && !redo;
    }
    if (!rc && ((!read && !write) || redo)) rc = run_pass(c, PH_PUSH | PH_MOVE, first_step + s, &local, sort_due);
    const bool download = write && !written;
    if (!rc && download && !sort_due) {
      rc = download_enqueue(c, c->M, !c->slot_map_valid, pos, vel);
      enqueued = true;
    }
    if (!rc && sort_due) rc = run_deposit_sort(c);
    else if (!rc) rc = run_pass(c, PH_DEPOSIT, 0, nullptr);
    if (!rc && download && sort_due) {
      rc = download_enqueue(c, c->MQ, true, pos, vel);
      enqueued = true;
    }
    if (rc) return rc;
    rc = finalize_moments(c, &local);
    if (rc) return rc;
    rc = potential(c, &local.solve);
    if (rc) return rc;
    if (sort_due) {
      std::swap(c->M, c->MQ);
      std::swap(c->starts, c->starts_next);
      c->since_sort = 0;
      c->slot_map_valid = false;
    }
  }
  if (enqueued) {
    CH_CUDA_OK(cudaStreamSynchronize(c->copy_stream));
    c->slot_map_valid = true;  // download_enqueue rebuilt it from the current order
  } else if (!c->slot_map_valid) {
    launch_slot_map(c->M, c->slot_of_id, c->sms, c->stream);
    c->slot_map_valid = true;
  }
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  prof_flush(c);
  if (info) *info = local;
  return CH_OK;
}

extern "C" ch_status ch_step(ch_ctx* c, int64_t first_step, int32_t nsteps, ch_step_info* info) {
  return run_steps(c, first_step, nsteps, info);
}

extern "C" ch_status ch_step_host(ch_ctx* c, int64_t first_step, int32_t nsteps, ch_real_vector* pos,
                                  ch_real_vector* vel, ch_step_info* info) {
  if (!c || !pos || !vel) return ch_fail(CH_ERR_ARG, "ch_step_host: null argument");
  if (c->np == 0) return ch_fail(CH_ERR_STATE, "no ions");
  if (nsteps < 1) return ch_fail(CH_ERR_ARG, "nsteps < 1");
  const uint64_t bytes = sizeof(double4_32a) * (uint64_t)c->np;
  if (c->mixed && c->slot_map_valid && c->solved_once) {
    void* dp = device_view(pos, bytes, 16);
    void* dv = device_view(vel, bytes, 16);
    if (dp && dv) {
      ch_status rh = run_steps_host(c, first_step, nsteps, info, dp, dv, pos, vel);
      if (rh && c->copy_stream) cudaStreamSynchronize(c->copy_stream);
      return rh;
    }
  }
  ch_status rc = ch_particles_upload(c, pos, vel, c->np);
  if (rc) return rc;
  const bool overlap = c->mixed && device_view(pos, bytes, 16) && device_view(vel, bytes, 16);
  if (!overlap) {
    rc = run_steps(c, first_step, nsteps, info);
    return rc ? rc : ch_particles_download(c, pos, vel);
  }
  rc = run_steps(c, first_step, nsteps, info, pos, vel);
  if (rc && c->copy_stream) cudaStreamSynchronize(c->copy_stream);  // no copy left running on failure
  return rc;
}

extern "C" ch_status ch_set_moments(ch_ctx* c, const ch_grid_node* in) {
  if (!c || !in) return ch_fail(CH_ERR_ARG, "null argument");
  const int64_t N = c->g.N;
  for (int q = 0; q < 4; ++q)
    CH_CUDA_OK(cudaMemcpy2DAsync(c->mom + q * N, sizeof(double), (const char*)in + q * sizeof(double),
                                 sizeof(ch_grid_node), sizeof(double), N, cudaMemcpyHostToDevice, c->stream));
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  c->moments_valid = true;
  return CH_OK;
}

extern "C" ch_status ch_get_phi(ch_ctx* c, double* out) {
  if (!c || !out) return ch_fail(CH_ERR_ARG, "null argument");
  CH_CUDA_OK(cudaMemcpyAsync(out, c->phi, sizeof(double) * c->g.N, cudaMemcpyDeviceToHost, c->stream));
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  return CH_OK;
}

extern "C" ch_status ch_set_phi(ch_ctx* c, const double* in) {
  if (!c || !in) return ch_fail(CH_ERR_ARG, "null argument");
  CH_CUDA_OK(cudaMemcpyAsync(c->phi, in, sizeof(double) * c->g.N, cudaMemcpyHostToDevice, c->stream));
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  c->solved_once = true;
  return CH_OK;
}

extern "C" ch_status ch_get_rhs(ch_ctx* c, double* out) {
  if (!c || !out) return ch_fail(CH_ERR_ARG, "null argument");
  if (!c->moments_valid) return ch_fail(CH_ERR_STATE, "no moments");
  c->solver.build_rhs(c->mom, c->rhs, c->stream);
  CH_CUDA_OK(cudaMemcpyAsync(out, c->rhs, sizeof(double) * c->g.N, cudaMemcpyDeviceToHost, c->stream));
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  return CH_OK;
}

extern "C" ch_status ch_apply_operator(ch_ctx* c, const double* x, double* y) {
  if (!c || !x || !y) return ch_fail(CH_ERR_ARG, "null argument");
  if (!c->moments_valid) return ch_fail(CH_ERR_STATE, "no moments");
  const int64_t N = c->g.N;
  double* dx = c->rhs;  // scratch: the next RHS build overwrites it
  double* dy = c->nfz;
  if (c->p.faithful & CH_FAITHFUL_D7) return ch_fail(CH_ERR_UNSUPPORTED, "apply with a frozen operator");
  CH_CUDA_OK(cudaMemcpyAsync(dx, x, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
  c->solver.apply64(c->mom, dx, dy, c->stream);
  CH_CUDA_OK(cudaMemcpyAsync(y, dy, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
  CH_CUDA_OK(cudaStreamSynchronize(c->stream));
  return CH_OK;
}

extern "C" ch_status ch_host_register(void* ptr, uint64_t bytes) {
  if (!ptr || !bytes) return ch_fail(CH_ERR_ARG, "null argument");
  CH_CUDA_OK(cudaHostRegister(ptr, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable));
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, ptr, 0) != cudaSuccess) {
    cudaGetLastError();
    d = nullptr;
  }
  std::lock_guard<std::mutex> lk(g_hr_mu);
  g_hr.push_back(HostRange{static_cast<char*>(ptr), bytes, static_cast<char*>(d)});
  return CH_OK;
}

extern "C" ch_status ch_host_unregister(void* ptr) {
  if (!ptr) return ch_fail(CH_ERR_ARG, "null argument");
  {
    std::lock_guard<std::mutex> lk(g_hr_mu);
    for (size_t i = 0; i < g_hr.size(); ++i)
      if (g_hr[i].p == ptr) {
        g_hr.erase(g_hr.begin() + (long)i);
        break;
      }
  }
  CH_CUDA_OK(cudaHostUnregister(ptr));
  return CH_OK;
}

// Allocations of ch_host_alloc: anonymous mappings backed by transparent
// huge pages where the kernel offers them, page-locked and mapped for the
// GPU.  The GPU reads and writes host memory through its own page tables;
// a range of huge pages keeps them few and contiguous, so the link runs at
// its full rate however fragmented free memory has become (registered base
// pages of an ordinary allocation, scattered after heavy allocation churn,
// were measured 10 to 30 times slower).
struct HostAlloc {
  char* p;
  uint64_t n;
};
static std::vector<HostAlloc> g_ha;

extern "C" ch_status ch_host_alloc(uint64_t bytes, void** out) {
  if (!out || !bytes) return ch_fail(CH_ERR_ARG, "null argument");
  *out = nullptr;
  void* p = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (p == MAP_FAILED)
    return ch_fail(CH_ERR_NOMEM, "ch_host_alloc: mmap of %llu bytes failed", (unsigned long long)bytes);
#ifdef MADV_HUGEPAGE
  madvise(p, bytes, MADV_HUGEPAGE);  // advisory: base pages where huge ones are not offered
#endif
  // touch every page now, so that the pinning below finds them in place
  const long pg = sysconf(_SC_PAGESIZE) > 0 ? sysconf(_SC_PAGESIZE) : 4096;
  for (uint64_t o = 0; o < bytes; o += (uint64_t)pg) static_cast<volatile char*>(p)[o] = 0;
  cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable);
  void* d = nullptr;
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(&d, p, 0);
  if (e != cudaSuccess) {
    cudaHostUnregister(p);
    cudaGetLastError();
    munmap(p, bytes);
    return ch_cuda_fail(e, "ch_host_alloc: cudaHostRegister", __FILE__, __LINE__);
  }
  std::lock_guard<std::mutex> lk(g_hr_mu);
  g_hr.push_back(HostRange{static_cast<char*>(p), bytes, static_cast<char*>(d)});
  g_ha.push_back(HostAlloc{static_cast<char*>(p), bytes});
  *out = p;
  return CH_OK;
}

extern "C" ch_status ch_host_free(void* ptr) {
  if (!ptr) return CH_OK;
  uint64_t n = 0;
  {
    std::lock_guard<std::mutex> lk(g_hr_mu);
    for (size_t i = 0; i < g_ha.size(); ++i)
      if (g_ha[i].p == ptr) {
        n = g_ha[i].n;
        g_ha.erase(g_ha.begin() + (long)i);
        break;
      }
    if (!n) return ch_fail(CH_ERR_ARG, "ch_host_free: not an allocation of ch_host_alloc");
    for (size_t i = 0; i < g_hr.size(); ++i)
      if (g_hr[i].p == ptr) {
        g_hr.erase(g_hr.begin() + (long)i);
        break;
      }
  }
  CH_CUDA_OK(cudaHostUnregister(ptr));
  munmap(ptr, n);
  return CH_OK;
}

extern "C" ch_status ch_set_profiling(ch_ctx* c, int32_t enable) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  if (!enable) prof_flush(c);
  c->prof = enable != 0;
  return CH_OK;
}

extern "C" ch_status ch_get_profile(ch_ctx* c, ch_profile* out) {
  if (!c || !out) return ch_fail(CH_ERR_ARG, "null argument");
  prof_flush(c);
  *out = c->pr;
  out->launches = (int64_t)g_launches.load();
  return CH_OK;
}

extern "C" ch_status ch_reset_profile(ch_ctx* c) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  prof_flush(c);
  c->pr = ch_profile{};
  return CH_OK;
}

extern "C" ch_status ch_get_stream(ch_ctx* c, void** stream) {
  if (!c || !stream) return ch_fail(CH_ERR_ARG, "null argument");
  *stream = (void*)c->stream;
  return CH_OK;
}

// ------------------------------------------------------------------ output
// OutputHDF5 (src/fileio.c:73-126) without HDF5: the fields of one step --
// density, x/y/z flux, rhs, potential, in the reference's dataset names --
// are snapshot on the device, copied to pinned host memory on a second
// stream while the next step runs, and written by a host thread as raw
// little-endian FP64 files (DMDA natural order) with a JSON manifest.
namespace {
constexpr int OUT_SLOTS = 2;
constexpr int OUT_FIELDS = 6;
const char* const OUT_NAMES[OUT_FIELDS] = {"density", "x flux", "y flux", "z flux", "rhs", "potential"};
const char* const OUT_FILES[OUT_FIELDS] = {"density", "x_flux", "y_flux", "z_flux", "rhs", "potential"};
}  // namespace

struct ChOutput {
  std::string stem;
  int device = 0;
  GridDesc g{};
  ch_params p{};
  cudaStream_t stream = nullptr;
  double* dev[OUT_SLOTS] = {nullptr, nullptr};
  double* host[OUT_SLOTS] = {nullptr, nullptr};
  cudaEvent_t snap[OUT_SLOTS] = {nullptr, nullptr};
  cudaEvent_t ready[OUT_SLOTS] = {nullptr, nullptr};
  bool busy[OUT_SLOTS] = {false, false};
  int next = 0;
  std::thread writer;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::pair<int, std::string>> jobs;
  bool stop = false;
  std::string error;
  int64_t written = 0;
};

static void output_write(ChOutput* o, int slot, const std::string& insert) {
  const int64_t N = o->g.N;
  const std::string base = o->stem + insert;
  std::string err;
  for (int f = 0; f < OUT_FIELDS && err.empty(); ++f) {
    const std::string name = base + "." + OUT_FILES[f] + ".f64";
    FILE* fp = fopen(name.c_str(), "wb");
    if (!fp) { err = "cannot open " + name; break; }
    if (fwrite(o->host[slot] + (size_t)f * N, sizeof(double), (size_t)N, fp) != (size_t)N) err = "short write " + name;
    if (fclose(fp) != 0 && err.empty()) err = "close " + name;
  }
  if (err.empty()) {
    const std::string name = base + ".json";
    FILE* fp = fopen(name.c_str(), "w");
    if (!fp) {
      err = "cannot open " + name;
    } else {
      fprintf(fp, "{\n  \"format\": \"raw little-endian float64, DMDA natural order (x fastest)\",\n");
      fprintf(fp, "  \"grid\": {\"Nx\": %d, \"Ny\": %d, \"Nz\": %d, \"x0\": %.17g, \"x1\": %.17g, "
                  "\"y0\": %.17g, \"y1\": %.17g, \"z0\": %.17g, \"z1\": %.17g},\n",
              o->g.Nx, o->g.Ny, o->g.Nz, o->p.x0, o->p.x1, o->p.y0, o->p.y1, o->p.z0, o->p.z1);
      fprintf(fp, "  \"datasets\": {");
      for (int f = 0; f < OUT_FIELDS; ++f) {
        const std::string file = base + "." + OUT_FILES[f] + ".f64";
        const size_t cut = file.find_last_of('/');
        fprintf(fp, "%s\n    \"%s\": \"%s\"", f ? "," : "", OUT_NAMES[f],
                (cut == std::string::npos ? file : file.substr(cut + 1)).c_str());
      }
      fprintf(fp, "\n  }\n}\n");
      if (fclose(fp) != 0) err = "close " + name;
    }
  }
  std::lock_guard<std::mutex> lk(o->mu);
  if (!err.empty() && o->error.empty()) o->error = err;
  if (err.empty()) o->written++;
}

static void output_thread(ChOutput* o) {
  cudaSetDevice(o->device);
  for (;;) {
    std::pair<int, std::string> job;
    {
      std::unique_lock<std::mutex> lk(o->mu);
      o->cv.wait(lk, [&] { return o->stop || !o->jobs.empty(); });
      if (o->jobs.empty()) return;
      job = o->jobs.front();
      o->jobs.pop_front();
    }
    const cudaError_t e = cudaEventSynchronize(o->ready[job.first]);
    if (e != cudaSuccess) {
      std::lock_guard<std::mutex> lk(o->mu);
      if (o->error.empty()) o->error = std::string("output copy: ") + cudaGetErrorString(e);
    } else {
      output_write(o, job.first, job.second);
    }
    {
      std::lock_guard<std::mutex> lk(o->mu);
      o->busy[job.first] = false;
    }
    o->cv.notify_all();
  }
}

static void output_close(ch_ctx* c) {
  ChOutput* o = c->out;
  if (!o) return;
  {
    std::lock_guard<std::mutex> lk(o->mu);
    o->stop = true;
  }
  o->cv.notify_all();
  if (o->writer.joinable()) o->writer.join();
  for (int k = 0; k < OUT_SLOTS; ++k) {
    if (o->dev[k]) cudaFree(o->dev[k]);
    if (o->host[k]) cudaFreeHost(o->host[k]);
    if (o->snap[k]) cudaEventDestroy(o->snap[k]);
    if (o->ready[k]) cudaEventDestroy(o->ready[k]);
  }
  if (o->stream) cudaStreamDestroy(o->stream);
  delete o;
  c->out = nullptr;
}

extern "C" ch_status ch_output_open(ch_ctx* c, const char* stem) {
  if (!c || !stem) return ch_fail(CH_ERR_ARG, "null argument");
  output_close(c);
  ChOutput* o = new (std::nothrow) ChOutput();
  if (!o) return ch_fail(CH_ERR_NOMEM, "host allocation");
  o->stem = stem;
  o->device = c->device;
  o->g = c->g;
  o->p = c->p;
  c->out = o;
  const size_t b = sizeof(double) * OUT_FIELDS * (size_t)c->g.N;
  cudaError_t e = cudaStreamCreateWithFlags(&o->stream, cudaStreamNonBlocking);
  for (int k = 0; k < OUT_SLOTS && e == cudaSuccess; ++k) {
    e = cudaMalloc(&o->dev[k], b);
    if (e == cudaSuccess) e = cudaMallocHost(&o->host[k], b);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&o->snap[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&o->ready[k], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    output_close(c);
    return ch_cuda_fail(e, "ch_output_open", __FILE__, __LINE__);
  }
  o->writer = std::thread(output_thread, o);
  return CH_OK;
}

extern "C" ch_status ch_output(ch_ctx* c, const char* insert) {
  if (!c || !insert) return ch_fail(CH_ERR_ARG, "null argument");
  ChOutput* o = c->out;
  if (!o) return ch_fail(CH_ERR_STATE, "ch_output_open first");
  if (!c->moments_valid || !c->solved_once) return ch_fail(CH_ERR_STATE, "no moments or potential to output");
  const int k = o->next;
  o->next = (o->next + 1) % OUT_SLOTS;
  {
    std::unique_lock<std::mutex> lk(o->mu);
    o->cv.wait(lk, [&] { return !o->busy[k]; });  // the slot's previous write is done
    if (!o->error.empty()) return ch_fail(CH_ERR_CUDA, "output: %s", o->error.c_str());
    o->busy[k] = true;
  }
  const int64_t N = c->g.N;
  // snapshot on the compute stream (the next step overwrites the fields) ...
  CH_CUDA_OK(cudaMemcpyAsync(o->dev[k], c->mom, sizeof(double) * 4 * N, cudaMemcpyDeviceToDevice, c->stream));
  CH_CUDA_OK(cudaMemcpyAsync(o->dev[k] + 4 * N, c->rhs, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
  CH_CUDA_OK(cudaMemcpyAsync(o->dev[k] + 5 * N, c->phi, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
  CH_CUDA_OK(cudaEventRecord(o->snap[k], c->stream));
  // ... and the copy to the host on the output stream, beside the next step
  CH_CUDA_OK(cudaStreamWaitEvent(o->stream, o->snap[k], 0));
  CH_CUDA_OK(cudaMemcpyAsync(o->host[k], o->dev[k], sizeof(double) * OUT_FIELDS * N, cudaMemcpyDeviceToHost,
                             o->stream));
  CH_CUDA_OK(cudaEventRecord(o->ready[k], o->stream));
  {
    std::lock_guard<std::mutex> lk(o->mu);
    o->jobs.emplace_back(k, std::string(insert));
  }
  o->cv.notify_all();
  return CH_OK;
}

extern "C" ch_status ch_output_wait(ch_ctx* c, int64_t* written) {
  if (!c) return ch_fail(CH_ERR_ARG, "null ctx");
  ChOutput* o = c->out;
  if (!o) return ch_fail(CH_ERR_STATE, "ch_output_open first");
  std::unique_lock<std::mutex> lk(o->mu);
  o->cv.wait(lk, [&] {
    bool idle = o->jobs.empty();
    for (int k = 0; k < OUT_SLOTS; ++k) idle = idle && !o->busy[k];
    return idle;
  });
  if (written) *written = o->written;
  if (!o->error.empty()) return ch_fail(CH_ERR_CUDA, "output: %s", o->error.c_str());
  return CH_OK;
}
