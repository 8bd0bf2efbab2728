// chybrid_batch.cu -- the ensemble C ABI (ch_batch_*, include/chybrid.h).
//
// nruns independent runs share one set of device arrays: the ions of run r
// occupy slots [ion_off[r], ion_off[r+1]) of one mixed-form ion array, its
// grid vectors the nodes [node_off[r], node_off[r+1]) of the batch grid
// arrays.  A step is four launches over all runs -- the fused ion pass over
// every run's bricks, the per-run sums of its brick partials, the moment
// conversion, the potential solve with one thread-block cluster per run --
// plus the counting sort every sort_period steps (its keys node_off[r] + cell
// keep the runs contiguous).  The step number lives on the device, so a step
// is captured once as a CUDA graph and replayed.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <new>
#include <algorithm>
#include <vector>

#include "batch.cuh"
#include "particles.cuh"

using namespace ch;

ch_status ch_fail(ch_status code, const char* fmt, ...);
ch_status ch_cuda_fail(cudaError_t e, const char* what, const char* file, int line);

namespace {

constexpr int64_t MG_BATCH_MIN_EDGE = 4;  // a halved axis keeps >= 4 nodes

struct Pool {
  std::vector<void*> ptrs;
  cudaError_t err = cudaSuccess;
  template <typename T>
  T* get(size_t n) {
    void* p = nullptr;
    if (err == cudaSuccess) err = cudaMalloc(&p, sizeof(T) * (n ? n : 1));
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

// src/particles.c:510-519 (as ch_step)
int64_t collision_count(const ch_params& p, int64_t np) {
  const double viTr = sqrt(p.viT[0] * p.viT[0] + p.viT[1] * p.viT[1] + p.viT[2] * p.viT[2]);
  const double dvx = p.vi0[0] - p.vn0[0], dvy = p.vi0[1] - p.vn0[1], dvz = p.vi0[2] - p.vn0[2];
  const double vrm = 4.0 * viTr + sqrt(dvx * dvx + dvy * dvy + dvz * dvz);
  const double vn0r = sqrt(p.vn0[0] * p.vn0[0] + p.vn0[1] * p.vn0[1] + p.vn0[2] * p.vn0[2]);
  const double den = (p.vnT + vn0r) * sqrt(p.mn / p.mi);
  if (!(den > 0.0)) return np;
  const double v = ((double)np * p.nui * p.dt * vrm) / den;
  if (v >= (double)np) return np;
  if (v < 0.0) return 0;
  return (int64_t)v;
}

}  // namespace

struct ch_batch {
  int device = 0, sms = 1, nruns = 0;
  cudaStream_t stream = nullptr;
  std::vector<ch_params> p;
  std::vector<GridDesc> g;
  std::vector<int64_t> node_off, ion_off, np;
  std::vector<int> tile_off;
  int64_t Ntot = 0, NPtot = 0;
  int total_tiles = 0;
  int sort_period = 4;
  double dep_scale = 0.0;
  int dep_log2 = 40;
  Pool pool;
  // device
  BatchRunDev* d_runs = nullptr;
  int* d_tile_off = nullptr;
  int64_t* d_ion_off = nullptr;
  MixParticles M{}, MQ{};
  uint32_t *counts = nullptr, *starts = nullptr, *cursor = nullptr, *block_sums = nullptr, *dstep = nullptr;
  uint32_t* starts_next = nullptr;  // the order a sort step's deposit writes (swaps with starts)
  double *phi = nullptr, *mom = nullptr, *b64 = nullptr, *r64 = nullptr;
  float4* E32 = nullptr;
  unsigned long long* acc = nullptr;
  double *tile_part = nullptr, *run_sums = nullptr, *sbar = nullptr, *part = nullptr;
  int* flags = nullptr;  // nruns + 1 (the last: deposit range)
  BSolveRun* d_solve = nullptr;
  BSolveOut* d_out = nullptr;
  // host mirrors
  std::vector<BatchRunDev> runs;
  std::vector<BSolveRun> solve;
  // the solve records in the device order: largest grid first (see below)
  std::vector<BSolveRun> solve_order;
  BSolveOut* h_out = nullptr;
  double* h_sums = nullptr;
  int* h_flags = nullptr;
  // state
  std::vector<char> present;  // ions of run r loaded or uploaded
  bool loaded = false, initialized = false, parity = false;
  int since_sort = 0;
  ch_batch_tuning tune{4, 3, 0.0, 0.0, 0};
  cudaGraphExec_t graphs[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [sort_due][parity]
  long long graph_nodes[2][2] = {{0, 0}, {0, 0}};
  bool prof = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  ch_profile pr{};
  // Runs of at least twice the mean node count ("large": the first nbig
  // solve records) may be solved by clusters of tune.cluster_big CTAs in a
  // launch of their own, beside the others' launch on stream s2
  // (tune.cluster_big 0: one launch for all).
  int nbig = 0;
  cudaStream_t s2 = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
};

// The cluster solve of every run: one launch, or the large runs with
// clusters of Cbig CTAs on s and the others with C on s2, joined back to s
// (graph-capturable).
__global__ void k_scaled_copy(int64_t n, const double* __restrict__ a, double f, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = f * a[i];
}

static cudaError_t solve_launch(ch_batch* b, int C, int Cbig, cudaStream_t s) {
  if (Cbig > 0 && b->nbig > 0 && b->nbig < b->nruns) {
    cudaEventRecord(b->fork_ev, s);
    cudaStreamWaitEvent(b->s2, b->fork_ev, 0);
    const cudaError_t e1 = launch_batch_solve(b->d_solve, b->nbig, Cbig, s);
    const cudaError_t e2 = launch_batch_solve(b->d_solve + b->nbig, b->nruns - b->nbig, C, b->s2);
    cudaEventRecord(b->join_ev, b->s2);
    cudaStreamWaitEvent(s, b->join_ev, 0);
    return e1 != cudaSuccess ? e1 : e2;
  }
  return launch_batch_solve(b->d_solve, b->nruns, C, s);
}

static BatchDev batch_dev(const ch_batch* b) {
  BatchDev B;
  B.runs = b->d_runs;
  B.tile_off = b->d_tile_off;
  B.ion_off = b->d_ion_off;
  B.nruns = b->nruns;
  B.total_tiles = b->total_tiles;
  return B;
}

static MixParticles slice(const MixParticles& M, int64_t off, int64_t n) {
  MixParticles s;
  s.pos = M.pos + off;
  s.vel = M.vel + off;
  s.np = n;
  s.rank = nullptr;
  return s;
}

static void drop_graphs(ch_batch* b) {
  for (auto& row : b->graphs)
    for (auto& e : row)
      if (e) { cudaGraphExecDestroy(e); e = nullptr; }
}

extern "C" ch_status ch_batch_destroy(ch_batch* b) {
  if (!b) return CH_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  b->pool.release();
  if (b->h_out) cudaFreeHost(b->h_out);
  if (b->h_sums) cudaFreeHost(b->h_sums);
  if (b->h_flags) cudaFreeHost(b->h_flags);
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  if (b->join_ev) cudaEventDestroy(b->join_ev);
  if (b->s2) cudaStreamDestroy(b->s2);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return CH_OK;
}

static StepConsts run_consts(const ch_params& p, const GridDesc& g, double dep_scale) {
  StepConsts k;
  memset(&k, 0, sizeof(k));
  k.g = g;
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
  k.dep_scale = dep_scale;
  ch_consts_finish(k);
  return k;
}

static ch_status check_run(const ch_params& p, int r, const ch_params& p0) {
  if (p.precision != CH_MIXED) return ch_fail(CH_ERR_UNSUPPORTED, "batch run %d: only the mixed form", r);
  if (p.lhs_type != CH_LHS_FULL || p.rhs_type != CH_RHS_FULL)
    return ch_fail(CH_ERR_UNSUPPORTED, "batch run %d: full LHS and RHS only", r);
  if (p.ksp_type != CH_KSP_CG || p.pc_type != CH_PC_MG)
    return ch_fail(CH_ERR_UNSUPPORTED, "batch run %d: CG with the multigrid preconditioner only", r);
  if (p.kappa_e[0] != 0.0 || p.kappa_e[1] != 0.0 || p.kappa_e[2] != 0.0)
    return ch_fail(CH_ERR_UNSUPPORTED, "batch run %d: kappa_e != 0 makes A non-symmetric (CG needs kappa_e = 0)", r);
  if (p.faithful & ~(uint32_t)(CH_FAITHFUL_D2 | CH_FAITHFUL_D8))
    return ch_fail(CH_ERR_UNSUPPORTED, "batch run %d: faithful bits other than D2/D8", r);
  if (p.Nx < 3 || p.Ny < 3 || p.Nz < 3 || p.Nx > CH_MAX_NX || p.Ny > CH_MAX_NY || p.Nz > CH_MAX_NZ ||
      (int64_t)p.Nx * p.Ny * p.Nz >= (1LL << 31))
    return ch_fail(CH_ERR_ARG, "batch run %d: grid %dx%dx%d", r, p.Nx, p.Ny, p.Nz);
  if (!(p.x1 > p.x0) || !(p.y1 > p.y0) || !(p.z1 > p.z0) || !(p.mi > 0.0) || !(p.dt > 0.0))
    return ch_fail(CH_ERR_ARG, "batch run %d: empty domain, mass or dt", r);
  if (!(p.ksp_rtol > 0.0) || p.ksp_max_it < 1) return ch_fail(CH_ERR_ARG, "batch run %d: bad tolerance", r);
  if (p.mn > 0.0 && !(p.viT[0] > 0.0 || p.viT[1] > 0.0 || p.viT[2] > 0.0))
    return ch_fail(CH_ERR_ARG, "batch run %d: collisions need a positive ion thermal speed", r);
  if (p.sort_period != p0.sort_period || p.deposit_scale_log2 != p0.deposit_scale_log2)
    return ch_fail(CH_ERR_ARG, "batch run %d: sort_period and deposit_scale_log2 must agree across runs", r);
  return CH_OK;
}

// Multigrid hierarchy of one run (the rule of the single-run solver).
static ch_status build_levels(ch_batch* b, int r, BSolveRun& S) {
  const ch_params& p = b->p[r];
  GridDesc gl[CH_MG_MAX_LEVELS];
  int hx[CH_MG_MAX_LEVELS] = {0}, hy[CH_MG_MAX_LEVELS] = {0}, hz[CH_MG_MAX_LEVELS] = {0};
  gl[0] = b->g[r];
  int L = 1;
  while (L < CH_MG_MAX_LEVELS) {
    const GridDesc& f = gl[L - 1];
    const int ax = (f.Nx % 2 == 0 && f.Nx / 2 >= MG_BATCH_MIN_EDGE), ay = (f.Ny % 2 == 0 && f.Ny / 2 >= MG_BATCH_MIN_EDGE),
              az = (f.Nz % 2 == 0 && f.Nz / 2 >= MG_BATCH_MIN_EDGE);
    if (!(ax || ay || az) || f.N <= 64) break;
    GridDesc c = f;
    c.Nx = ax ? f.Nx / 2 : f.Nx; c.Ny = ay ? f.Ny / 2 : f.Ny; c.Nz = az ? f.Nz / 2 : f.Nz;
    c.dx = ax ? 2 * f.dx : f.dx; c.dy = ay ? 2 * f.dy : f.dy; c.dz = az ? 2 * f.dz : f.dz;
    ch_grid_finish(c);
    hx[L - 1] = ax; hy[L - 1] = ay; hz[L - 1] = az;
    gl[L++] = c;
  }
  if (gl[L - 1].N > BATCH_COARSE_MAX)
    return ch_fail(CH_ERR_UNSUPPORTED, "batch run %d: coarsest multigrid level %dx%dx%d exceeds %d nodes", r,
                   gl[L - 1].Nx, gl[L - 1].Ny, gl[L - 1].Nz, BATCH_COARSE_MAX);
  S.L = L;
  for (int l = 0; l < L; ++l) {
    BLevel& V = S.lv[l];
    V.g = gl[l];
    V.C = dev_coefs<float>(op_coefs(p, gl[l]));
    V.hx = hx[l]; V.hy = hy[l]; V.hz = hz[l];
    V.sR = 1.0f;  // full operator: finite-difference scaled
    const size_t n = (size_t)gl[l].N;
    V.n = b->pool.get<float>(n);
    V.dinv = b->pool.get<float>(n);
    V.r = b->pool.get<float>(n);
    V.t = b->pool.get<float>(n);
    V.x = l ? b->pool.get<float>(n) : nullptr;
    V.b = l ? b->pool.get<float>(n) : nullptr;
  }
  return b->pool.err == cudaSuccess ? CH_OK : ch_cuda_fail(b->pool.err, "cudaMalloc(batch levels)", __FILE__, __LINE__);
}

extern "C" ch_status ch_batch_create(const ch_params* runs, const int64_t* np, int32_t nruns, int32_t device,
                                     ch_batch** out) {
  if (!runs || !np || !out || nruns < 1) return ch_fail(CH_ERR_ARG, "ch_batch_create: bad arguments");
  *out = nullptr;
  for (int r = 0; r < nruns; ++r) {
    ch_status rc = check_run(runs[r], r, runs[0]);
    if (rc) return rc;
    if (np[r] < 1) return ch_fail(CH_ERR_ARG, "batch run %d: no ions", r);
  }
  if (device >= 0) CH_CUDA_OK(cudaSetDevice(device));
  ch_batch* b = new (std::nothrow) ch_batch();
  if (!b) return ch_fail(CH_ERR_NOMEM, "ch_batch_create: host allocation");
  CH_CUDA_OK(cudaGetDevice(&b->device));
  CH_CUDA_OK(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device));
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->s2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) { ch_batch_destroy(b); return ch_cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__); }
  b->nruns = nruns;
  b->p.assign(runs, runs + nruns);
  b->np.assign(np, np + nruns);
  b->sort_period = runs[0].sort_period > 0 ? runs[0].sort_period : 4;
  b->dep_log2 = (int)(runs[0].deposit_scale_log2 > 0.0 ? runs[0].deposit_scale_log2 : 40.0);
  if (b->dep_log2 < 22 || b->dep_log2 > 62) { ch_batch_destroy(b); return ch_fail(CH_ERR_ARG, "deposit scale"); }
  b->dep_scale = ldexp(1.0, b->dep_log2);
  b->node_off.assign(nruns + 1, 0);
  b->ion_off.assign(nruns + 1, 0);
  b->tile_off.assign(nruns + 1, 0);
  for (int r = 0; r < nruns; ++r) {
    const ch_params& q = runs[r];
    GridDesc g;
    g.Nx = q.Nx; g.Ny = q.Ny; g.Nz = q.Nz;
    ch_grid_finish(g);
    g.x0 = q.x0; g.y0 = q.y0; g.z0 = q.z0;
    g.Lx = q.x1 - q.x0; g.Ly = q.y1 - q.y0; g.Lz = q.z1 - q.z0;
    g.dx = g.Lx / q.Nx; g.dy = g.Ly / q.Ny; g.dz = g.Lz / q.Nz;
    b->g.push_back(g);
    b->node_off[r + 1] = b->node_off[r] + g.N;
    b->ion_off[r + 1] = b->ion_off[r] + np[r];
    b->tile_off[r + 1] = b->tile_off[r] + tiles_of(g);
  }
  b->Ntot = b->node_off[nruns];
  b->NPtot = b->ion_off[nruns];
  b->total_tiles = b->tile_off[nruns];
  if (b->NPtot > 0xFFFFFFFFll || b->Ntot > 0x7FFFFFFFll) {
    ch_batch_destroy(b);
    return ch_fail(CH_ERR_ARG, "batch too large: 2^32 ion slots and 2^31 nodes at most");
  }
  // device arrays
  Pool& P = b->pool;
  const int64_t N = b->Ntot, NP = b->NPtot;
  b->M.pos = P.get<float4>(NP); b->M.vel = P.get<float4>(NP); b->M.np = NP;
  b->MQ.pos = P.get<float4>(NP); b->MQ.vel = P.get<float4>(NP); b->MQ.np = NP;
  b->M.rank = b->MQ.rank = P.get<uint32_t>(NP);
  b->counts = P.get<uint32_t>(N);
  b->starts = P.get<uint32_t>(N + 1);
  b->starts_next = P.get<uint32_t>(N + 1);
  b->cursor = P.get<uint32_t>(N);
  b->block_sums = P.get<uint32_t>((N + 1023) / 1024 + 1);
  b->dstep = P.get<uint32_t>(1);
  b->phi = P.get<double>(N);
  b->mom = P.get<double>(4 * N);
  b->b64 = P.get<double>(N);
  b->r64 = P.get<double>(N);
  b->E32 = P.get<float4>(N);
  b->acc = P.get<unsigned long long>(4 * N);
  b->tile_part = P.get<double>(8 * (size_t)b->total_tiles);  // push partials, then the deposit's (unused)
  b->run_sums = P.get<double>(4 * (size_t)nruns);
  b->sbar = P.get<double>(nruns);
  b->part = P.get<double>((size_t)grid_for(NP, 256, b->sms, 8) * 4);
  b->flags = P.get<int>(nruns + 1);
  b->d_runs = P.get<BatchRunDev>(nruns);
  b->d_tile_off = P.get<int>(nruns + 1);
  b->d_ion_off = P.get<int64_t>(nruns + 1);
  b->d_solve = P.get<BSolveRun>(nruns);
  b->d_out = P.get<BSolveOut>(nruns);
  float* f32[6];
  for (auto& q : f32) q = P.get<float>(N);
  if (P.err != cudaSuccess) {
    const cudaError_t pe = P.err;
    ch_batch_destroy(b);
    return ch_cuda_fail(pe, "cudaMalloc(batch)", __FILE__, __LINE__);
  }
  if (cudaMallocHost(&b->h_out, sizeof(BSolveOut) * nruns) != cudaSuccess ||
      cudaMallocHost(&b->h_sums, sizeof(double) * 4 * nruns) != cudaSuccess ||
      cudaMallocHost(&b->h_flags, sizeof(int) * (nruns + 1)) != cudaSuccess) {
    ch_batch_destroy(b);
    return ch_fail(CH_ERR_NOMEM, "pinned host allocation");
  }
  // per-run descriptors
  b->present.assign(nruns, 0);
  b->runs.resize(nruns);
  b->solve.resize(nruns);
  for (int r = 0; r < nruns; ++r) {
    BatchRunDev& R = b->runs[r];
    R.c = run_consts(runs[r], b->g[r], b->dep_scale);
    R.node_off = b->node_off[r];
    R.ion_off = b->ion_off[r];
    R.np = np[r];
    R.tile_off = b->tile_off[r];
    R.ntiles = b->tile_off[r + 1] - b->tile_off[r];
    R.Nc = R.c.collide ? (double)collision_count(runs[r], np[r]) : 0.0;
    BSolveRun& S = b->solve[r];
    memset(&S, 0, sizeof(S));
    const int64_t no = b->node_off[r];
    S.g = b->g[r];
    S.C64 = dev_coefs<double>(op_coefs(runs[r], b->g[r]));
    // R = I + kappa kappa^T + [kappa]x with kappa_e = 0: the identity
    const double Rm[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    S.K = rhs_coefs(Rm, 1.0, runs[r].E0, runs[r].cth, runs[r].cG, (runs[r].faithful & CH_FAITHFUL_D8) != 0,
                    b->g[r].dx, b->g[r].dy, b->g[r].dz);
    S.rtol = runs[r].ksp_rtol;
    S.atol = runs[r].ksp_atol;
    S.maxit = runs[r].ksp_max_it;
    S.tscale = R.c.tscale;
    S.mom = b->mom + 4 * no;
    S.phi = b->phi + no;
    S.b64 = b->b64 + no;
    S.r64 = b->r64 + no;
    S.b32 = f32[0] + no; S.x32 = f32[1] + no; S.r32 = f32[2] + no;
    S.z32 = f32[3] + no; S.p32 = f32[4] + no; S.q32 = f32[5] + no;
    S.E32 = b->E32 + no;
    S.out = b->d_out + r;
    ch_status rc = build_levels(b, r, S);
    if (rc) { ch_batch_destroy(b); return rc; }
  }
  cudaStream_t s = b->stream;
  CH_CUDA_OK(cudaMemcpyAsync(b->d_runs, b->runs.data(), sizeof(BatchRunDev) * nruns, cudaMemcpyHostToDevice, s));
  // The cluster solve runs the largest grids first: the CTAs of one launch do
  // not all fit at once, and a large run left to the last wave sets the
  // time of the whole launch.  Each record carries its own arrays and output,
  // so the order is free.
  b->solve_order = b->solve;
  std::stable_sort(b->solve_order.begin(), b->solve_order.end(),
                   [](const BSolveRun& a, const BSolveRun& c) { return a.g.N > c.g.N; });
  {
    double mean = 0.0;
    for (const BSolveRun& R : b->solve_order) mean += (double)R.g.N / nruns;
    b->nbig = 0;
    while (b->nbig < nruns && (double)b->solve_order[b->nbig].g.N >= 2.0 * mean) ++b->nbig;
  }
  CH_CUDA_OK(cudaMemcpyAsync(b->d_solve, b->solve_order.data(), sizeof(BSolveRun) * nruns, cudaMemcpyHostToDevice,
                             s));
  CH_CUDA_OK(cudaMemcpyAsync(b->d_tile_off, b->tile_off.data(), sizeof(int) * (nruns + 1), cudaMemcpyHostToDevice, s));
  CH_CUDA_OK(cudaMemcpyAsync(b->d_ion_off, b->ion_off.data(), sizeof(int64_t) * (nruns + 1), cudaMemcpyHostToDevice,
                             s));
  CH_CUDA_OK(cudaMemsetAsync(b->phi, 0, sizeof(double) * N, s));
  CH_CUDA_OK(cudaMemsetAsync(b->acc, 0, sizeof(unsigned long long) * 4 * N, s));
  CH_CUDA_OK(cudaMemsetAsync(b->sbar, 0, sizeof(double) * nruns, s));
  CH_CUDA_OK(cudaMemsetAsync(b->flags, 0, sizeof(int) * (nruns + 1), s));
  CH_CUDA_OK(cudaMemsetAsync(b->E32, 0, sizeof(float4) * N, s));
  batch_pass_prepare();
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { ch_batch_destroy(b); return ch_cuda_fail(e, "ch_batch_create", __FILE__, __LINE__); }
  *out = b;
  return CH_OK;
}

static ch_status after_load(ch_batch* b, int run) {
  if (run < 0) b->present.assign(b->nruns, 1);
  else b->present[run] = 1;
  b->loaded = true;
  for (char q : b->present) b->loaded = b->loaded && q;
  b->initialized = false;
  drop_graphs(b);
  return CH_OK;
}

extern "C" ch_status ch_batch_load(ch_batch* b, const ch_loader* L) {
  if (!b || !L) return ch_fail(CH_ERR_ARG, "ch_batch_load: null argument");
  for (int r = 0; r < b->nruns; ++r) {
    const double s = fabs(L[r].amp[0]) + fabs(L[r].amp[1]) + fabs(L[r].amp[2]);
    if (!(s < 1.0)) return ch_fail(CH_ERR_ARG, "batch run %d: perturbation amplitudes must sum below 1", r);
    F64Particles none{};
    launch_load(true, b->g[r], L[r], b->p[r].seed, b->p[r].run, none, slice(b->M, b->ion_off[r], b->np[r]), b->sms,
                b->stream);
  }
  CH_CUDA_OK(cudaStreamSynchronize(b->stream));
  return after_load(b, -1);
}

extern "C" ch_status ch_batch_upload(ch_batch* b, int32_t run, const ch_real_vector* pos, const ch_real_vector* vel) {
  if (!b || !pos || !vel || run < 0 || run >= b->nruns) return ch_fail(CH_ERR_ARG, "ch_batch_upload: bad arguments");
  const int64_t n = b->np[run];
  double4_32a *sp = nullptr, *sv = nullptr;
  CH_CUDA_OK(cudaMalloc(&sp, sizeof(double4_32a) * n));
  cudaError_t e = cudaMalloc(&sv, sizeof(double4_32a) * n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sp, pos, sizeof(double4_32a) * n, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sv, vel, sizeof(double4_32a) * n, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) {
    F64Particles none{};
    launch_aos_in(true, b->g[run], sp, sv, none, slice(b->M, b->ion_off[run], n), b->sms, b->stream);
    e = cudaStreamSynchronize(b->stream);
  }
  cudaFree(sp);
  if (sv) cudaFree(sv);
  if (e != cudaSuccess) return ch_cuda_fail(e, "ch_batch_upload", __FILE__, __LINE__);
  return after_load(b, run);
}

extern "C" ch_status ch_batch_download(ch_batch* b, int32_t run, ch_real_vector* pos, ch_real_vector* vel) {
  if (!b || !pos || !vel || run < 0 || run >= b->nruns)
    return ch_fail(CH_ERR_ARG, "ch_batch_download: bad arguments");
  const int64_t n = b->np[run];
  double4_32a *sp = nullptr, *sv = nullptr;
  CH_CUDA_OK(cudaMalloc(&sp, sizeof(double4_32a) * n));
  cudaError_t e = cudaMalloc(&sv, sizeof(double4_32a) * n);
  if (e == cudaSuccess) {
    F64Particles none{};
    launch_aos_out(true, b->g[run], none, slice(b->M, b->ion_off[run], n), sp, sv, b->sms, b->stream);
    e = cudaMemcpyAsync(pos, sp, sizeof(double4_32a) * n, cudaMemcpyDeviceToHost, b->stream);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(vel, sv, sizeof(double4_32a) * n, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  cudaFree(sp);
  if (sv) cudaFree(sv);
  if (e != cudaSuccess) return ch_cuda_fail(e, "ch_batch_download", __FILE__, __LINE__);
  return CH_OK;
}

// Full counting sort of every run's ions (counts are recounted).  The step
// graphs hold the ion and order buffers of their parity, which this swap does
// not follow, so they are captured again.
static void full_sort(ch_batch* b) {
  drop_graphs(b);
  cudaMemsetAsync(b->counts, 0, sizeof(uint32_t) * b->Ntot, b->stream);
  launch_batch_hist(batch_dev(b), b->M, b->counts, b->sms, b->stream);
  launch_batch_sort(batch_dev(b), b->Ntot, b->M, b->MQ, b->counts, b->starts, b->cursor, b->block_sums, b->sms,
                    b->stream);
  std::swap(b->M, b->MQ);
  b->since_sort = 0;
}

static ch_status read_status(ch_batch* b, ch_run_info* info) {
  cudaStream_t s = b->stream;
  CH_CUDA_OK(cudaMemcpyAsync(b->h_out, b->d_out, sizeof(BSolveOut) * b->nruns, cudaMemcpyDeviceToHost, s));
  CH_CUDA_OK(cudaMemcpyAsync(b->h_sums, b->run_sums, sizeof(double) * 4 * b->nruns, cudaMemcpyDeviceToHost, s));
  CH_CUDA_OK(cudaMemcpyAsync(b->h_flags, b->flags, sizeof(int) * (b->nruns + 1), cudaMemcpyDeviceToHost, s));
  CH_CUDA_OK(cudaStreamSynchronize(s));
  ch_status first = CH_OK;
  int first_run = -1;
  for (int r = 0; r < b->nruns; ++r) {
    const BSolveOut& o = b->h_out[r];
    int fl = o.flags | b->h_flags[r];
    if (b->h_flags[b->nruns] & 1) fl |= 32;
    ch_status st = (ch_status)o.status;
    if (fl & 16) st = CH_ERR_NAN;
    else if (fl & 32) st = CH_ERR_RANGE;
    else if (fl & 8) st = CH_ERR_COLLISION_LIMIT;
    if (info) {
      ch_run_info& I = info[r];
      I.Nc = (int64_t)b->runs[r].Nc;
      I.expected = b->h_sums[4 * r + 0];
      I.collisions = (int64_t)b->h_sums[4 * r + 2];
      I.refused = (int64_t)b->h_sums[4 * r + 3];
      I.solve.iterations = o.iterations;
      I.solve.refinements = o.refinements;
      I.solve.rnorm = o.rnorm;
      I.solve.bnorm = o.bnorm;
      I.status = st;
      I.flags = fl;
    }
    if (st != CH_OK && first == CH_OK) { first = st; first_run = r; }
  }
  if (first != CH_OK)
    return ch_fail(first, "batch run %d failed (status %d, flags %d)", first_run, (int)first,
                   b->h_out[first_run].flags | b->h_flags[first_run]);
  return CH_OK;
}

extern "C" ch_status ch_batch_initialize(ch_batch* b) {
  if (!b) return ch_fail(CH_ERR_ARG, "null batch");
  if (!b->loaded) return ch_fail(CH_ERR_STATE, "ions missing: load, or upload every run, first");
  cudaStream_t s = b->stream;
  full_sort(b);
  // S of every run for the first step's collision rates
  for (int r = 0; r < b->nruns; ++r) {
    if (!(b->p[r].mn > 0.0)) continue;
    F64Particles none{};
    const int nb = launch_sbar(true, b->runs[r].c, none, slice(b->M, b->ion_off[r], b->np[r]), b->part, b->sms, s);
    launch_reduce_partials(b->part, nb, 1, b->sbar + r, s);
  }
  CH_CUDA_OK(cudaMemsetAsync(b->flags, 0, sizeof(int) * (b->nruns + 1), s));
  launch_batch_pass(PH_DEPOSIT, batch_dev(b), b->dstep, b->M, b->E32, b->starts, b->acc, b->sbar, b->dep_log2,
                    nullptr, b->tile_part, b->flags, b->tune.pass_ctas_per_sm, b->sms, s);
  launch_batch_finalize(4 * b->Ntot, b->acc, 1.0 / b->dep_scale, b->mom, b->flags + b->nruns, b->sms, s);
  CH_CUDA_OK(solve_launch(b, b->tune.cluster, b->tune.cluster_big, s));
  CH_CUDA_OK(cudaGetLastError());
  ch_status rc = read_status(b, nullptr);
  if (rc) return rc;
  b->initialized = true;
  return CH_OK;
}

// One step on the stream (graph-capturable).  Returns the launch error.
static cudaError_t enqueue_step(ch_batch* b, bool sort_due) {
  cudaStream_t s = b->stream;
  const BatchDev B = batch_dev(b);
  if (b->prof) cudaEventRecord(b->ev[0], s);
  if (sort_due) cudaMemsetAsync(b->counts, 0, sizeof(uint32_t) * b->Ntot, s);
  // push + collide + move, then the deposit (two launches, as the single-run step).
  // Sort due: the push counts the new cells, the scan orders them, and the
  // deposit writes every ion to its sorted slot of MQ.
  launch_batch_pass(PH_PUSH | PH_MOVE, B, b->dstep, b->M, b->E32, b->starts, b->acc, b->sbar, b->dep_log2,
                    sort_due ? b->counts : nullptr, b->tile_part, b->flags, b->tune.pass_ctas_per_sm, b->sms, s);
  if (sort_due) launch_scan(b->Ntot, b->counts, b->starts_next, b->cursor, b->block_sums, s);
  launch_batch_pass(PH_DEPOSIT, B, b->dstep, b->M, b->E32, b->starts, b->acc, b->sbar, b->dep_log2, nullptr,
                    b->tile_part + 4 * (size_t)b->total_tiles, b->flags, b->tune.pass_ctas_per_sm, b->sms, s,
                    b->MQ, sort_due ? b->starts_next : nullptr);
  launch_batch_runsum(B, b->tile_part, b->run_sums, b->sbar, b->flags, b->dstep, s);
  launch_batch_finalize(4 * b->Ntot, b->acc, 1.0 / b->dep_scale, b->mom, b->flags + b->nruns, b->sms, s);
  if (b->prof) cudaEventRecord(b->ev[1], s);
  cudaError_t e = solve_launch(b, b->tune.cluster, b->tune.cluster_big, s);
  if (b->prof) cudaEventRecord(b->ev[2], s);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

static ch_status step_graph(ch_batch* b, bool sort_due) {
  const int si = sort_due ? 1 : 0, pi = b->parity ? 1 : 0;
  if (!b->graphs[si][pi]) {
    cudaGraph_t graph;
    const unsigned long long before = ::ch::launches_now();
    CH_CUDA_OK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t le = enqueue_step(b, sort_due);
    cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
    if (le != cudaSuccess) return ch_cuda_fail(le, "batch step capture", __FILE__, __LINE__);
    if (ce != cudaSuccess) return ch_cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
    const long long nodes = (long long)(::ch::launches_now() - before);
    ::ch::note_launch_n(-nodes);
    ce = cudaGraphInstantiate(&b->graphs[si][pi], graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return ch_cuda_fail(ce, "cudaGraphInstantiate", __FILE__, __LINE__);
    b->graph_nodes[si][pi] = nodes;
  }
  CH_CUDA_OK(cudaGraphLaunch(b->graphs[si][pi], b->stream));
  ::ch::note_launch_n(b->graph_nodes[si][pi]);
  return CH_OK;
}

extern "C" ch_status ch_batch_step(ch_batch* b, int64_t first_step, int32_t nsteps, ch_run_info* info) {
  if (!b) return ch_fail(CH_ERR_ARG, "null batch");
  if (!b->initialized) return ch_fail(CH_ERR_STATE, "call ch_batch_initialize first");
  if (nsteps < 0) return ch_fail(CH_ERR_ARG, "nsteps < 0");
  cudaStream_t s = b->stream;
  const uint32_t st = (uint32_t)first_step;
  CH_CUDA_OK(cudaMemcpyAsync(b->dstep, &st, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  CH_CUDA_OK(cudaMemsetAsync(b->flags, 0, sizeof(int) * (b->nruns + 1), s));
  for (int32_t k = 0; k < nsteps; ++k) {
    const bool sort_due = b->since_sort + 1 >= b->sort_period;
    if (b->prof) {
      CH_CUDA_OK(enqueue_step(b, sort_due));
      float t0 = 0.0f, t1 = 0.0f;
      CH_CUDA_OK(cudaStreamSynchronize(s));
      cudaEventElapsedTime(&t0, b->ev[0], b->ev[1]);
      cudaEventElapsedTime(&t1, b->ev[1], b->ev[2]);
      b->pr.pass_ms += t0;
      b->pr.pass_calls += 1;
      b->pr.solve_ms += t1;
      b->pr.solve_calls += 1;
    } else {
      ch_status rc = step_graph(b, sort_due);
      if (rc) return rc;
    }
    if (sort_due) {
      std::swap(b->M, b->MQ);
      std::swap(b->starts, b->starts_next);
      b->parity = !b->parity;
      b->since_sort = 0;
    } else {
      b->since_sort++;
    }
  }
  // the uploaded step value is read by the first pass: keep the host copy alive
  CH_CUDA_OK(cudaStreamSynchronize(s));
  return read_status(b, info);
}

extern "C" ch_status ch_batch_get_phi(ch_batch* b, int32_t run, double* out) {
  if (!b || !out || run < 0 || run >= b->nruns) return ch_fail(CH_ERR_ARG, "bad arguments");
  CH_CUDA_OK(cudaMemcpyAsync(out, b->phi + b->node_off[run], sizeof(double) * b->g[run].N, cudaMemcpyDeviceToHost,
                             b->stream));
  CH_CUDA_OK(cudaStreamSynchronize(b->stream));
  return CH_OK;
}

extern "C" ch_status ch_batch_set_phi(ch_batch* b, int32_t run, const double* in) {
  if (!b || !in || run < 0 || run >= b->nruns) return ch_fail(CH_ERR_ARG, "bad arguments");
  CH_CUDA_OK(cudaMemcpyAsync(b->phi + b->node_off[run], in, sizeof(double) * b->g[run].N, cudaMemcpyHostToDevice,
                             b->stream));
  // the next push reads the node field the solve would have left
  launch_node_efield(true, b->g[run], b->runs[run].c.tscale, b->phi + b->node_off[run], nullptr,
                     b->E32 + b->node_off[run], b->sms, b->stream);
  CH_CUDA_OK(cudaStreamSynchronize(b->stream));
  return CH_OK;
}

extern "C" ch_status ch_batch_get_moments(ch_batch* b, int32_t run, ch_grid_node* out) {
  if (!b || !out || run < 0 || run >= b->nruns) return ch_fail(CH_ERR_ARG, "bad arguments");
  const int64_t N = b->g[run].N;
  const double* m = b->mom + 4 * b->node_off[run];
  for (int q = 0; q < 4; ++q)
    CH_CUDA_OK(cudaMemcpy2DAsync((char*)out + q * sizeof(double), sizeof(ch_grid_node), m + q * N, sizeof(double),
                                 sizeof(double), N, cudaMemcpyDeviceToHost, b->stream));
  CH_CUDA_OK(cudaStreamSynchronize(b->stream));
  return CH_OK;
}

extern "C" ch_status ch_batch_set_tuning(ch_batch* b, const ch_batch_tuning* t) {
  if (!b || !t) return ch_fail(CH_ERR_ARG, "null argument");
  if (!(t->cluster == 1 || t->cluster == 2 || t->cluster == 4 || t->cluster == 8))
    return ch_fail(CH_ERR_ARG, "cluster must be 1, 2, 4 or 8");
  if (t->pass_ctas_per_sm < 1 || t->pass_ctas_per_sm > 3) return ch_fail(CH_ERR_ARG, "pass_ctas_per_sm: 1 to 3");
  b->tune.cluster = t->cluster;
  if (!(t->cluster_big == 0 || t->cluster_big == 8 || t->cluster_big == 16))
    return ch_fail(CH_ERR_ARG, "cluster_big must be 0, 8 or 16");
  if (t->cluster_big == 16 && !batch_solve_allow_wide())
    return ch_fail(CH_ERR_UNSUPPORTED, "clusters of 16 CTAs are not available on this device");
  b->tune.pass_ctas_per_sm = t->pass_ctas_per_sm;
  b->tune.cluster_big = t->cluster_big;
  drop_graphs(b);
  return CH_OK;
}

extern "C" ch_status ch_batch_get_tuning(ch_batch* b, ch_batch_tuning* out) {
  if (!b || !out) return ch_fail(CH_ERR_ARG, "null argument");
  *out = b->tune;
  return CH_OK;
}

// Times each launch shape on the current state.  The solve is timed from the
// same phi (saved and restored); the pass from the same ions (saved in the
// sort's spare buffers and restored), with the deposit discarded.  The
// pass shape is the deposit launch's CTAs per SM.
extern "C" ch_status ch_batch_autotune(ch_batch* b, ch_batch_tuning* out) {
  if (!b) return ch_fail(CH_ERR_ARG, "null batch");
  if (!b->initialized) return ch_fail(CH_ERR_STATE, "call ch_batch_initialize first");
  cudaStream_t s = b->stream;
  const int64_t N = b->Ntot, NP = b->NPtot;
  cudaEvent_t e0, e1;
  CH_CUDA_OK(cudaEventCreate(&e0));
  CH_CUDA_OK(cudaEventCreate(&e1));
  double* phi0 = nullptr;
  cudaError_t err = cudaMalloc(&phi0, sizeof(double) * N);
  if (err != cudaSuccess) return ch_cuda_fail(err, "cudaMalloc(autotune)", __FILE__, __LINE__);
  auto timed = [&](auto&& fn) {
    cudaEventRecord(e0, s);
    fn();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    return (double)t;
  };
  uint32_t step_now = 0;
  cudaMemcpyAsync(&step_now, b->dstep, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(phi0, b->phi, sizeof(double) * N, cudaMemcpyDeviceToDevice, s);
  // solve: clusters of 1, 2, 4, 8 CTAs for every run, or the large runs with
  // clusters of 8 or 16 beside the others.  Each shape starts from the saved
  // phi scaled by 0.999 (a residual of about 1e-3 of b, as a step's warm
  // start), not from the converged phi, which would time a solve of a few
  // iterations.
  const bool wide = batch_solve_allow_wide();
  double best_solve = 1e30;
  int best_c = b->tune.cluster, best_big = 0;
  const int shapes[][2] = {{1, 0}, {2, 0}, {4, 0}, {8, 0}, {1, 8}, {2, 8}, {4, 8}, {2, 16}, {4, 16}, {8, 16}};
  for (const auto& sh : shapes) {
    const int C = sh[0], Cb = sh[1];
    if (Cb > 0 && (b->nbig == 0 || b->nbig == b->nruns)) continue;
    if (Cb > 8 && !wide) continue;
    double t = 0.0;
    bool ok = true;
    for (int rep = 0; rep < 2 && ok; ++rep) {  // the first launch of a shape warms up
      k_scaled_copy<<<grid_for(N, 256, b->sms, 4), 256, 0, s>>>(N, phi0, 0.999, b->phi);
      ::ch::note_launch();
      t = timed([&] { ok = solve_launch(b, C, Cb, s) == cudaSuccess; });
    }
    if (cudaGetLastError() != cudaSuccess || !ok) continue;
    if (t < best_solve) { best_solve = t; best_c = C; best_big = Cb; }
  }
  cudaMemcpyAsync(b->phi, phi0, sizeof(double) * N, cudaMemcpyDeviceToDevice, s);
  // pass: 1 or 2 persistent CTAs per SM, from the same ions each time
  cudaMemcpyAsync(b->MQ.pos, b->M.pos, sizeof(float4) * NP, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(b->MQ.vel, b->M.vel, sizeof(float4) * NP, cudaMemcpyDeviceToDevice, s);
  double best_pass = 1e30;
  int best_k = b->tune.pass_ctas_per_sm;
  for (int k : {1, 2, 3}) {
    double t = 0.0;
    for (int rep = 0; rep < 2; ++rep) {
      cudaMemcpyAsync(b->M.pos, b->MQ.pos, sizeof(float4) * NP, cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(b->M.vel, b->MQ.vel, sizeof(float4) * NP, cudaMemcpyDeviceToDevice, s);
      t = timed([&] {
        launch_batch_pass(PH_PUSH | PH_MOVE, batch_dev(b), b->dstep, b->M, b->E32, b->starts, b->acc, b->sbar,
                          b->dep_log2, nullptr, b->tile_part, b->flags, k, b->sms, s);
        launch_batch_pass(PH_DEPOSIT, batch_dev(b), b->dstep, b->M, b->E32, b->starts, b->acc, b->sbar,
                          b->dep_log2, nullptr, b->tile_part + 4 * (size_t)b->total_tiles, b->flags, k, b->sms, s);
      });
    }
    if (t < best_pass) { best_pass = t; best_k = k; }
  }
  cudaMemcpyAsync(b->M.pos, b->MQ.pos, sizeof(float4) * NP, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(b->M.vel, b->MQ.vel, sizeof(float4) * NP, cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(b->acc, 0, sizeof(unsigned long long) * 4 * N, s);
  cudaMemsetAsync(b->flags, 0, sizeof(int) * (b->nruns + 1), s);
  cudaMemcpyAsync(b->dstep, &step_now, sizeof(uint32_t), cudaMemcpyHostToDevice, s);
  err = cudaStreamSynchronize(s);
  cudaFree(phi0);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return ch_cuda_fail(err, "ch_batch_autotune", __FILE__, __LINE__);
  b->tune.cluster = best_c;
  b->tune.cluster_big = best_big;
  b->tune.pass_ctas_per_sm = best_k;
  b->tune.solve_ms = best_solve;
  b->tune.pass_ms = best_pass;
  drop_graphs(b);
  if (out) *out = b->tune;
  return CH_OK;
}

extern "C" ch_status ch_batch_set_profiling(ch_batch* b, int32_t enable) {
  if (!b) return ch_fail(CH_ERR_ARG, "null batch");
  if (enable && !b->ev[0])
    for (auto& e : b->ev) CH_CUDA_OK(cudaEventCreate(&e));
  b->prof = enable != 0;
  return CH_OK;
}

extern "C" ch_status ch_batch_get_profile(ch_batch* b, ch_profile* out) {
  if (!b || !out) return ch_fail(CH_ERR_ARG, "null argument");
  *out = b->pr;
  out->launches = (int64_t)::ch::launches_now();
  return CH_OK;
}

extern "C" ch_status ch_batch_get_stream(ch_batch* b, void** stream) {
  if (!b || !stream) return ch_fail(CH_ERR_ARG, "null argument");
  *stream = (void*)b->stream;
  return CH_OK;
}

// ------------------------------------------------------------------ tuning cache
// The launch shape ch_batch_autotune picks depends on the device and on the
// batch's shape: the run count and how the nodes and ions are spread over
// the runs.  A batch whose class (device name and SM count, run count, and
// the power-of-two buckets of its total nodes, total ions and largest run)
// matches a line of the cache file takes that line's shape without timing.
static int log2_bucket(int64_t v) {
  int b = 0;
  while (b < 62 && (int64_t(1) << (b + 1)) <= v) ++b;
  return b;
}

static void tuning_key(const ch_batch* b, char* key, size_t n) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, b->device) != cudaSuccess) {
    cudaGetLastError();
    snprintf(prop.name, sizeof(prop.name), "unknown");
  }
  for (char* q = prop.name; *q; ++q)
    if (*q == ' ' || *q == '"' || *q == '|') *q = '_';
  int64_t maxrun = 0;
  for (const GridDesc& g : b->g) maxrun = g.N > maxrun ? g.N : maxrun;
  snprintf(key, n, "%s|sm%d|runs%d|nodes2^%d|ions2^%d|maxrun2^%d", prop.name, b->sms, b->nruns,
           log2_bucket(b->Ntot), log2_bucket(b->NPtot), log2_bucket(maxrun));
}

extern "C" ch_status ch_batch_autotune_cached(ch_batch* b, const char* path, ch_batch_tuning* out, int32_t* hit) {
  if (!b || !path) return ch_fail(CH_ERR_ARG, "null argument");
  if (hit) *hit = 0;
  char key[256];
  tuning_key(b, key, sizeof(key));
  FILE* f = fopen(path, "r");
  if (f) {
    char line[512];
    ch_batch_tuning t, r;
    bool found = false;
    while (fgets(line, sizeof(line), f)) {
      char k[256];
      memset(&r, 0, sizeof(r));
      if (sscanf(line,
                 "{\"key\": \"%255[^\"]\", \"cluster\": %d, \"pass_ctas_per_sm\": %d, \"cluster_big\": %d, "
                 "\"pass_ms\": %lf, \"solve_ms\": %lf}",
                 k, &r.cluster, &r.pass_ctas_per_sm, &r.cluster_big, &r.pass_ms, &r.solve_ms) == 6 &&
          !strcmp(k, key)) {
        t = r;  // the last matching line wins
        found = true;
      }
    }
    fclose(f);
    if (found) {
      ch_status rc = ch_batch_set_tuning(b, &t);
      if (rc) return rc;
      b->tune.pass_ms = t.pass_ms;
      b->tune.solve_ms = t.solve_ms;
      if (hit) *hit = 1;
      if (out) *out = b->tune;
      return CH_OK;
    }
  }
  ch_batch_tuning t;
  ch_status rc = ch_batch_autotune(b, &t);
  if (rc) return rc;
  f = fopen(path, "a");
  if (!f) return ch_fail(CH_ERR_ARG, "ch_batch_autotune_cached: cannot append to %s", path);
  fprintf(f, "{\"key\": \"%s\", \"cluster\": %d, \"pass_ctas_per_sm\": %d, \"cluster_big\": %d, "
             "\"pass_ms\": %.6f, \"solve_ms\": %.6f}\n",
          key, t.cluster, t.pass_ctas_per_sm, t.cluster_big, t.pass_ms, t.solve_ms);
  fclose(f);
  if (out) *out = t;
  return CH_OK;
}
