// noalloc.cu -- a cloud-in-cell deposit that allocates no memory.
//
// ch_collect_moments needs a ch_ctx, whose creation allocates device
// buffers.  Some callers cannot allocate: a host whose device memory is all
// owned by its own pool allocator, code that records its launches into a CUDA
// graph (allocation is not allowed while a stream is being captured), or a
// time-critical loop that cannot afford the implicit device synchronisation
// of cudaMalloc/cudaFree.  ch_collect_moments_noalloc serves them: the caller
// passes device pointers for the ions and the output moments, and the only
// scratch the deposit needs -- its 64-bit fixed-point accumulators -- lives in
// a fixed array in this file, sized for grids of at most
// CH_NOALLOC_MAX_NODES nodes.
#include <mutex>

#include "common.cuh"

// 64^3 nodes: 4 moments x 2^18 nodes x 8 bytes = 8 MiB, held by every GPU
// that loads this library until the process exits.
#define CH_NOALLOC_MAX_NODES (1 << 18)
#define CH_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned long long g_noalloc_acc[4 * CH_NOALLOC_MAX_NODES];

// Device address of g_noalloc_acc per device.  In host code the array's name
// is only a host-side stand-in, so the address is looked up once per device
// with that device current.
static unsigned long long* g_noalloc_dev[CH_NOALLOC_MAX_DEVICES] = {};
static std::mutex g_noalloc_mu;

namespace {

__global__ void k_noalloc_zero(unsigned long long* __restrict__ acc, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    acc[c] = 0ull;
}

// CIC weights of src/particles.c:189-211, fixed point with scale 2^s.
__global__ void k_noalloc_deposit(GridDesc g, double scale, const double* __restrict__ x,
                                  const double* __restrict__ y, const double* __restrict__ z,
                                  const double* __restrict__ vx, const double* __restrict__ vy,
                                  const double* __restrict__ vz, int64_t np, unsigned long long* __restrict__ acc) {
  const int64_t N = g.N;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < np; ip += (int64_t)gridDim.x * blockDim.x) {
    const double X = (x[ip] - g.x0) / g.dx, Y = (y[ip] - g.y0) / g.dy, Z = (z[ip] - g.z0) / g.dz;
    const double fi = floor(X), fj = floor(Y), fk = floor(Z);
    if (!(isfinite(fi) && isfinite(fj) && isfinite(fk))) continue;
    const int i = ch_wrap((int)fi, g.Nx), j = ch_wrap((int)fj, g.Ny), k = ch_wrap((int)fk, g.Nz);
    const double wxh = X - fi, wyh = Y - fj, wzh = Z - fk;
    const double wxl = 1.0 - wxh, wyl = 1.0 - wyh, wzl = 1.0 - wzh;
    const int i1 = i + 1 == g.Nx ? 0 : i + 1, j1 = j + 1 == g.Ny ? 0 : j + 1, k1 = k + 1 == g.Nz ? 0 : k + 1;
    const int64_t rz0 = (int64_t)k * g.Ny, rz1 = (int64_t)k1 * g.Ny;
    const int64_t c[8] = {(rz1 + j1) * g.Nx + i1, (rz0 + j1) * g.Nx + i1, (rz1 + j) * g.Nx + i1,
                          (rz0 + j) * g.Nx + i1,  (rz1 + j1) * g.Nx + i,  (rz0 + j1) * g.Nx + i,
                          (rz1 + j) * g.Nx + i,   (rz0 + j) * g.Nx + i};
    const double w[8] = {wzh * wyh * wxh, wzl * wyh * wxh, wzh * wyl * wxh, wzl * wyl * wxh,
                         wzh * wyh * wxl, wzl * wyh * wxl, wzh * wyl * wxl, wzl * wyl * wxl};
    const double v0 = vx[ip], v1 = vy[ip], v2 = vz[ip];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      atomicAdd(acc + c[q], (unsigned long long)__double2ll_rn(w[q] * scale));
      atomicAdd(acc + N + c[q], (unsigned long long)__double2ll_rn(v0 * w[q] * scale));
      atomicAdd(acc + 2 * N + c[q], (unsigned long long)__double2ll_rn(v1 * w[q] * scale));
      atomicAdd(acc + 3 * N + c[q], (unsigned long long)__double2ll_rn(v2 * w[q] * scale));
    }
  }
}

__global__ void k_noalloc_finalize(const unsigned long long* __restrict__ acc, int64_t n4, double inv_scale,
                                   double* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n4; c += (int64_t)gridDim.x * blockDim.x)
    out[c] = (double)(long long)acc[c] * inv_scale;
}

}  // namespace

// Looks up the device address of the scratch array for the current device,
// once per device.
static ch_status noalloc_scratch(unsigned long long** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return ch_cuda_fail(e, "cudaGetDevice", __FILE__, __LINE__);
  if (dev < 0 || dev >= CH_NOALLOC_MAX_DEVICES)
    return ch_fail(CH_ERR_UNSUPPORTED, "device %d: at most %d devices", dev, CH_NOALLOC_MAX_DEVICES);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_dev[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_acc);
    if (e != cudaSuccess) return ch_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_acc)", __FILE__, __LINE__);
    g_noalloc_dev[dev] = static_cast<unsigned long long*>(ptr);
  }
  *out = g_noalloc_dev[dev];
  return CH_OK;
}

extern "C" ch_status ch_collect_moments_noalloc(const ch_params* p, const double* x, const double* y,
                                                const double* z, const double* vx, const double* vy,
                                                const double* vz, int64_t np, double* moments, void* stream) {
  if (!p || !moments || (np > 0 && (!x || !y || !z || !vx || !vy || !vz)))
    return ch_fail(CH_ERR_ARG, "ch_collect_moments_noalloc: null argument");
  if (np < 0) return ch_fail(CH_ERR_ARG, "ch_collect_moments_noalloc: np < 0");
  if (p->Nx < 3 || p->Ny < 3 || p->Nz < 3 || !(p->x1 > p->x0) || !(p->y1 > p->y0) || !(p->z1 > p->z0))
    return ch_fail(CH_ERR_ARG, "ch_collect_moments_noalloc: bad grid");
  const int64_t N = (int64_t)p->Nx * p->Ny * p->Nz;
  if (N > CH_NOALLOC_MAX_NODES)
    return ch_fail(CH_ERR_ARG,
                   "ch_collect_moments_noalloc: grid %dx%dx%d has %lld nodes; this entry point holds scratch for at "
                   "most %d nodes (use ch_collect_moments)",
                   p->Nx, p->Ny, p->Nz, (long long)N, CH_NOALLOC_MAX_NODES);
  unsigned long long* acc = nullptr;
  ch_status rc = noalloc_scratch(&acc);
  if (rc) return rc;
  GridDesc g;
  g.Nx = p->Nx; g.Ny = p->Ny; g.Nz = p->Nz;
  ch_grid_finish(g);
  g.x0 = p->x0; g.y0 = p->y0; g.z0 = p->z0;
  g.Lx = p->x1 - p->x0; g.Ly = p->y1 - p->y0; g.Lz = p->z1 - p->z0;
  g.dx = g.Lx / p->Nx; g.dy = g.Ly / p->Ny; g.dz = g.Lz / p->Nz;
  const double scale = ldexp(1.0, (int)(p->deposit_scale_log2 > 0.0 ? p->deposit_scale_log2 : 40.0));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int sms = 1, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // the array keeps the previous call's sums: clear it first
  k_noalloc_zero<<<sms * 4, 256, 0, s>>>(acc, 4 * N);
  if (np > 0) {
    int64_t nb = (np + 255) / 256;
    if (nb > (int64_t)sms * 8) nb = (int64_t)sms * 8;
    k_noalloc_deposit<<<(int)nb, 256, 0, s>>>(g, scale, x, y, z, vx, vy, vz, np, acc);
  }
  k_noalloc_finalize<<<sms * 4, 256, 0, s>>>(acc, 4 * N, 1.0 / scale, moments);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ch_cuda_fail(e, "ch_collect_moments_noalloc launch", __FILE__, __LINE__);
  return CH_OK;
}
