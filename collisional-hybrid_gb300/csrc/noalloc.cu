// noalloc.cu -- a cloud-in-cell deposit that allocates no memory.
//
// ch_collect_moments needs a ch_ctx, whose creation allocates device
// buffers.  Some callers cannot allocate: a host whose device memory is all
// owned by its own pool allocator (a framework that reserves the GPU's memory
// up front and hands out sub-blocks), or a time-critical loop that cannot
// afford the implicit device synchronisation of cudaMalloc/cudaFree.
// ch_collect_moments_noalloc serves them: the caller passes device pointers
// for the ions and the output moments, and the only scratch the deposit
// needs -- its 64-bit fixed-point accumulators -- lives in a fixed array in
// this file, sized for grids of at most CH_NOALLOC_MAX_NODES nodes.
#include <mutex>

#include "common.cuh"
#include "ion_dev.cuh"

// 64^3 nodes: 4 moments x 2^18 nodes x 8 bytes = 8 MiB, held by every GPU
// that loads this library until the process exits.
#define CH_NOALLOC_MAX_NODES (1 << 18)
#define CH_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned long long g_noalloc_acc[4 * CH_NOALLOC_MAX_NODES];
// Error bits of the call in flight: 1 = an ion with a non-finite position or
// velocity, 2 = an ion outside the fixed-point or cell-index range, 4 = a
// density sum outside the fixed-point range.  Cleared at the start of every
// call; device code names it directly.
static __device__ unsigned int g_noalloc_status;

// Device address of g_noalloc_acc per device.  In host code the array's name
// is only a host-side stand-in, so the address is looked up once per device
// with that device current (in its primary context).
static unsigned long long* g_noalloc_dev[CH_NOALLOC_MAX_DEVICES] = {};
static std::mutex g_noalloc_mu;

namespace {

__global__ void k_noalloc_zero(unsigned long long* __restrict__ acc, int64_t n) {
  if (blockIdx.x == 0 && threadIdx.x == 0) g_noalloc_status = 0u;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    acc[c] = 0ull;
}

// The FP64 deposit of CollectVlasovQuantities (src/particles.c:189-235): the
// same CIC weights and fixed-point sums (deposit_cic) as ch_collect_moments,
// so finite, in-range ions give bit-identical moments.  An ion that would
// give a meaningless or undefined contribution is skipped and flagged.
__global__ void k_noalloc_deposit(GridDesc g, double scale, double vmax, const double* __restrict__ x,
                                  const double* __restrict__ y, const double* __restrict__ z,
                                  const double* __restrict__ vx, const double* __restrict__ vy,
                                  const double* __restrict__ vz, int64_t np, unsigned long long* __restrict__ acc) {
  unsigned int bad = 0u;
  for (int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ip < np; ip += (int64_t)gridDim.x * blockDim.x) {
    const double v0 = vx[ip], v1 = vy[ip], v2 = vz[ip];
    const double X = (x[ip] - g.x0) / g.dx, Y = (y[ip] - g.y0) / g.dy, Z = (z[ip] - g.z0) / g.dz;
    if (!(isfinite(X) && isfinite(Y) && isfinite(Z) && isfinite(v0) && isfinite(v1) && isfinite(v2))) {
      bad |= 1u;
      continue;
    }
    // the cell index must fit an int before the periodic wrap, and one
    // contribution |v| w 2^s must fit the 64-bit accumulator word
    if (fabs(X) >= 1073741824.0 || fabs(Y) >= 1073741824.0 || fabs(Z) >= 1073741824.0 || fabs(v0) >= vmax ||
        fabs(v1) >= vmax || fabs(v2) >= vmax) {
      bad |= 2u;
      continue;
    }
    const double fi = floor(X), fj = floor(Y), fk = floor(Z);
    ch::deposit_cic<double>(g, acc, ch_wrap((int)fi, g.Nx), ch_wrap((int)fj, g.Ny), ch_wrap((int)fk, g.Nz),
                            X - fi, Y - fj, Z - fk, v0, v1, v2, scale);
  }
  if (bad) atomicOr(&g_noalloc_status, bad);
}

// Fixed point -> FP64, with the density range check of k_finalize_moments:
// density contributions are non-negative, so a wrapped sum shows up as a
// negative or near-limit word.
__global__ void k_noalloc_finalize(const unsigned long long* __restrict__ acc, int64_t N, double inv_scale,
                                   double* __restrict__ out) {
  unsigned int bad = 0u;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < 4 * N; c += (int64_t)gridDim.x * blockDim.x) {
    const long long a = (long long)acc[c];
    if (c < N && (a < 0 || a > (1LL << 61))) bad = 4u;
    out[c] = (double)a * inv_scale;
  }
  if (bad) atomicOr(&g_noalloc_status, bad);
}

// A flagged call overwrites every output with NaN: the asynchronous form of
// the CH_ERR_NAN / CH_ERR_RANGE that ch_collect_moments returns.
__global__ void k_noalloc_poison(int64_t n4, double* __restrict__ out) {
  if (*(volatile unsigned int*)&g_noalloc_status == 0u) return;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n4; c += (int64_t)gridDim.x * blockDim.x)
    out[c] = __longlong_as_double(0x7ff8000000000000LL);
}

}  // namespace

// Looks up the device address of the scratch array for the current device,
// once per device.
static ch_status noalloc_scratch(int dev, unsigned long long** out) {
  if (dev < 0 || dev >= CH_NOALLOC_MAX_DEVICES)
    return ch_fail(CH_ERR_UNSUPPORTED, "device %d: at most %d devices", dev, CH_NOALLOC_MAX_DEVICES);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_dev[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_acc);
    if (e != cudaSuccess) return ch_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_acc)", __FILE__, __LINE__);
    g_noalloc_dev[dev] = static_cast<unsigned long long*>(ptr);
  }
  *out = g_noalloc_dev[dev];
  return CH_OK;
}

extern "C" ch_status ch_collect_moments_noalloc(const ch_params* p, const double* x, const double* y,
                                                const double* z, const double* vx, const double* vy,
                                                const double* vz, int64_t np, double* moments, void* stream) {
  // every argument check comes before the first CUDA call
  if (!p || !moments || (np > 0 && (!x || !y || !z || !vx || !vy || !vz)))
    return ch_fail(CH_ERR_ARG, "ch_collect_moments_noalloc: null argument");
  if (np < 0) return ch_fail(CH_ERR_ARG, "ch_collect_moments_noalloc: np < 0");
  if (p->Nx < 3 || p->Ny < 3 || p->Nz < 3)
    return ch_fail(CH_ERR_ARG, "ch_collect_moments_noalloc: grid %dx%dx%d: each axis needs at least 3 nodes",
                   p->Nx, p->Ny, p->Nz);
  // each axis first, so that the node count below cannot overflow
  if (p->Nx > CH_NOALLOC_MAX_NODES || p->Ny > CH_NOALLOC_MAX_NODES || p->Nz > CH_NOALLOC_MAX_NODES ||
      (int64_t)p->Nx * p->Ny * p->Nz > CH_NOALLOC_MAX_NODES)
    return ch_fail(CH_ERR_ARG,
                   "ch_collect_moments_noalloc: grid %dx%dx%d exceeds the scratch of this entry point, which holds at "
                   "most %d nodes (use ch_collect_moments)",
                   p->Nx, p->Ny, p->Nz, CH_NOALLOC_MAX_NODES);
  if (!(p->x1 > p->x0) || !(p->y1 > p->y0) || !(p->z1 > p->z0) || !isfinite(p->x1 - p->x0) ||
      !isfinite(p->y1 - p->y0) || !isfinite(p->z1 - p->z0) || !isfinite(p->x0) || !isfinite(p->y0) ||
      !isfinite(p->z0))
    return ch_fail(CH_ERR_ARG, "ch_collect_moments_noalloc: empty or non-finite domain");
  // the FP64 form's scale range of ch_create
  if (p->deposit_scale_log2 != 0.0 && !(p->deposit_scale_log2 >= 1.0 && p->deposit_scale_log2 <= 62.0))
    return ch_fail(CH_ERR_ARG, "ch_collect_moments_noalloc: deposit_scale_log2 %g outside [1, 62]",
                   p->deposit_scale_log2);
  const int64_t N = (int64_t)p->Nx * p->Ny * p->Nz;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return ch_cuda_fail(e, "cudaGetDevice", __FILE__, __LINE__);
  unsigned long long* acc = nullptr;
  ch_status rc = noalloc_scratch(dev, &acc);
  if (rc) return rc;
  GridDesc g;
  g.Nx = p->Nx; g.Ny = p->Ny; g.Nz = p->Nz;
  ch_grid_finish(g);
  g.x0 = p->x0; g.y0 = p->y0; g.z0 = p->z0;
  g.Lx = p->x1 - p->x0; g.Ly = p->y1 - p->y0; g.Lz = p->z1 - p->z0;
  g.dx = g.Lx / p->Nx; g.dy = g.Ly / p->Ny; g.dz = g.Lz / p->Nz;
  const int s2 = (int)(p->deposit_scale_log2 > 0.0 ? p->deposit_scale_log2 : 48.0);  // the FP64 form's default
  const double scale = ldexp(1.0, s2);
  // |v| w 2^s < 2^62 for every weight w <= 1
  const double vmax = ldexp(1.0, 62 - s2);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int sms = 1;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return ch_cuda_fail(e, "cudaDeviceGetAttribute", __FILE__, __LINE__);
  // the array keeps the previous call's sums: clear it (and the status) first
  k_noalloc_zero<<<sms * 4, 256, 0, s>>>(acc, 4 * N);
  if (np > 0) {
    int64_t nb = (np + 255) / 256;
    if (nb > (int64_t)sms * 8) nb = (int64_t)sms * 8;
    k_noalloc_deposit<<<(int)nb, 256, 0, s>>>(g, scale, vmax, x, y, z, vx, vy, vz, np, acc);
  }
  k_noalloc_finalize<<<sms * 4, 256, 0, s>>>(acc, N, 1.0 / scale, moments);
  k_noalloc_poison<<<sms * 4, 256, 0, s>>>(4 * N, moments);
  e = cudaGetLastError();
  if (e != cudaSuccess) return ch_cuda_fail(e, "ch_collect_moments_noalloc launch", __FILE__, __LINE__);
  return CH_OK;
}
