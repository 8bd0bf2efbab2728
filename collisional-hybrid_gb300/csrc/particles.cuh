// particles.cuh -- ion state layouts and host launchers of particles.cu.
#pragma once

#include "common.cuh"

namespace ch {

enum { PH_PUSH = 1, PH_MOVE = 2, PH_DEPOSIT = 4 };

struct F64Particles {
  double *x, *y, *z, *vx, *vy, *vz;
  uint32_t* id;
  int64_t np;
};

struct MixParticles {
  float4* pos;  // (ox, oy, oz, packed cell bits)
  float4* vel;  // (vx, vy, vz, id bits)
  int64_t np;
};

// Launch configuration: grid-stride kernels sized to a multiple of the SM count.
int grid_for(int64_t n, int threads, int sms, int per_sm);

void launch_load(bool mixed, const GridDesc& g, const ch_loader& L, uint64_t seed, uint32_t run, F64Particles P,
                 MixParticles M, int sms, cudaStream_t s);
void launch_aos_in(bool mixed, const GridDesc& g, const double4_32a* pos, const double4_32a* vel, F64Particles P,
                   MixParticles M, int sms, cudaStream_t s);
void launch_aos_out(bool mixed, const GridDesc& g, F64Particles P, MixParticles M, double4_32a* pos, double4_32a* vel,
                    int sms, cudaStream_t s);
void launch_node_efield(bool mixed, const GridDesc& g, double tscale, const double* phi, double* E64, float4* E32,
                        int sms, cudaStream_t s);
// PUSH/MOVE/DEPOSIT mask; part receives nblocks x 2 partials (expected, S next).
// Mixed form: a brick-tiled kernel over the cell-sorted ions (starts = first
// slot of each cell at the last sort); hist (nullable) counts the ions' new
// cells for the next sort.
int launch_pass(bool mixed, int phases, const StepConsts& c, F64Particles P, MixParticles M, const double* E64,
                const float4* E32, const double* phi, unsigned long long* acc, double Nc, double sbar,
                DevCounters* cnt, double* part, const uint32_t* starts, uint32_t* hist, int sms, cudaStream_t s);
int launch_sbar(bool mixed, const StepConsts& c, F64Particles P, MixParticles M, double* part, int sms,
                cudaStream_t s);
void launch_reduce_partials(const double* part, int nblocks, int K, double* out, cudaStream_t s);
int launch_finalize(int64_t N, unsigned long long* acc, double inv_scale, int reset, double* mom, double* part,
                    DevCounters* cnt, int sms, cudaStream_t s);
// Counting sort by cell: counts (N), starts (N+1), cursor (N), keys (np),
// block_sums (ceil(N/1024)+1).  Results land in the Q buffers.
// have_hist: counts already hold the per-cell ion counts (mixed form, counted
// by the preceding pass).
void launch_sort(bool mixed, const GridDesc& g, F64Particles P, F64Particles Q, MixParticles M, MixParticles MQ,
                 uint32_t* counts, uint32_t* starts, uint32_t* cursor, uint32_t* keys, uint32_t* block_sums,
                 bool have_hist, int sms, cudaStream_t s);

}  // namespace ch
