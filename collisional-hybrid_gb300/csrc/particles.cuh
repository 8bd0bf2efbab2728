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
  uint32_t* rank;  // nullable: a pass that counts new cells stores each ion's rank in its cell here
};

// Launch configuration: grid-stride kernels sized to a multiple of the SM count.
int grid_for(int64_t n, int threads, int sms, int per_sm);

void launch_load(bool mixed, const GridDesc& g, const ch_loader& L, uint64_t seed, uint32_t run, F64Particles P,
                 MixParticles M, int sms, cudaStream_t s);
void launch_aos_in(bool mixed, const GridDesc& g, const double4_32a* pos, const double4_32a* vel, F64Particles P,
                   MixParticles M, int sms, cudaStream_t s);
// Copies bytes (a multiple of 16; both pointers 16-byte aligned) on the SMs;
// dst may be mapped host memory.
// AoS arrays (16-byte aligned; mapped host memory for the upload) in ion-id
// order: the slot map of the current order, the conversion of an id range,
// and the upload that puts every ion back into its slot.
void launch_slot_map(MixParticles M, uint32_t* slot_of_id, int sms, cudaStream_t s);
// The reference's --density-type placements (CH_DENSITY_FLAT_SOBOL,
// CH_DENSITY_UNIFORM, CH_DENSITY_SINUSOIDAL) with Maxwellian velocities.
void launch_load_placed(bool mixed, const GridDesc& g, const ch_loader& L, int type, uint64_t seed, uint32_t run,
                        F64Particles P, MixParticles M, int sms, cudaStream_t s);
// One step's push / collisions / move of ions held in registered host arrays
// (id order, read and written in place through their device addresses);
// returns the number of blocks, whose 3 partials (expected events, S after
// the push, S of the ions read) are in part.
int launch_host_push(const StepConsts& c, void* pos, void* vel, const uint32_t* slot_of_id, MixParticles M,
                     MixParticles B, const float4* E32, double Nc, double sbar, uint32_t* hist, bool read, bool write,
                     DevCounters* cnt, double* part, int sms, cudaStream_t s);
void launch_mixed_to_host(const GridDesc& g, MixParticles M, const uint32_t* slot_of_id, void* pos, void* vel,
                          int64_t i_begin, int64_t i_end, int sms, cudaStream_t s);
void launch_host_to_mixed(const GridDesc& g, const void* pos, const void* vel, const uint32_t* slot_of_id,
                          MixParticles M, int sms, cudaStream_t s);
void launch_stream_copy(void* dst, const void* src, uint64_t bytes, int sms, cudaStream_t s);
// AoS in from 16-byte aligned arrays that the device can read directly
// (mapped host memory).
void launch_aos_in_u16(bool mixed, const GridDesc& g, const void* pos, const void* vel, F64Particles P,
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
// block_sums (ceil(N/1024)+1).
// Exclusive scan of the cell counts into starts (and cursor).
void launch_scan(int64_t N, const uint32_t* counts, uint32_t* starts, uint32_t* cursor, uint32_t* block_sums,
                 cudaStream_t s);
// The deposit of a step that ends with a sort, fused with the sort's scatter
// of M (order of starts) into MQ (order of dst_starts, ranks in M.rank).
void launch_deposit_sort(const StepConsts& c, MixParticles M, MixParticles MQ, const uint32_t* starts,
                         const uint32_t* dst_starts, unsigned long long* acc, DevCounters* cnt, int sms,
                         cudaStream_t s);
// Counting sort of P (FP64 form) or M (mixed) into Q / MQ: cell count,
// scan, scatter with atomic cursors.  The mixed step's own sort is the scan
// plus launch_deposit_sort, whose push counted the cells and ranks.
void launch_sort(bool mixed, const GridDesc& g, F64Particles P, F64Particles Q, MixParticles M, MixParticles MQ,
                 uint32_t* counts, uint32_t* starts, uint32_t* cursor, uint32_t* keys, uint32_t* block_sums, int sms,
                 cudaStream_t s);

// ------------------------------------------------------------------ ensembles
// One run of a batch (independent runs of different grids and parameters
// that share the device arrays): its constants and its slices.  Grid arrays
// of run r start at node_off (acc and mom: 4 x N_r SoA from 4 x node_off).
struct BatchRunDev {
  StepConsts c;       // c.step is set by the pass
  int64_t node_off;
  int64_t ion_off, np;
  int tile_off, ntiles;
  double Nc;          // collisions per step (src/particles.c:510-519)
};
struct BatchDev {
  const BatchRunDev* runs;
  const int* tile_off;     // nruns + 1 prefix sums of bricks
  const int64_t* ion_off;  // nruns + 1 prefix sums of ions
  int nruns;
  int total_tiles;
};
// Bricks of a run's grid in the tiled pass.
int tiles_of(const GridDesc& g);
// The fused pass over every run's bricks in one persistent launch.  Per
// brick 4 partials (expected events, S next, collisions, refused) land in
// tile_part; flags[r] |= 16 for a non-finite ion of run r.  hist (nullable)
// counts the ions' new cells over the batch grid.
// The step number is read from *dstep (device), so a captured step can be
// replayed.  phases: PH_DEPOSIT alone (CollectVlasovQuantities), PH_PUSH |
// PH_MOVE, or all three.  Brick partials (tile_part) come from the push.
void batch_pass_prepare();  // once, before any capture
void launch_batch_pass(int phases, const BatchDev& B, const uint32_t* dstep, MixParticles P, const float4* E,
                       const uint32_t* starts, unsigned long long* acc, const double* sbar, int dep_log2,
                       uint32_t* hist, double* tile_part, int* flags, int ctas_per_sm, int sms, cudaStream_t s,
                       MixParticles Q = MixParticles{}, const uint32_t* dst_starts = nullptr);
// sums[4r + q] = the run's brick partials summed in a fixed order; sbar[r] =
// S for the next step (runs with collisions); flags[r] |= 8 at the refusal
// limit; *dstep advances by one.
void launch_batch_runsum(const BatchDev& B, const double* tile_part, double* sums, double* sbar, int* flags,
                         uint32_t* dstep, cudaStream_t s);
// Cell counts of every run's ions over the batch grid (counts zeroed first).
void launch_batch_hist(const BatchDev& B, MixParticles M, uint32_t* counts, int sms, cudaStream_t s);
// acc -> mom elementwise (n4 = 4 x batch nodes), acc cleared; flag |= 1 if a
// sum is out of the fixed-point range.
void launch_batch_finalize(int64_t n4, unsigned long long* acc, double inv_scale, double* mom, int* flag, int sms,
                           cudaStream_t s);
// Counting sort over the batch grid (keys node_off[r] + cell keep the runs
// contiguous); counts hold the cell counts.
void launch_batch_sort(const BatchDev& B, int64_t Ntot, MixParticles M, MixParticles MQ, uint32_t* counts,
                       uint32_t* starts, uint32_t* cursor, uint32_t* block_sums, int sms, cudaStream_t s);

}  // namespace ch
