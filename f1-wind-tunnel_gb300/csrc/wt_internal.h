// Internal declarations of libwt: device data layout, kernel argument blocks
// and launchers shared by the translation units.  Not installed.
//
// Device data of one lattice (n = nx*ny*nz cells, np = n rounded up to 64):
//   pop        19*np populations, one contiguous array per direction, in the
//              AA in-place layout (see wt_lbm.cu); f32, or f - w_i as f16/bf16
//   cellw      n  u32 cell words: link bits, solid, belt, duct (wt_lattice.cuh)
//   solid      n  u8 solid group (0 fluid, 1 body, 2 front wing, 3 rear wing)
//   emit       n  f32 heat source / duct marker (VOXELIZE output)
//   fields     n  float4 (ux, uy, uz, rho), written on the last step of a call
//   tA, tB     n  f32 heat scalar ping-pong (result always ends in tA)
//   outlet_u   ny*nz float4: previous velocity of the outlet column x = nx-1
//   tau0_x     nx f32: the x-dependent base relaxation time (sponges)
//   scratch    force partial records of the pending steps + mass partials
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "wt.h"

#define WT_HIST_CAP 16384u    // per-step force records kept on the device (ring)
#define WT_PENDING_MAX 64u    // steps whose partials wait for one reduction launch
#define WT_RED_FCHUNKS 8u     // blocks per step of the force reduction
#define WT_RED_MCHUNKS 32u    // blocks of the mass reduction
// scratch doubles per lattice for the reduction's chunk sums
#define WT_RED_PART ((size_t)WT_PENDING_MAX * WT_RED_FCHUNKS * 16 + WT_RED_MCHUNKS)

namespace wt {

// Per-block force partial of one step: FP64 sums (x,y,z per group) and the
// reference's i32 fixed-point sums (x,y per group, wrapping).
struct ForceSlot {
  double f[9];
  int32_t raw[6];
};

struct StepArgs {
  void* pop;
  const uint32_t* cellw;
  const uint8_t* solid;
  float4* fields;
  float4* outlet_u;
  const float* tau0_x;
  const int32_t* block_slot;   // block -> slot or -1
  ForceSlot* slots;            // this step's partial records [nslots]
  uint32_t nslots;             // records per step (force-carrying blocks)
  double* mass_partial;        // [nblocks * warps per block] (field steps only)
  unsigned int* guard_count;
  uint32_t nx, ny, nz;
  uint64_t n, np;
  float u_in, ks2;             // ks2 = (18*1.41421356 as f32) * smag * smag
  float guard_uu;              // largest u.u whose square root rounds to <= 0.35f
  float feq_in[19];            // feq(i, 1, (u_in, 0, 0))
  float floor_k[19];           // 6 * w_i * c_ix (belt term coefficient)
  float feq_guard[19];         // feq(i, 1, (u_in/2, 0, 0)): the divergence guard's reset state
  // the same three tables as scaled deviations S (f - w_i) for f16 / bf16 storage
  // (S = 2^14 / 1), the step's working form there
  float dev_in[19], floor_kd[19], dev_guard[19];
  // Slot offsets relative to the cell index, modulo 2^32 (19 * np < 2^32):
  uint32_t own_ofs[19];        // i * np:                  pop[i][x]
  uint32_t pull_ofs[19];       // opp(i) * np - off(c_i):  pop[opp(i)][x - c_i]
  uint32_t push_ofs[19];       // i * np + off(c_i):       pop[i][x + c_i]
  uint32_t prefetch_ahead;     // blocks ahead whose rows a block prefetches into L2 (0: none)
  uint64_t pop_bytes;          // size of the population allocation
};

// Fills own_ofs / pull_ofs / push_ofs from nx, ny, np.
void fill_slot_offsets(StepArgs& a);
// The divergence guard's bound on u.u: the largest float whose square root
// rounds to <= 0.35f (length(u) > 0.35, src/engine/wgsl.ts:238).
float guard_threshold();

struct HeatArgs {
  const float4* fields;
  const float* emit;
  const float* src;  // the neighbours' largest emission (launch_heat_sources)
  const float* tin;
  float* tout;
  uint32_t nx, ny, nz;
  float dt, cool, diffuse, src_mix;
};

// Launch geometry of the step kernels.
struct StepGeom {
  dim3 block, grid;
  uint32_t nblocks;
};

StepGeom step_geometry(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t bx, uint32_t by);
// Blocks of the collide-stream kernel resident on the whole device at this block
// shape: the L2 prefetch distance, or 0 where the prefetch stays off (f16/bf16;
// f32 populations within twice the L2).
uint32_t step_resident_blocks(uint32_t storage, const StepGeom& g, uint32_t sm_count, uint64_t pop_bytes,
                              uint64_t l2_bytes);

// Block ranges of the lattices of a batch launch (see batch_step_kernel).
struct BatchTiles {
  uint32_t base;        // first block of this lattice
  uint32_t gx, gy, gz;  // the lattice's grid in blocks
};

// wt_lbm.cu
cudaError_t launch_init(uint32_t storage, void* pop, float4* fields, float4* outlet_u, uint32_t nx, uint32_t ny,
                        uint32_t nz, uint64_t np, float u_in, cudaStream_t s);
cudaError_t launch_step(uint32_t storage, bool gather, bool write_fields, const StepGeom& g, const StepArgs& a,
                        cudaStream_t s);
cudaError_t launch_batch_step(uint32_t storage, bool gather, bool write_fields, dim3 block, uint32_t total_blocks,
                              const StepArgs* args, const BatchTiles* tiles, uint32_t count, uint32_t pending,
                              cudaStream_t s);
// Persistent batch: one cooperative launch advances every lattice by nsteps
// (<= WT_PENDING_MAX) steps, step k0 + k of the call being a gather step when
// even; sync[0] is the grid barrier's counter (zero before the launch), sync[1]
// is raised if a barrier wait expires.  grid = batch_persist_blocks(...), the
// blocks that can be resident at once (0: not available).
uint32_t batch_persist_blocks(uint32_t storage, dim3 block, uint32_t sm_count);
cudaError_t launch_batch_persist(uint32_t storage, dim3 block, uint32_t grid, uint32_t total_blocks,
                                 const StepArgs* args, const BatchTiles* tiles, uint32_t count, uint32_t k0,
                                 uint32_t nsteps, uint32_t pending0, bool fields_last, unsigned int* sync,
                                 cudaStream_t s);
// Per-lattice arguments of the force reduction (one record per lattice, in device memory).
struct ReduceArgs {
  const ForceSlot* slots;
  uint32_t nslots;
  uint32_t hist_cap;
  double* hist;
  unsigned long long* hist_pos;  // steps recorded so far (advanced by the reduction itself)
  double* totals;
  int32_t* raw_totals;
  const double* mass_partial;
  uint32_t nmass;
  double* mass_out;
  unsigned int* counter;
  double* part;  // WT_RED_PART doubles: chunk sums of the force records, then of the mass
};
cudaError_t launch_force_reduce(const ReduceArgs* args, uint32_t count, uint32_t nsteps, bool with_mass,
                                cudaStream_t s);
// The force accumulators (FP64 totals[10]: sums and mass, raw i32[12], guard
// counter) into *out, a wt_forces in host-mapped memory; zeroed after if reset.
cudaError_t launch_force_readback(double* totals, int32_t* raw, unsigned int* counters, wt_forces* out,
                                  uint64_t steps, int reset, cudaStream_t s);
cudaError_t launch_read_pop(uint32_t storage, const void* pop, float* out, uint32_t n, uint64_t np, cudaStream_t s);
cudaError_t launch_write_pop(uint32_t storage, const float* in, void* pop, uint32_t n, uint64_t np, cudaStream_t s);
// Box average of the fluid cells' (ux, uy, uz, rho) onto a cx x cy x cz grid
// (fine cell i of an axis belongs to coarse cell i * c / n); boxes without fluid
// give (0, 0, 0, 1).
cudaError_t launch_coarse_average(const float4* fields, const uint32_t* cellw, uint32_t nx, uint32_t ny, uint32_t nz,
                                  float4* coarse, uint32_t cx, uint32_t cy, uint32_t cz, cudaStream_t s);
cudaError_t launch_resample_init(uint32_t storage, const float4* coarse, uint32_t cx, uint32_t cy, uint32_t cz,
                                 void* pop, float4* fields, float4* outlet_u, uint32_t nx, uint32_t ny, uint32_t nz,
                                 uint64_t np, cudaStream_t s);

// wt_voxel.cu
// The baked W17 model's device buffers (wt_set_car_model); empty = no model.
struct CarView {
  const uint16_t* body = nullptr;   // 368 x 84 x 67 binary16 body distances, x fastest
  const uint16_t* parts = nullptr;  // parts atlas, pdims[0] x [1] x [2] binary16, x fastest
  uint32_t pdims[3] = {1, 1, 1};
  const float4* rig = nullptr;      // the Rig uniform: front[71], hinges, angles, extra, fly, grids[12]
};

cudaError_t launch_voxelize(const wt_shape& shape, const CarView& car, const wt_grid& grid, uint8_t* solid, float* emit,
                            cudaStream_t s);
cudaError_t launch_sdf_sample(const wt_shape& shape, const wt_grid& grid, float* out, cudaStream_t s);
cudaError_t launch_cell_words(const uint8_t* solid, const float* emit, uint32_t* cellw, uint32_t nx, uint32_t ny,
                              uint32_t nz, cudaStream_t s);
cudaError_t launch_block_flags(const uint32_t* cellw, const StepGeom& g, uint32_t nx, uint32_t ny, uint32_t nz,
                               uint8_t* flags, cudaStream_t s);
cudaError_t launch_links_out(const uint32_t* cellw, uint32_t* links, uint64_t n, cudaStream_t s);
cudaError_t launch_solid_u32(const uint8_t* solid, uint32_t* out, uint64_t n, cudaStream_t s);
cudaError_t launch_solid_from_u32(const uint32_t* in, uint8_t* solid, uint64_t n, cudaStream_t s);

// wt_heat.cu
cudaError_t launch_heat(const HeatArgs& a, cudaStream_t s);
cudaError_t launch_heat_sources(const float* emit, float* src, uint32_t nx, uint32_t ny, uint32_t nz, cudaStream_t s);

// wt_conv.cu: last error of the calling thread in the network operators (wt_net.h)
std::string& net_error();

}  // namespace wt
