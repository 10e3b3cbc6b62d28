// The C ABI of the block-shape autotuner and of batches (many lattices advanced
// by one kernel launch per step: the aero-map sweep, src/ui/aeromap.ts:73-114).
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "wt_ctx.h"
#include "wt_fmath.h"
#include "wt_internal.h"
#include "wt_fields.h"
#include "wt_render.h"
#include "wt_mesh.h"
#include "wt_lattice.cuh"

using namespace wt;
using namespace wt::api;

// ---------------------------------------------------------------------------
// Autotuner: time the step kernel under each candidate block shape and keep
// the fastest.  The lattice state (populations, fields, outlet velocities,
// force accumulators and history position) is saved before and restored after,
// so tuning does not advance the simulation.
// ---------------------------------------------------------------------------
namespace {

const uint32_t kShapes[][2] = {{128, 1}, {64, 2}, {32, 4}, {256, 1}, {128, 2}, {64, 4}, {32, 8}};

struct Saved {
  void* pop = nullptr;
  float4* fields = nullptr;
  float4* outlet = nullptr;
  double totals[18];
  int32_t raw[12];
  unsigned int counters[4];
  unsigned long long hist_pos = 0;
};

int save_state(wt_ctx* c, Saved& sv) {
  if (int rc = flush_forces(c)) return rc;
  const size_t pb = 19 * c->np * c->elem;
  WT_CUDA(c, cudaMallocAsync(&sv.pop, pb, c->stream));
  WT_CUDA(c, cudaMallocAsync((void**)&sv.fields, c->n * 16, c->stream));
  WT_CUDA(c, cudaMallocAsync((void**)&sv.outlet, (size_t)c->ny * c->nz * 16, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(sv.pop, c->pop, pb, cudaMemcpyDeviceToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(sv.fields, c->fields, c->n * 16, cudaMemcpyDeviceToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(sv.outlet, c->outlet_u, (size_t)c->ny * c->nz * 16, cudaMemcpyDeviceToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(sv.totals, c->totals, sizeof(sv.totals), cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(sv.raw, c->raw_totals, sizeof(sv.raw), cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(sv.counters, c->counters, sizeof(sv.counters), cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(&sv.hist_pos, c->hist_pos, 8, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

int restore_state(wt_ctx* c, Saved& sv) {
  const size_t pb = 19 * c->np * c->elem;
  WT_CUDA(c, cudaMemcpyAsync(c->pop, sv.pop, pb, cudaMemcpyDeviceToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(c->fields, sv.fields, c->n * 16, cudaMemcpyDeviceToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(c->outlet_u, sv.outlet, (size_t)c->ny * c->nz * 16, cudaMemcpyDeviceToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(c->totals, sv.totals, sizeof(sv.totals), cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(c->raw_totals, sv.raw, sizeof(sv.raw), cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(c->counters, sv.counters, sizeof(sv.counters), cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(c->hist_pos, &sv.hist_pos, 8, cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaFreeAsync(sv.pop, c->stream));
  WT_CUDA(c, cudaFreeAsync(sv.fields, c->stream));
  WT_CUDA(c, cudaFreeAsync(sv.outlet, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  c->pending = 0;  // the trial steps' records are dropped with them
  c->mass_pending = false;
  return WT_OK;
}

// ms per LBM step of `step(n)` on stream s (events around `reps` calls of 16 steps)
template <class Step>
float time_steps(cudaStream_t s, Step&& step) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  if (step(2) != WT_OK) return -1.0f;  // capture + warm
  cudaEventRecord(a, s);
  for (int r = 0; r < 3; r++)
    if (step(16) != WT_OK) return -1.0f;
  cudaEventRecord(b, s);
  cudaEventSynchronize(b);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / 48.0f;
}

}  // namespace

extern "C" {

int wt_tune(wt_ctx* c, uint32_t* bx_out, uint32_t* by_out, float* ms_out) {
  int rc = check_ctx(c);
  if (rc) return rc;
  Saved sv;
  if ((rc = save_state(c, sv))) return rc;
  const uint64_t steps_total = c->steps_total, since = c->steps_since_read, rec = c->steps_recorded;
  float best = 1e30f;
  uint32_t bbx = c->bx, bby = c->by;
  for (auto& sh : kShapes) {
    if ((rc = set_geometry(c, sh[0], sh[1]))) return rc;
    const float ms = time_steps(c->stream, [&](int n) { return wt_step(c, n, 0, 0.0f); });
    if (ms > 0.0f && ms < best) {
      best = ms;
      bbx = c->bx;
      bby = c->by;
    }
  }
  if ((rc = set_geometry(c, bbx, bby))) return rc;
  if ((rc = restore_state(c, sv))) return rc;
  c->steps_total = steps_total;
  c->steps_since_read = since;
  c->steps_recorded = rec;
  if (bx_out) *bx_out = bbx;
  if (by_out) *by_out = bby;
  if (ms_out) *ms_out = best;
  return WT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: many lattices advanced by one kernel launch per step.
// ---------------------------------------------------------------------------
namespace {

int bfail(wt_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  else g_create_error = m;
  return code;
}

#define WT_BCUDA(b, call)                                                                                 \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess) return bfail((b), WT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

uint64_t batch_version(const wt_batch* b) {
  uint64_t v = ((uint64_t)b->bx << 32) ^ ((uint64_t)b->by << 48) ^ ((uint64_t)b->persist << 62);
  for (auto* c : b->lat) v = v * 1000003ull + c->version + ((uint64_t)c->bx << 40) + ((uint64_t)c->by << 52);
  return v;
}

// Device tables (per-lattice step arguments, block ranges, reduction records).
// Every member first takes the batch's block shape (the launch uses b->bx x b->by
// for all lattices, and each member's block map and per-warp buffers are sized
// for its own shape); only then is the table version compared.
int refresh_batch(wt_batch* b) {
  for (auto* c : b->lat) {
    if (c->bx != b->bx || c->by != b->by) {
      int rc = set_geometry(c, b->bx, b->by);
      if (rc) return bfail(b, rc, c->err);
      if (c->bx != b->bx || c->by != b->by) return bfail(b, WT_ERR_ARG, "batch block shape not accepted");
    }
  }
  const uint64_t v = batch_version(b);
  if (v == b->version) return WT_OK;
  const size_t count = b->lat.size();
  std::vector<StepArgs> args(count);
  std::vector<BatchTiles> tiles(count);
  std::vector<ReduceArgs> red(count);
  uint32_t base = 0, cap = WT_PENDING_MAX;
  for (size_t i = 0; i < count; i++) {
    wt_ctx* c = b->lat[i];
    args[i] = step_args(c);
    tiles[i].base = base;
    tiles[i].gx = c->geom.grid.x;
    tiles[i].gy = c->geom.grid.y;
    tiles[i].gz = c->geom.grid.z;
    base += c->geom.nblocks;
    red[i] = reduce_args(c);
    if (c->pending_cap < cap) cap = c->pending_cap;
  }
  b->total_blocks = base;
  b->pending_cap = cap;
  b->persist_grid = std::min(base, batch_persist_blocks(b->storage, dim3(b->bx, b->by, 1), b->lat[0]->sm_count));
  WT_BCUDA(b, cudaMemcpyAsync(b->d_args, args.data(), count * sizeof(StepArgs), cudaMemcpyHostToDevice, b->stream));
  WT_BCUDA(b, cudaMemcpyAsync(b->d_tiles, tiles.data(), count * sizeof(BatchTiles), cudaMemcpyHostToDevice, b->stream));
  WT_BCUDA(b, cudaMemcpyAsync(b->d_reduce, red.data(), count * sizeof(ReduceArgs), cudaMemcpyHostToDevice, b->stream));
  WT_BCUDA(b, cudaStreamSynchronize(b->stream));
  b->version = batch_version(b);
  return WT_OK;
}

cudaError_t enqueue_batch(wt_batch* b, int n, int heat_passes, float dt, cudaStream_t s) {
  const uint32_t count = (uint32_t)b->lat.size();
  const dim3 block(b->bx, b->by, 1);
  for (auto* c : b->lat)  // the tables were built for exactly this shape
    if (c->geom.block.x != block.x || c->geom.block.y != block.y) return cudaErrorInvalidConfiguration;
  uint32_t pending = 0;
  if (b->persist && b->persist_grid) {
    // one cooperative launch per run of steps that fills the force records
    for (uint32_t k = 0; k < (uint32_t)n;) {
      const uint32_t chunk = std::min((uint32_t)n - k, b->pending_cap - pending);
      const bool last = k + chunk == (uint32_t)n;
      cudaError_t e = cudaMemsetAsync(b->d_sync, 0, sizeof(unsigned int), s);
      if (e == cudaSuccess)
        e = launch_batch_persist(b->storage, block, b->persist_grid, b->total_blocks, b->d_args, b->d_tiles, count, k,
                                 chunk, pending, last, b->d_sync, s);
      if (e != cudaSuccess) return e;
      pending += chunk;
      k += chunk;
      if (pending == b->pending_cap || last) {
        e = launch_force_reduce(b->d_reduce, count, pending, last, s);
        if (e != cudaSuccess) return e;
        pending = 0;
      }
    }
    // the barrier's expiry flag, read back by the next call
    cudaError_t e = cudaMemcpyAsync(b->h_flag, b->d_sync + 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
  } else {
    for (int k = 0; k < n; k++) {
      const bool last = (k == n - 1);
      cudaError_t e = launch_batch_step(b->storage, (k & 1) == 0, last, block, b->total_blocks, b->d_args,
                                        b->d_tiles, count, pending, s);
      if (e != cudaSuccess) return e;
      pending++;
      if (pending == b->pending_cap || last) {
        e = launch_force_reduce(b->d_reduce, count, pending, last, s);
        if (e != cudaSuccess) return e;
        pending = 0;
      }
    }
  }
  for (auto* c : b->lat) {
    cudaError_t e = enqueue_heat(c, heat_passes, dt, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

extern "C" {

int wt_batch_create(const wt_grid* grids, uint32_t count, const wt_sim* sim, wt_batch** out) {
  if (!grids || !sim || !out || count == 0 || count > 1024) return bfail(nullptr, WT_ERR_ARG, "wt_batch_create: bad arguments");
  *out = nullptr;
  wt_batch* b = new wt_batch();
  cudaGetDevice(&b->device);
  b->storage = sim->storage;
  auto cleanup = [&](int code) { std::string m = b->err; wt_batch_destroy(b); g_create_error = m; return code; };
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { b->err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e); return cleanup(WT_ERR_CUDA); }
  for (uint32_t i = 0; i < count; i++) {
    wt_ctx* c = nullptr;
    int rc = create_ctx(&grids[i], sim, b->stream, &c);
    if (rc) { b->err = "lattice " + std::to_string(i) + ": " + g_create_error; return cleanup(rc); }
    b->lat.push_back(c);
  }
  if (cudaMalloc((void**)&b->d_args, count * sizeof(StepArgs)) != cudaSuccess ||
      cudaMalloc((void**)&b->d_tiles, count * sizeof(BatchTiles)) != cudaSuccess ||
      cudaMalloc((void**)&b->d_reduce, count * sizeof(ReduceArgs)) != cudaSuccess ||
      cudaMalloc((void**)&b->d_sync, 2 * sizeof(unsigned int)) != cudaSuccess ||
      cudaHostAlloc((void**)&b->h_flag, sizeof(unsigned int), cudaHostAllocDefault) != cudaSuccess) {
    b->err = "wt_batch_create: device tables";
    return cleanup(WT_ERR_NOMEM);
  }
  *b->h_flag = 0u;
  if (cudaMemsetAsync(b->d_sync, 0, 2 * sizeof(unsigned int), b->stream) != cudaSuccess) {
    b->err = "wt_batch_create: cudaMemsetAsync";
    return cleanup(WT_ERR_CUDA);
  }
  if (const char* e = getenv("WT_BATCH_PERSIST")) b->persist = atoi(e) != 0;
  int rc = refresh_batch(b);
  if (rc) return cleanup(rc);
  *out = b;
  return WT_OK;
}

int wt_batch_destroy(wt_batch* b) {
  if (!b) return WT_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
  for (auto* c : b->lat) wt_destroy(c);
  if (b->d_args) cudaFree(b->d_args);
  if (b->d_tiles) cudaFree(b->d_tiles);
  if (b->d_reduce) cudaFree(b->d_reduce);
  if (b->d_sync) cudaFree(b->d_sync);
  if (b->h_flag) cudaFreeHost(b->h_flag);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return WT_OK;
}

uint32_t wt_batch_count(const wt_batch* b) { return b ? (uint32_t)b->lat.size() : 0u; }

wt_ctx* wt_batch_lattice(wt_batch* b, uint32_t i) { return (b && i < b->lat.size()) ? b->lat[i] : nullptr; }

int wt_batch_step(wt_batch* b, int n_lbm_steps, int heat_passes, float heat_dt) {
  if (!b) return WT_ERR_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, WT_ERR_CUDA, "cudaSetDevice");
  if (n_lbm_steps < 2 || (n_lbm_steps & 1)) return bfail(b, WT_ERR_ARG, "wt_batch_step: n_lbm_steps must be even and >= 2");
  if (heat_passes < 0 || (heat_passes & 1)) return bfail(b, WT_ERR_ARG, "wt_batch_step: heat_passes must be 0 or even");
  if (*b->h_flag) {  // written by an earlier call's persistent launch (see enqueue_batch)
    *b->h_flag = 0u;
    return bfail(b, WT_ERR_CUDA, "wt_batch_step: a grid barrier of the persistent launch timed out");
  }
  int rc = refresh_batch(b);
  if (rc) return rc;
  const float dt = heat_dt > 0.0f ? heat_dt : (float)n_lbm_steps / 2.0f;
  for (auto* c : b->lat)
    if ((rc = flush_forces(c))) return bfail(b, rc, c->err);
  if ((rc = run_graphed(b, b->graphs, b->version, n_lbm_steps, heat_passes, dt, 0u,
                        [&](cudaStream_t s) { return enqueue_batch(b, n_lbm_steps, heat_passes, dt, s); })))
    return rc;
  for (auto* c : b->lat) {
    c->steps_total += n_lbm_steps;
    c->steps_since_read += n_lbm_steps;
    c->steps_recorded += n_lbm_steps;
  }
  return WT_OK;
}

int wt_batch_tune(wt_batch* b, uint32_t* bx_out, uint32_t* by_out, float* ms_out) {
  if (!b) return WT_ERR_ARG;
  std::vector<Saved> sv(b->lat.size());
  std::vector<uint64_t> keep(3 * b->lat.size());
  for (size_t i = 0; i < b->lat.size(); i++) {
    wt_ctx* c = b->lat[i];
    int rc = save_state(c, sv[i]);
    if (rc) return bfail(b, rc, c->err);
    keep[3 * i] = c->steps_total; keep[3 * i + 1] = c->steps_since_read; keep[3 * i + 2] = c->steps_recorded;
  }
  float best = 1e30f;
  uint32_t bbx = b->bx, bby = b->by;
  bool bpersist = b->persist;
  // launch per step, and the persistent launch, unless WT_BATCH_PERSIST fixes it
  std::vector<bool> modes{b->persist};
  if (!getenv("WT_BATCH_PERSIST")) modes = {false, true};
  for (auto& sh : kShapes) {
    for (bool persist : modes) {
      b->bx = sh[0];
      b->by = sh[1];
      b->persist = persist;
      const float ms = time_steps(b->stream, [&](int n) { return wt_batch_step(b, n, 0, 0.0f); });
      if (ms > 0.0f && ms < best) {
        best = ms;
        bbx = b->bx;
        bby = b->by;
        bpersist = persist;
      }
    }
  }
  b->bx = bbx;
  b->by = bby;
  b->persist = bpersist;
  int rc = refresh_batch(b);
  if (rc) return rc;
  for (size_t i = 0; i < b->lat.size(); i++) {
    wt_ctx* c = b->lat[i];
    if ((rc = restore_state(c, sv[i]))) return bfail(b, rc, c->err);
    c->steps_total = keep[3 * i]; c->steps_since_read = keep[3 * i + 1]; c->steps_recorded = keep[3 * i + 2];
  }
  if (bx_out) *bx_out = bbx;
  if (by_out) *by_out = bby;
  if (ms_out) *ms_out = best;
  return WT_OK;
}

void* wt_batch_stream(wt_batch* b) { return b ? (void*)b->stream : nullptr; }

uint32_t wt_batch_persistent_grid(const wt_batch* b) { return (b && b->persist) ? b->persist_grid : 0u; }

const char* wt_batch_last_error(const wt_batch* b) { return b ? b->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

