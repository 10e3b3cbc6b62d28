// The C ABI of libwt (include/wt.h): context lifetime, device memory, the
// engine calls of the reference (src/engine/engine.ts AeroEngine: constructor
// :226, reset :371, setShape :426, frame :574-729, maybeReadForces :739,
// debugRead :763) mapped onto the device kernels, and error reporting.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

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

// Largest float t with sqrt_rn(t) <= 0.35f: sqrt_rn(x) > 0.35f <=> x > t (correctly
// rounded sqrt is monotonic), so the kernel can test u.u without a square root.
float wt::guard_threshold() {
  static float t = [] {
    float x = 0.35f * 0.35f;
    while (__builtin_sqrtf(x) > 0.35f) x = __builtin_nextafterf(x, 0.0f);
    while (__builtin_sqrtf(__builtin_nextafterf(x, 1.0f)) <= 0.35f) x = __builtin_nextafterf(x, 1.0f);
    return x;
  }();
  return t;
}

namespace {
// WGSL smoothstep/min/max (host copy of the same float arithmetic).
float h_min(float a, float b) { return b < a ? b : a; }
float h_max(float a, float b) { return a < b ? b : a; }
float h_smooth(float lo, float hi, float x) {
  const float t = h_min(h_max((x - lo) / (hi - lo), 0.0f), 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

}  // namespace

namespace wt {
namespace api {

thread_local std::string g_create_error;

int fail(wt_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_error = msg;
  return code;
}


bool valid_storage(uint32_t s) { return s == WT_STORE_F32 || s == WT_STORE_F16 || s == WT_STORE_BF16; }


// x-dependent base relaxation time (wgsl.ts:260).
float tau0_at(const wt_sim& s, uint32_t nx, uint32_t x) {
  const float fnx = (float)nx, fx = (float)x;
  return s.tau0 + s.sponge_amp * h_smooth(fnx - s.sponge_cells, fnx - 1.0f, fx) +
         s.inlet_amp * (1.0f - h_smooth(0.0f, s.inlet_cells, fx));
}

// Every relaxation time must be finite and >= 2^-10 (physical runs use > 0.5;
// the collision kernel's Smagorinsky quotient relies on tau0^2 >= 2^-20).
bool valid_tau(const wt_sim& s, uint32_t nx) {
  for (uint32_t x = 0; x < nx; x++) {
    const float t = tau0_at(s, nx, x);
    if (!(t >= 0x1p-10f) || !(t < 1e30f)) return false;
  }
  return true;
}

// Per-parameter tables: x-dependent tau0 (wgsl.ts:260), Smagorinsky factor,
// inlet equilibrium, belt coefficients.
int apply_sim(wt_ctx* c) {
  const wt_sim& s = c->sim;
  std::vector<float>& t0 = c->tau_host;
  t0.resize(c->nx);
  for (uint32_t x = 0; x < c->nx; x++) t0[x] = tau0_at(s, c->nx, x);
  WT_CUDA(c, cudaMemcpyAsync(c->tau0_x, t0.data(), c->nx * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  const float K = 0x1.974b24p+4f;  // 18 * 1.41421356 evaluated as an abstract constant, rounded once
  c->ks2 = K * s.smag * s.smag;
  for (int i = 0; i < 19; i++) {
    const float u = s.u_in;
    const float cu = (float)CXd(i) * u + (float)CYd(i) * 0.0f + (float)CZd(i) * 0.0f;
    const float uu = u * u + 0.0f * 0.0f + 0.0f * 0.0f;
    c->feq_in[i] = Wd(i) * 1.0f * (1.0f + 3.0f * cu + 4.5f * cu * cu - 1.5f * uu);
    c->floor_k[i] = 6.0f * Wd(i) * (float)CXd(i);
    // guard reset state (wgsl.ts:239-241): rho = 1, u = uin * 0.5
    const float gx = u * 0.5f, gy = 0.0f * 0.5f, gz = 0.0f * 0.5f;
    const float gcu = (float)CXd(i) * gx + (float)CYd(i) * gy + (float)CZd(i) * gz;
    const float guu = gx * gx + gy * gy + gz * gz;
    c->feq_guard[i] = Wd(i) * 1.0f * (1.0f + 3.0f * gcu + 4.5f * gcu * gcu - 1.5f * guu);
  }
  c->version++;
  return WT_OK;
}

uint32_t warps_per_block(const StepGeom& g);

ReduceArgs reduce_args(const wt_ctx* c) {
  ReduceArgs r;
  r.slots = c->slots;
  r.nslots = c->nslots;
  r.hist_cap = WT_HIST_CAP;
  r.hist = c->hist;
  r.hist_pos = c->hist_pos;
  r.totals = c->totals;
  r.raw_totals = c->raw_totals;
  r.mass_partial = c->mass_partial;
  r.nmass = c->geom.nblocks * warps_per_block(c->geom);
  r.mass_out = c->totals + 9;
  r.counter = c->counters + 1;
  r.part = c->red_part;
  return r;
}

int flush_forces(wt_ctx* c);

// After new flags: cell words, force-carrying blocks and their partial slots.
int rebuild_links(wt_ctx* c) {
  if (int rc = flush_forces(c)) return rc;  // pending records use the current slot layout
  WT_CUDA(c, launch_cell_words(c->solid, c->emit, c->cellw, c->nx, c->ny, c->nz, c->stream));
  WT_CUDA(c, launch_heat_sources(c->emit, c->heat_src, c->nx, c->ny, c->nz, c->stream));
  uint8_t* dflags = nullptr;
  WT_CUDA(c, cudaMallocAsync((void**)&dflags, c->geom.nblocks, c->stream));
  WT_CUDA(c, launch_block_flags(c->cellw, c->geom, c->nx, c->ny, c->nz, dflags, c->stream));
  std::vector<uint8_t> flags(c->geom.nblocks);
  std::vector<uint8_t> sol(c->n);
  WT_CUDA(c, cudaMemcpyAsync(flags.data(), dflags, c->geom.nblocks, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(sol.data(), c->solid, c->n, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaFreeAsync(dflags, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  std::vector<int32_t> map(c->geom.nblocks);
  uint32_t ns = 0;
  for (uint32_t b = 0; b < c->geom.nblocks; b++) map[b] = flags[b] ? (int32_t)ns++ : -1;
  c->nslots = ns;
  c->fluid_cells = 0;
  c->solid_cells[0] = c->solid_cells[1] = c->solid_cells[2] = 0;
  for (uint64_t i = 0; i < c->n; i++) {
    if (sol[i] == 0) c->fluid_cells++;
    else c->solid_cells[(sol[i] - 1) % 3]++;
  }
  // Partial records for up to WT_PENDING_MAX steps, capped at 64 MiB.
  uint64_t per_step = (uint64_t)(ns ? ns : 1) * sizeof(ForceSlot);
  uint64_t cap_steps = (64ull << 20) / per_step;
  if (cap_steps < 2) cap_steps = 2;
  if (cap_steps > WT_PENDING_MAX) cap_steps = WT_PENDING_MAX;
  const uint64_t need = cap_steps * (ns ? ns : 1);
  if (need > c->slot_cap) {
    if (c->slots) {
      cudaFree(c->slots);
      c->device_bytes -= (uint64_t)c->slot_cap * sizeof(ForceSlot);
      c->slots = nullptr;
    }
    int rc = dalloc(c, &c->slots, need * sizeof(ForceSlot));
    if (rc) return rc;
    c->slot_cap = (uint32_t)need;
  }
  c->pending_cap = (uint32_t)cap_steps;
  WT_CUDA(c, cudaMemcpyAsync(c->block_slot, map.data(), map.size() * 4, cudaMemcpyHostToDevice, c->stream));
  ReduceArgs ra = reduce_args(c);
  WT_CUDA(c, cudaMemcpyAsync(c->d_reduce, &ra, sizeof(ra), cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  c->version++;
  return WT_OK;
}


uint32_t warps_per_block(const StepGeom& g) { return (g.block.x * g.block.y + 31) / 32; }

StepArgs step_args(const wt_ctx* c) {
  StepArgs a;
  a.pop = c->pop; a.cellw = c->cellw; a.solid = c->solid; a.fields = c->fields; a.outlet_u = c->outlet_u;
  a.tau0_x = c->tau0_x; a.block_slot = c->block_slot; a.mass_partial = c->mass_partial;
  a.slots = c->slots; a.nslots = c->nslots;
  a.guard_count = c->counters;
  a.nx = c->nx; a.ny = c->ny; a.nz = c->nz; a.n = c->n; a.np = c->np;
  a.u_in = c->sim.u_in; a.ks2 = c->ks2;
  memcpy(a.feq_in, c->feq_in, sizeof(a.feq_in));
  memcpy(a.floor_k, c->floor_k, sizeof(a.floor_k));
  memcpy(a.feq_guard, c->feq_guard, sizeof(a.feq_guard));
  const float S = c->sim.storage == WT_STORE_F16 ? 16384.0f : 1.0f;  // f16 keeps (f - w) 2^14, bf16 f - w
  for (int i = 0; i < 19; i++) {
    a.dev_in[i] = (c->feq_in[i] - Wd(i)) * S;
    a.floor_kd[i] = c->floor_k[i] * S;
    a.dev_guard[i] = (c->feq_guard[i] - Wd(i)) * S;
  }
  a.guard_uu = guard_threshold();
  fill_slot_offsets(a);
  a.prefetch_ahead = c->prefetch_ahead;
  a.pop_bytes = 19ull * c->np * c->elem;
  return a;
}

cudaError_t enqueue_heat(wt_ctx* c, int heat_passes, float dt, cudaStream_t s) {
  HeatArgs h;
  h.fields = c->fields; h.emit = c->emit; h.src = c->heat_src;
  h.nx = c->nx; h.ny = c->ny; h.nz = c->nz;
  h.dt = dt;
  h.cool = c->sim.heat_cool; h.diffuse = c->sim.heat_diffuse; h.src_mix = c->sim.heat_src_mix;
  for (int p = 0; p < heat_passes; p++) {
    h.tin = (p & 1) ? c->tB : c->tA;
    h.tout = (p & 1) ? c->tA : c->tB;
    cudaError_t e = launch_heat(h, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The kernels of one wt_step call: collide-stream steps (gather/local
// alternating, fields on the last), a force reduction every pending_cap steps
// and at the end, then the heat passes.  Pure launches: capturable in a graph.
cudaError_t enqueue_frame(wt_ctx* c, int n, int heat_passes, float dt, uint32_t pending0, cudaStream_t s) {
  StepArgs a = step_args(c);
  uint32_t pending = pending0;
  for (int k = 0; k < n; k++) {
    const bool last = (k == n - 1);
    a.slots = c->slots + (size_t)pending * (c->nslots ? c->nslots : 1);
    cudaError_t e = launch_step(c->sim.storage, (k & 1) == 0, last, c->geom, a, s);
    if (e != cudaSuccess) return e;
    pending++;
    if (pending == c->pending_cap) {
      e = launch_force_reduce(c->d_reduce, 1, pending, last, s);
      if (e != cudaSuccess) return e;
      pending = 0;
    }
  }
  return enqueue_heat(c, heat_passes, dt, s);
}

// Sums the force records of the pending steps (and the mass of the last field
// step) into the history and the totals; the deferred part of enqueue_frame.
int flush_forces(wt_ctx* c) {
  if (c->pending == 0 && !c->mass_pending) return WT_OK;
  WT_CUDA(c, launch_force_reduce(c->d_reduce, 1, c->pending, c->mass_pending, c->stream));
  c->pending = 0;
  c->mass_pending = false;
  return WT_OK;
}

// Change the block shape of the step kernels: block maps are rebuilt.
int set_geometry(wt_ctx* c, uint32_t bx, uint32_t by) {
  StepGeom g = step_geometry(c->nx, c->ny, c->nz, bx, by);
  if (g.block.x == c->geom.block.x && g.block.y == c->geom.block.y) return WT_OK;
  // Pending force records and mass partials refer to the buffers freed below:
  // sum them first (their reduction reads block_slot's records and mass_partial).
  if (int rc = flush_forces(c)) return rc;
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  cudaFree(c->block_slot);
  cudaFree(c->mass_partial);
  c->device_bytes -= (uint64_t)c->geom.nblocks * 4 + (uint64_t)c->geom.nblocks * warps_per_block(c->geom) * 8;
  c->block_slot = nullptr;
  c->mass_partial = nullptr;
  c->geom = g;
  c->prefetch_ahead = step_resident_blocks(c->sim.storage, g, c->sm_count, 19ull * c->np * c->elem, c->l2_bytes);
  c->bx = g.block.x;
  c->by = g.block.y;
  int rc;
  if ((rc = dalloc(c, &c->block_slot, (uint64_t)g.nblocks * 4)) ||
      (rc = dalloc(c, &c->mass_partial, (uint64_t)g.nblocks * warps_per_block(g) * 8)))
    return rc;
  return rebuild_links(c);
}

int check_ctx(wt_ctx* c) {
  if (!c) return WT_ERR_ARG;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(c, WT_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  return WT_OK;
}



int create_ctx(const wt_grid* grid, const wt_sim* sim, cudaStream_t ext, wt_ctx** out) {
  if (!grid || !sim || !out) return fail(nullptr, WT_ERR_ARG, "wt_create: null argument");
  *out = nullptr;
  if (grid->nx < 8 || grid->ny < 2 || grid->nz < 2) return fail(nullptr, WT_ERR_ARG, "wt_create: grid must be at least 8x2x2");
  const uint64_t n = (uint64_t)grid->nx * grid->ny * grid->nz;
  const uint64_t np = (n + 63) / 64 * 64;
  if (np * 19 >= (1ull << 32)) return fail(nullptr, WT_ERR_ARG, "wt_create: lattice too large (19 * cells must stay below 2^32)");
  if (!(grid->h > 0.0f)) return fail(nullptr, WT_ERR_ARG, "wt_create: cell size must be positive");
  if (!valid_storage(sim->storage)) return fail(nullptr, WT_ERR_ARG, "wt_create: unknown storage format");
  if (!valid_tau(*sim, grid->nx)) return fail(nullptr, WT_ERR_ARG, "wt_create: relaxation time below 2^-10 or not finite");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(nullptr, WT_ERR_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return fail(nullptr, WT_ERR_DEVICE, std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
  if (!(prop.major == 10 && prop.minor == 3))
    return fail(nullptr, WT_ERR_DEVICE, "libwt is built for sm_103a (GB300); device " + std::string(prop.name) + " is sm_" +
                                            std::to_string(prop.major) + std::to_string(prop.minor));
  wt_ctx* c = new wt_ctx();
  c->device = dev;
  c->grid = *grid;
  c->sim = *sim;
  c->nx = grid->nx; c->ny = grid->ny; c->nz = grid->nz;
  c->n = n; c->np = np;
  c->elem = sim->storage == WT_STORE_F32 ? 4 : 2;
  c->sm_count = prop.multiProcessorCount;
  if (const char* s = getenv("WT_STEP_BX")) c->bx = (uint32_t)atoi(s);
  if (const char* s = getenv("WT_STEP_BY")) c->by = (uint32_t)atoi(s);
  c->geom = step_geometry(c->nx, c->ny, c->nz, c->bx, c->by);
  c->l2_bytes = (uint64_t)prop.l2CacheSize;
  c->prefetch_ahead = step_resident_blocks(c->sim.storage, c->geom, c->sm_count, 19ull * np * c->elem, c->l2_bytes);
  c->bx = c->geom.block.x;
  c->by = c->geom.block.y;
  int rc = 0;
  auto cleanup = [&](int code) { std::string m = c->err; wt_destroy(c); g_create_error = m; return code; };
  if (ext) {
    c->stream = ext;
    c->own_stream = false;
  } else {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { c->err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e); return cleanup(WT_ERR_CUDA); }
  }
  if ((rc = dalloc(c, &c->pop, 19 * np * c->elem)) || (rc = dalloc(c, &c->cellw, n * 4)) ||
      (rc = dalloc(c, &c->solid, n)) || (rc = dalloc(c, &c->emit, n * 4)) || (rc = dalloc(c, &c->fields, n * 16)) ||
      (rc = dalloc(c, &c->tA, n * 4)) || (rc = dalloc(c, &c->tB, n * 4)) ||
      (rc = dalloc(c, &c->outlet_u, (uint64_t)c->ny * c->nz * 16)) || (rc = dalloc(c, &c->tau0_x, c->nx * 4)) ||
      (rc = dalloc(c, &c->block_slot, (uint64_t)c->geom.nblocks * 4)) ||
      (rc = dalloc(c, &c->mass_partial, (uint64_t)c->geom.nblocks * warps_per_block(c->geom) * 8)) ||
      (rc = dalloc(c, &c->hist, (uint64_t)WT_HIST_CAP * 16 * 8)) || (rc = dalloc(c, &c->totals, 18 * 8)) ||
      (rc = dalloc(c, &c->raw_totals, 12 * 4)) || (rc = dalloc(c, &c->counters, 4 * 4)) ||
      (rc = dalloc(c, &c->hist_pos, 8)) || (rc = dalloc(c, &c->d_reduce, sizeof(ReduceArgs))) ||
      (rc = dalloc(c, &c->red_part, WT_RED_PART * 8)) || (rc = dalloc(c, &c->heat_src, n * 4)))
    return cleanup(rc);
  if (cudaMemsetAsync(c->solid, 0, n, c->stream) != cudaSuccess || cudaMemsetAsync(c->emit, 0, n * 4, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->heat_src, 0, n * 4, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->totals, 0, 18 * 8, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->raw_totals, 0, 48, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->counters, 0, 16, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->hist_pos, 0, 8, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->pop, 0, 19 * np * c->elem, c->stream) != cudaSuccess) {
    c->err = "initial cudaMemsetAsync failed";
    return cleanup(WT_ERR_CUDA);
  }
  if ((rc = apply_sim(c)) || (rc = rebuild_links(c)) || (rc = wt_reset(c))) return cleanup(rc);
  *out = c;
  return WT_OK;
}

}  // namespace api
}  // namespace wt

extern "C" {

const char* wt_version(void) { return "libwt 0.1 sm_103a"; }

const char* wt_last_error(const wt_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

extern "C" {

int wt_create(const wt_grid* grid, const wt_sim* sim, wt_ctx** out) { return create_ctx(grid, sim, nullptr, out); }

int wt_destroy(wt_ctx* c) {
  if (!c) return WT_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  // Renderers still open over this lattice lose their targets here; a later
  // wt_render_destroy only frees the handle, and other calls on it fail.
  for (wt_renderer* r : c->renderers) release_renderer_buffers(r);
  c->renderers.clear();
  for (wt_mesh* m : c->meshes) release_mesh_buffers(m);
  c->meshes.clear();
  if (c->fpinned) cudaFreeHost(c->fpinned);
  for (cudaEvent_t& ev : c->fevent)
    if (ev) cudaEventDestroy(ev);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  void* bufs[] = {c->pop, c->cellw, c->solid, c->emit, c->fields, c->tA, c->tB, c->outlet_u, c->tau0_x,
                  c->block_slot, c->slots, c->mass_partial, c->hist, c->totals, c->raw_totals, c->counters,
                  c->hist_pos, c->d_reduce, c->car_body, c->car_parts, c->car_rig, c->red_part, c->heat_src};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (c->stream && c->own_stream) cudaStreamDestroy(c->stream);
  delete c;
  return WT_OK;
}

int wt_set_sim(wt_ctx* c, const wt_sim* sim) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!sim) return fail(c, WT_ERR_ARG, "wt_set_sim: null sim");
  if (sim->storage != c->sim.storage) return fail(c, WT_ERR_ARG, "wt_set_sim: storage format is fixed at wt_create");
  if (!valid_tau(*sim, c->nx)) return fail(c, WT_ERR_ARG, "wt_set_sim: relaxation time below 2^-10 or not finite");
  // Identical parameters (syncSim runs every frame) still upload the per-x table,
  // but leave the kernel arguments - and so the captured step sequences - valid.
  const bool same = memcmp(&c->sim, sim, sizeof(wt_sim)) == 0;
  const uint64_t version = c->version;
  c->sim = *sim;
  if ((rc = apply_sim(c))) return rc;
  if (same) c->version = version;
  return WT_OK;
}

int wt_reset(wt_ctx* c) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if ((rc = flush_forces(c))) return rc;
  WT_CUDA(c, launch_init(c->sim.storage, c->pop, c->fields, c->outlet_u, c->nx, c->ny, c->nz, c->np, c->sim.u_in, c->stream));
  WT_CUDA(c, cudaMemsetAsync(c->tA, 0, c->n * 4, c->stream));
  WT_CUDA(c, cudaMemsetAsync(c->tB, 0, c->n * 4, c->stream));
  c->steps_total = 0;
  return WT_OK;
}

}  // extern "C"

CarView wt::api::car_view(const wt_ctx* c) {
  CarView v;
  v.body = c->car_body;
  v.parts = c->car_parts;
  for (int i = 0; i < 3; i++) v.pdims[i] = c->car_pdims[i];
  v.rig = c->car_rig;
  return v;
}

extern "C" {

int wt_set_car_model(wt_ctx* c, const uint16_t* body, const uint16_t* parts, const uint32_t parts_dims[3],
                     const wt_rig* rig) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!body || !parts || !parts_dims || !rig) return fail(c, WT_ERR_ARG, "wt_set_car_model: null argument");
  const uint64_t np = (uint64_t)parts_dims[0] * parts_dims[1] * parts_dims[2];
  if (np == 0 || parts_dims[0] > 4096 || parts_dims[1] > 4096 || parts_dims[2] > 4096)
    return fail(c, WT_ERR_ARG, "wt_set_car_model: parts atlas dimensions must be 1..4096");
  static_assert(sizeof(wt_rig) == 87 * 16, "wt_rig is the 87 vec4 of the Rig uniform");
  const size_t nb = (size_t)368 * 84 * 67;
  WT_CUDA(c, cudaStreamSynchronize(c->stream));  // earlier work may still read the old model
  uint16_t* b = nullptr;
  uint16_t* pa = nullptr;
  float4* rg = nullptr;
  cudaError_t e = cudaMalloc((void**)&b, nb * 2);
  if (e == cudaSuccess) e = cudaMalloc((void**)&pa, np * 2);
  if (e == cudaSuccess) e = cudaMalloc((void**)&rg, sizeof(wt_rig));
  if (e == cudaSuccess) e = cudaMemcpy(b, body, nb * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(pa, parts, np * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(rg, rig, sizeof(wt_rig), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(b);
    cudaFree(pa);
    cudaFree(rg);
    return fail(c, e == cudaErrorMemoryAllocation ? WT_ERR_NOMEM : WT_ERR_CUDA,
                std::string("wt_set_car_model: ") + cudaGetErrorString(e));
  }
  cudaFree(c->car_body);
  cudaFree(c->car_parts);
  cudaFree(c->car_rig);
  c->car_body = b;
  c->car_parts = pa;
  c->car_rig = rg;
  for (int i = 0; i < 3; i++) c->car_pdims[i] = parts_dims[i];
  return WT_OK;
}

int wt_voxelize(wt_ctx* c, const wt_shape* shape) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!shape) return fail(c, WT_ERR_ARG, "wt_voxelize: null shape");
  const uint32_t k = shape->kind;
  if (!(k == WT_KIND_F1 || k == WT_KIND_SPHERE || k == WT_KIND_CUBE || k == WT_KIND_WING || k == WT_KIND_EMPTY ||
        k == WT_KIND_BOX || k == WT_KIND_W17))
    return fail(c, WT_ERR_UNSUPPORTED, "wt_voxelize: scene kind " + std::to_string(k) +
                                           " is not built (custom profile scene)");
  if (k == WT_KIND_W17 && !c->car_body)
    return fail(c, WT_ERR_STATE, "wt_voxelize: the W17 scene needs a car model (wt_set_car_model)");
  WT_CUDA(c, launch_voxelize(*shape, car_view(c), c->grid, c->solid, c->emit, c->stream));
  c->shape = *shape;
  return rebuild_links(c);
}

int wt_set_solid(wt_ctx* c, const uint32_t* solid, const float* emit) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!solid || !emit) return fail(c, WT_ERR_ARG, "wt_set_solid: null buffer");
  uint32_t* tmp = nullptr;
  WT_CUDA(c, cudaMallocAsync((void**)&tmp, c->n * 4, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(tmp, solid, c->n * 4, cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, launch_solid_from_u32(tmp, c->solid, c->n, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(c->emit, emit, c->n * 4, cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaFreeAsync(tmp, c->stream));
  return rebuild_links(c);
}

int wt_step(wt_ctx* c, int n_lbm_steps, int heat_passes, float heat_dt) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (n_lbm_steps < 2 || (n_lbm_steps & 1))
    return fail(c, WT_ERR_ARG, "wt_step: n_lbm_steps must be even and >= 2 (the engine issues max(2, steps - steps % 2))");
  if (heat_passes < 0 || (heat_passes & 1)) return fail(c, WT_ERR_ARG, "wt_step: heat_passes must be 0 or even");
  const float dt = heat_dt > 0.0f ? heat_dt : (float)n_lbm_steps / 2.0f;
  const uint32_t pend0 = c->pending;
  if ((rc = run_graphed(c, c->graphs, c->version, n_lbm_steps, heat_passes, dt, pend0,
                        [&](cudaStream_t s) { return enqueue_frame(c, n_lbm_steps, heat_passes, dt, pend0, s); })))
    return rc;
  // the host copy of enqueue_frame's pending count
  const uint32_t total = pend0 + (uint32_t)n_lbm_steps;
  c->pending = total % c->pending_cap;
  c->mass_pending = (c->pending != 0);  // a reduction on the last step summed the mass too
  c->steps_total += n_lbm_steps;
  c->steps_since_read += n_lbm_steps;
  c->steps_recorded += n_lbm_steps;
  return WT_OK;
}

int wt_read_forces(wt_ctx* c, wt_forces* out, int reset) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!out) return fail(c, WT_ERR_ARG, "wt_read_forces: null output");
  uint64_t ticket = 0;
  if ((rc = wt_read_forces_async(c, reset, &ticket))) return rc;
  return wt_forces_collect(c, ticket, out);
}

int wt_read_forces_async(wt_ctx* c, int reset, uint64_t* ticket) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!ticket) return fail(c, WT_ERR_ARG, "wt_read_forces_async: null ticket");
  if (!c->fpinned) {  // landing slots the readout kernel writes directly (host-mapped)
    WT_CUDA(c, cudaHostAlloc((void**)&c->fpinned, WT_ASYNC_SLOTS * sizeof(wt_forces), cudaHostAllocMapped));
    WT_CUDA(c, cudaHostGetDevicePointer((void**)&c->fpinned_dev, c->fpinned, 0));
    for (cudaEvent_t& ev : c->fevent) WT_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  if ((rc = flush_forces(c))) return rc;
  const uint32_t slot = (uint32_t)(c->fticket % WT_ASYNC_SLOTS);
  if (c->fticket >= WT_ASYNC_SLOTS) WT_CUDA(c, cudaEventSynchronize(c->fevent[slot]));  // slot reused
  WT_CUDA(c, launch_force_readback(c->totals, c->raw_totals, c->counters, c->fpinned_dev + slot, c->steps_since_read,
                                   reset, c->stream));
  WT_CUDA(c, cudaEventRecord(c->fevent[slot], c->stream));
  if (reset) c->steps_since_read = 0;
  *ticket = c->fticket++;
  return WT_OK;
}

int wt_forces_collect(wt_ctx* c, uint64_t ticket, wt_forces* out) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!out) return fail(c, WT_ERR_ARG, "wt_forces_collect: null output");
  if (ticket >= c->fticket || c->fticket - ticket > WT_ASYNC_SLOTS)
    return fail(c, WT_ERR_ARG, "wt_forces_collect: unknown ticket or overwritten by newer readbacks");
  const uint32_t slot = (uint32_t)(ticket % WT_ASYNC_SLOTS);
  WT_CUDA(c, cudaEventSynchronize(c->fevent[slot]));
  memcpy(out, c->fpinned + slot, sizeof(wt_forces));
  return WT_OK;
}

int wt_read_force_history(wt_ctx* c, double* out, uint32_t count) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if ((rc = flush_forces(c))) return rc;
  if (!out && count) return fail(c, WT_ERR_ARG, "wt_read_force_history: null output");
  const uint64_t avail = c->steps_recorded < WT_HIST_CAP ? c->steps_recorded : WT_HIST_CAP;
  if (count > avail) return fail(c, WT_ERR_ARG, "wt_read_force_history: only " + std::to_string(avail) + " steps recorded");
  std::vector<double> rec((size_t)count * 16);
  const uint64_t first = c->steps_recorded - count;
  for (uint32_t k = 0; k < count;) {
    const uint64_t slot = (first + k) % WT_HIST_CAP;
    const uint32_t run = (uint32_t)((WT_HIST_CAP - slot) < (count - k) ? (WT_HIST_CAP - slot) : (count - k));
    WT_CUDA(c, cudaMemcpyAsync(rec.data() + (size_t)k * 16, c->hist + slot * 16, (size_t)run * 16 * 8,
                               cudaMemcpyDeviceToHost, c->stream));
    k += run;
  }
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  for (uint32_t k = 0; k < count; k++) memcpy(out + (size_t)k * 9, rec.data() + (size_t)k * 16, 9 * 8);
  return WT_OK;
}

int wt_read_fields(wt_ctx* c, float* u_rho, uint32_t* solid, float* temps, float* emit, uint32_t* links) {
  int rc = check_ctx(c);
  if (rc) return rc;
  const uint64_t n = c->n;
  if (u_rho) WT_CUDA(c, cudaMemcpyAsync(u_rho, c->fields, n * 16, cudaMemcpyDeviceToHost, c->stream));
  if (temps) WT_CUDA(c, cudaMemcpyAsync(temps, c->tA, n * 4, cudaMemcpyDeviceToHost, c->stream));
  if (emit) WT_CUDA(c, cudaMemcpyAsync(emit, c->emit, n * 4, cudaMemcpyDeviceToHost, c->stream));
  if (solid || links) {
    uint32_t* tmp = nullptr;
    WT_CUDA(c, cudaMallocAsync((void**)&tmp, n * 4, c->stream));
    if (solid) {
      WT_CUDA(c, launch_solid_u32(c->solid, tmp, n, c->stream));
      WT_CUDA(c, cudaMemcpyAsync(solid, tmp, n * 4, cudaMemcpyDeviceToHost, c->stream));
    }
    if (links) {
      WT_CUDA(c, launch_links_out(c->cellw, tmp, n, c->stream));
      WT_CUDA(c, cudaMemcpyAsync(links, tmp, n * 4, cudaMemcpyDeviceToHost, c->stream));
    }
    WT_CUDA(c, cudaFreeAsync(tmp, c->stream));
  }
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

int wt_read_populations(wt_ctx* c, float* f) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!f) return fail(c, WT_ERR_ARG, "wt_read_populations: null output");
  float* tmp = nullptr;
  WT_CUDA(c, cudaMallocAsync((void**)&tmp, c->n * 19 * 4, c->stream));
  WT_CUDA(c, launch_read_pop(c->sim.storage, c->pop, tmp, (uint32_t)c->n, c->np, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(f, tmp, c->n * 19 * 4, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaFreeAsync(tmp, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

int wt_write_state(wt_ctx* c, const float* f, const float* u_rho, const float* temps) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if ((rc = flush_forces(c))) return rc;
  if (f) {
    float* tmp = nullptr;
    WT_CUDA(c, cudaMallocAsync((void**)&tmp, c->n * 19 * 4, c->stream));
    WT_CUDA(c, cudaMemcpyAsync(tmp, f, c->n * 19 * 4, cudaMemcpyHostToDevice, c->stream));
    WT_CUDA(c, launch_write_pop(c->sim.storage, tmp, c->pop, (uint32_t)c->n, c->np, c->stream));
    WT_CUDA(c, cudaFreeAsync(tmp, c->stream));
  }
  if (u_rho) {
    WT_CUDA(c, cudaMemcpyAsync(c->fields, u_rho, c->n * 16, cudaMemcpyHostToDevice, c->stream));
    std::vector<float4> ou((size_t)c->ny * c->nz);
    for (uint32_t z = 0; z < c->nz; z++)
      for (uint32_t y = 0; y < c->ny; y++) {
        const uint64_t idx = (uint64_t)(c->nx - 1) + (uint64_t)c->nx * (y + (uint64_t)c->ny * z);
        ou[y + (size_t)c->ny * z] = make_float4(u_rho[4 * idx], u_rho[4 * idx + 1], u_rho[4 * idx + 2], 0.0f);
      }
    WT_CUDA(c, cudaMemcpyAsync(c->outlet_u, ou.data(), ou.size() * 16, cudaMemcpyHostToDevice, c->stream));
    WT_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  if (temps) WT_CUDA(c, cudaMemcpyAsync(c->tA, temps, c->n * 4, cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

int wt_reset_from(wt_ctx* c, const float* u_rho, uint32_t cx, uint32_t cy, uint32_t cz) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if ((rc = flush_forces(c))) return rc;
  if (!u_rho || cx == 0 || cy == 0 || cz == 0) return fail(c, WT_ERR_ARG, "wt_reset_from: empty coarse field");
  float4* tmp = nullptr;
  const size_t bytes = (size_t)cx * cy * cz * 16;
  WT_CUDA(c, cudaMallocAsync((void**)&tmp, bytes, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(tmp, u_rho, bytes, cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, launch_resample_init(c->sim.storage, tmp, cx, cy, cz, c->pop, c->fields, c->outlet_u, c->nx, c->ny, c->nz,
                                  c->np, c->stream));
  WT_CUDA(c, cudaFreeAsync(tmp, c->stream));
  WT_CUDA(c, cudaMemsetAsync(c->tA, 0, c->n * 4, c->stream));
  WT_CUDA(c, cudaMemsetAsync(c->tB, 0, c->n * 4, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  c->steps_total = 0;
  return WT_OK;
}

int wt_read_coarse(wt_ctx* c, uint32_t cx, uint32_t cy, uint32_t cz, float* u_rho) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!u_rho || cx == 0 || cy == 0 || cz == 0 || cx > c->nx || cy > c->ny || cz > c->nz)
    return fail(c, WT_ERR_ARG, "wt_read_coarse: coarse grid must be non-empty and no finer than the lattice");
  float4* tmp = nullptr;
  const size_t bytes = (size_t)cx * cy * cz * 16;
  WT_CUDA(c, cudaMallocAsync((void**)&tmp, bytes, c->stream));
  WT_CUDA(c, launch_coarse_average(c->fields, c->cellw, c->nx, c->ny, c->nz, tmp, cx, cy, cz, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(u_rho, tmp, bytes, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaFreeAsync(tmp, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

int wt_sdf_sample(const wt_shape* shape, const wt_grid* grid, float* out) {
  if (!shape || !grid || !out || grid->nx == 0 || grid->ny == 0 || grid->nz == 0 || !(grid->h > 0.0f))
    return fail(nullptr, WT_ERR_ARG, "wt_sdf_sample: invalid argument");
  if (shape->kind == 4 || shape->kind == 5 || shape->kind > WT_KIND_BOX)
    return fail(nullptr, WT_ERR_UNSUPPORTED, "wt_sdf_sample: scene kind not built");
  const size_t bytes = (size_t)grid->nx * grid->ny * grid->nz * 4;
  float* tmp = nullptr;
  cudaError_t e = cudaMalloc((void**)&tmp, bytes);
  if (e == cudaSuccess) e = launch_sdf_sample(*shape, *grid, tmp, 0);
  if (e == cudaSuccess) e = cudaMemcpy(out, tmp, bytes, cudaMemcpyDeviceToHost);
  if (tmp) cudaFree(tmp);
  if (e != cudaSuccess) return fail(nullptr, WT_ERR_CUDA, std::string("wt_sdf_sample: ") + cudaGetErrorString(e));
  return WT_OK;
}

int wt_info_get(wt_ctx* c, wt_info* out) {
  if (!c || !out) return WT_ERR_ARG;
  out->cells = c->n;
  out->device_bytes = c->device_bytes;
  out->steps_total = c->steps_total;
  out->storage = c->sim.storage;
  out->fluid_cells = c->fluid_cells;
  for (int k = 0; k < 3; k++) out->solid_cells[k] = c->solid_cells[k];
  out->boundary_blocks = c->nslots;
  out->history_capacity = WT_HIST_CAP;
  out->sm_count = c->sm_count;
  return WT_OK;
}

void* wt_stream(wt_ctx* c) { return c ? (void*)c->stream : nullptr; }

int wt_sync(wt_ctx* c) {
  int rc = check_ctx(c);
  if (rc) return rc;
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

}  // extern "C"

