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

#include "wt_fmath.h"
#include "wt_internal.h"
#include "wt_fields.h"
#include "wt_render.h"
#include "wt_mesh.h"
#include "wt_lattice.cuh"

using namespace wt;

#define WT_ASYNC_SLOTS 16  // force readbacks in flight per context

struct wt_renderer;
struct wt_mesh;

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
void release_renderer_buffers(wt_renderer* r);
void release_mesh_buffers(wt_mesh* m);
}

struct wt_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  wt_grid grid{};
  wt_sim sim{};
  uint32_t nx = 0, ny = 0, nz = 0;
  uint64_t n = 0, np = 0;
  size_t elem = 4;
  StepGeom geom{};
  uint32_t sm_count = 0;
  uint32_t prefetch_ahead = 0;  // resident step blocks at the current block shape
  // device buffers
  void* pop = nullptr;
  uint32_t* cellw = nullptr;
  uint8_t* solid = nullptr;
  float* emit = nullptr;
  float4* fields = nullptr;
  float* tA = nullptr;
  float* tB = nullptr;
  float4* outlet_u = nullptr;
  float* tau0_x = nullptr;
  int32_t* block_slot = nullptr;
  ForceSlot* slots = nullptr;
  uint32_t slot_cap = 0;      // records allocated
  uint32_t nslots = 0;        // records per step for the current scene
  uint32_t pending_cap = 1;   // steps per reduction launch
  double* mass_partial = nullptr;
  double* hist = nullptr;
  double* totals = nullptr;   // [9] FP64 force sums, [9] mass
  int32_t* raw_totals = nullptr;  // [12]
  unsigned int* counters = nullptr;  // [0] guard count, [1] reduce counter
  // host state
  uint64_t steps_total = 0, steps_since_read = 0, steps_recorded = 0;
  uint64_t device_bytes = 0;
  uint32_t fluid_cells = 0, solid_cells[3] = {0, 0, 0};
  float ks2 = 0.0f;
  float feq_in[19];
  float floor_k[19];
  float feq_guard[19];
  std::vector<float> tau_host;  // staging copy of tau0_x (pageable: copied before the call returns)
  bool own_stream = true;
  unsigned long long* hist_pos = nullptr;  // device: per-step records written so far
  ReduceArgs* d_reduce = nullptr;          // device: this lattice's reduction record
  double* red_part = nullptr;              // device: the reduction's chunk sums
  float* heat_src = nullptr;               // device: the neighbours' largest emission per cell
  uint32_t bx = 128, by = 1;               // step-kernel block shape
  uint64_t version = 0;                    // bumped whenever kernel arguments change
  // Force records of steps not yet reduced (single-lattice path): the reduction
  // runs when pending_cap steps have accumulated or before anything reads them.
  uint32_t pending = 0;
  bool mass_pending = false;               // mass partials of the last field step not yet summed
  struct Graph {
    int n, heat;
    float dt;
    uint64_t version;
    uint32_t pend0;                        // pending records when the sequence starts
    cudaGraphExec_t exec;
  };
  std::vector<Graph> graphs;               // captured wt_step sequences
  wt_shape shape{WT_KIND_EMPTY};           // last voxelized shape (the renderer's scene)
  // the baked W17 model (wt_set_car_model): device copies
  uint16_t* car_body = nullptr;
  uint16_t* car_parts = nullptr;
  float4* car_rig = nullptr;
  uint32_t car_pdims[3] = {1, 1, 1};
  std::vector<wt_renderer*> renderers;     // live renderers over this lattice
  std::vector<wt_mesh*> meshes;            // live car meshes on this context
  // asynchronous force readbacks: pinned landing slots, their events, next ticket
  wt_forces* fpinned = nullptr;
  wt_forces* fpinned_dev = nullptr;  // the same slots as the device sees them
  cudaEvent_t fevent[WT_ASYNC_SLOTS] = {};
  uint64_t fticket = 0;
  std::string err;
};

struct wt_batch {
  std::vector<wt_ctx*> lat;
  cudaStream_t stream = nullptr;
  int device = 0;
  uint32_t storage = 0;
  uint32_t bx = 128, by = 1;
  StepArgs* d_args = nullptr;
  BatchTiles* d_tiles = nullptr;
  ReduceArgs* d_reduce = nullptr;
  uint32_t total_blocks = 0;
  uint32_t pending_cap = 1;
  uint64_t version = ~0ull;                // sum of member versions the device tables were built for
  std::vector<wt_ctx::Graph> graphs;
  std::string err;
};

namespace {

thread_local std::string g_create_error;

int fail(wt_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_error = msg;
  return code;
}

#define WT_CUDA(c, call)                                                                       \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return fail((c), e_ == cudaErrorMemoryAllocation ? WT_ERR_NOMEM : WT_ERR_CUDA,           \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                         \
  } while (0)

// WGSL smoothstep/min/max (host copy of the same float arithmetic).
float h_min(float a, float b) { return b < a ? b : a; }
float h_max(float a, float b) { return a < b ? b : a; }
float h_smooth(float lo, float hi, float x) {
  const float t = h_min(h_max((x - lo) / (hi - lo), 0.0f), 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

bool valid_storage(uint32_t s) { return s == WT_STORE_F32 || s == WT_STORE_F16 || s == WT_STORE_BF16; }

template <class T>
int dalloc(wt_ctx* c, T** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) return fail(c, WT_ERR_NOMEM, std::string("cudaMalloc ") + std::to_string(bytes) + " B: " + cudaGetErrorString(e));
  c->device_bytes += bytes;
  return WT_OK;
}

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

// Launch a step sequence through a CUDA graph captured once per (n, heat, dt)
// and argument version; WT_NO_GRAPH=1 launches the kernels directly.
template <class Owner, class F>
int run_graphed(Owner* o, std::vector<wt_ctx::Graph>& cache, uint64_t version, int n, int heat, float dt,
                uint32_t pend0, F&& enqueue) {
  static const bool no_graph = getenv("WT_NO_GRAPH") && atoi(getenv("WT_NO_GRAPH")) != 0;
  cudaStream_t s = o->stream;
  if (no_graph) {
    cudaError_t e = enqueue(s);
    if (e != cudaSuccess) { o->err = std::string("kernel launch: ") + cudaGetErrorString(e); return WT_ERR_CUDA; }
    return WT_OK;
  }
  for (size_t i = 0; i < cache.size();) {
    if (cache[i].version != version) {
      cudaGraphExecDestroy(cache[i].exec);
      cache.erase(cache.begin() + i);
    } else {
      i++;
    }
  }
  cudaGraphExec_t exec = nullptr;
  for (auto& g : cache)
    if (g.n == n && g.heat == heat && g.dt == dt && g.pend0 == pend0) exec = g.exec;
  if (!exec) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { o->err = std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e); return WT_ERR_CUDA; }
    cudaError_t le = enqueue(s);
    e = cudaStreamEndCapture(s, &graph);
    if (le != cudaSuccess || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      o->err = std::string("graph capture: ") + cudaGetErrorString(le != cudaSuccess ? le : e);
      return WT_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { o->err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e); return WT_ERR_CUDA; }
    if (cache.size() >= 16) {
      cudaGraphExecDestroy(cache.front().exec);
      cache.erase(cache.begin());
    }
    cache.push_back({n, heat, dt, version, pend0, exec});
  }
  cudaError_t e = cudaGraphLaunch(exec, s);
  if (e != cudaSuccess) { o->err = std::string("cudaGraphLaunch: ") + cudaGetErrorString(e); return WT_ERR_CUDA; }
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
  c->prefetch_ahead = step_resident_blocks(c->sim.storage, g, c->sm_count);
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

}  // namespace

extern "C" {

const char* wt_version(void) { return "libwt 0.1 sm_103a"; }

const char* wt_last_error(const wt_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

namespace {

// New lattice; `ext` (may be null) is a stream owned by the caller, e.g. a batch.
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
  c->prefetch_ahead = step_resident_blocks(c->sim.storage, c->geom, c->sm_count);
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

}  // namespace

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

CarView car_view(const wt_ctx* c) {
  CarView v;
  v.body = c->car_body;
  v.parts = c->car_parts;
  for (int i = 0; i < 3; i++) v.pdims[i] = c->car_pdims[i];
  v.rig = c->car_rig;
  return v;
}

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

namespace {
FieldGrid field_grid(const wt_ctx* c) {
  FieldGrid g;
  g.nx = c->nx; g.ny = c->ny; g.nz = c->nz;
  g.ox = c->grid.origin[0]; g.oy = c->grid.origin[1]; g.oz = c->grid.origin[2];
  g.h = c->grid.h;
  g.fields = c->fields;
  g.temps = c->tA;
  return g;
}
ViewArgs view_args(const wt_view* v) {
  ViewArgs a;
  a.uIn = v->u_in; a.vReal = v->v_real; a.cpMin = v->cp_min; a.cpMax = v->cp_max;
  a.tMin = v->t_min; a.tMax = v->t_max; a.speedMax = v->speed_max; a.vortMax = v->vort_max;
  return a;
}
}  // namespace

int wt_sample_flow(wt_ctx* c, const float* pts, uint32_t n, float* out, float* vort) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (n == 0) return WT_OK;
  if (!pts || !out) return fail(c, WT_ERR_ARG, "wt_sample_flow: null buffer");
  float *dp = nullptr, *dout = nullptr, *dv = nullptr;
  WT_CUDA(c, cudaMallocAsync((void**)&dp, (size_t)n * 12, c->stream));
  WT_CUDA(c, cudaMallocAsync((void**)&dout, (size_t)n * 24, c->stream));
  if (vort) WT_CUDA(c, cudaMallocAsync((void**)&dv, (size_t)n * 4, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(dp, pts, (size_t)n * 12, cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, launch_sample_points(field_grid(c), dp, n, dout, dv, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(out, dout, (size_t)n * 24, cudaMemcpyDeviceToHost, c->stream));
  if (vort) WT_CUDA(c, cudaMemcpyAsync(vort, dv, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaFreeAsync(dp, c->stream));
  WT_CUDA(c, cudaFreeAsync(dout, c->stream));
  if (dv) WT_CUDA(c, cudaFreeAsync(dv, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

int wt_particles_step(wt_ctx* c, float* parts, int on_device, const wt_psim* p, const wt_view* v) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!parts || !p || !v) return fail(c, WT_ERR_ARG, "wt_particles_step: null argument");
  if (p->count == 0) return WT_OK;
  if (p->spawn_mode == 1u && (p->rake_rows == 0 || p->rake_cols == 0))
    return fail(c, WT_ERR_ARG, "wt_particles_step: rake spawn needs rake_rows, rake_cols > 0");
  PSimArgs a;
  a.count = p->count; a.spawnMode = p->spawn_mode; a.colorMode = p->color_mode; a.frame = p->frame;
  a.scatter = p->scatter; a.rakeRows = p->rake_rows; a.rakeCols = p->rake_cols;
  a.dt = p->dt; a.life = p->life;
  for (int k = 0; k < 3; k++) { a.smin[k] = p->spawn_min[k]; a.smax[k] = p->spawn_max[k]; }
  const size_t bytes = (size_t)p->count * 32;
  float4* d = reinterpret_cast<float4*>(parts);
  if (!on_device) {
    WT_CUDA(c, cudaMallocAsync((void**)&d, bytes, c->stream));
    WT_CUDA(c, cudaMemcpyAsync(d, parts, bytes, cudaMemcpyHostToDevice, c->stream));
  }
  WT_CUDA(c, launch_particles(field_grid(c), a, view_args(v), d, c->stream));
  if (!on_device) {
    WT_CUDA(c, cudaMemcpyAsync(parts, d, bytes, cudaMemcpyDeviceToHost, c->stream));
    WT_CUDA(c, cudaFreeAsync(d, c->stream));
    WT_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return WT_OK;
}

int wt_streamlines(wt_ctx* c, const wt_stream_params* s, const wt_view* v, float* pts) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!s || !v || !pts) return fail(c, WT_ERR_ARG, "wt_streamlines: null argument");
  if (s->lines == 0 || s->steps == 0) return WT_OK;
  if (s->seed_mode == 1u ? (s->per_emitter == 0 || s->emitters == 0 || s->emitters > 8)
                         : (s->rows == 0 || s->cols == 0))
    return fail(c, WT_ERR_ARG, "wt_streamlines: seeding needs rows, cols (or 1-8 emitters and per_emitter) > 0");
  if ((uint64_t)s->lines * s->steps >= (1ull << 31)) return fail(c, WT_ERR_ARG, "wt_streamlines: too many points");
  StreamArgs a;
  a.lines = s->lines; a.steps = s->steps; a.seedMode = s->seed_mode; a.colorMode = s->color_mode;
  a.rows = s->rows; a.cols = s->cols; a.perEmitter = s->per_emitter; a.emitters = s->emitters;
  for (int k = 0; k < 3; k++) { a.smin[k] = s->seed_min[k]; a.smax[k] = s->seed_max[k]; }
  a.stepLen = s->step_len; a.time = s->time;
  for (int e = 0; e < 8; e++)
    for (int k = 0; k < 4; k++) a.emit[e][k] = s->emitter[e][k];
  const size_t bytes = (size_t)s->lines * s->steps * 16;
  float4* d = nullptr;
  WT_CUDA(c, cudaMallocAsync((void**)&d, bytes, c->stream));
  WT_CUDA(c, launch_streamlines(field_grid(c), a, view_args(v), d, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(pts, d, bytes, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaFreeAsync(d, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

void wt_coef_ema_update(wt_coef_ema* e, double drag_n, double down_n, double q) {
  if (!e || !(q > 0.0)) return;
  const double a = e->n < 20 ? 0.15 : e->n < 60 ? 0.04 : 0.011;
  const double r = e->n == 0 ? 1.0 : a;
  e->cd += (drag_n / q - e->cd) * r;
  e->cl += (down_n / q - e->cl) * r;
  e->n++;
}

int wt_aeromap_sweep(wt_ctx* c, const wt_shape* base, const wt_sweep* s, wt_sweep_cell* out) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!base || !s || !out || !s->front || !s->rear || s->n_front == 0 || s->n_rear == 0)
    return fail(c, WT_ERR_ARG, "wt_aeromap_sweep: empty sweep");
  if (s->read_every == 0 || s->measure_steps < s->read_every || !(s->kmh > 0.0f))
    return fail(c, WT_ERR_ARG, "wt_aeromap_sweep: measure_steps >= read_every > 0 and kmh > 0 required");
  const auto even = [](uint32_t n) { return n + (n & 1u); };
  const uint32_t every = even(s->read_every);
  const uint32_t readings = s->measure_steps / s->read_every;
  const double v_real = (double)s->kmh / 3.6;
  uint32_t k = 0;
  for (uint32_t i = 0; i < s->n_front; i++) {
    for (uint32_t jj = 0; jj < s->n_rear; jj++, k++) {
      const uint32_t j = (i & 1u) ? s->n_rear - 1 - jj : jj;  // aeromap.ts:79-84
      wt_shape sh = *base;
      sh.ride_h = s->front[i];
      sh.rear_ride = s->rear[j];
      if ((rc = wt_voxelize(c, &sh))) return rc;
      wt_forces f;
      if (s->settle_steps && (rc = wt_step(c, (int)even(s->settle_steps), 0, 0.0f))) return rc;
      if ((rc = wt_read_forces(c, &f, 1))) return rc;  // readings of the settle phase are dropped
      wt_sweep_cell cell = {};
      for (uint32_t r = 0; r < readings; r++) {
        if ((rc = wt_step(c, (int)every, 0, 0.0f)) || (rc = wt_read_forces(c, &f, 1))) return rc;
        // engine.ts:750-753 in float, like the reference's JavaScript numbers (double)
        const double scale = (1.0 / 10000.0 / (double)f.steps) * 1.225 * (v_real / (double)c->sim.u_in) *
                             (v_real / (double)c->sim.u_in) * (double)c->grid.h * (double)c->grid.h * 2.0;
        for (int g = 0; g < 3; g++) {
          cell.group_drag_n[g] += (double)f.raw[3 * g] * scale;
          cell.group_down_n[g] += -(double)f.raw[3 * g + 1] * scale;
        }
      }
      double down = 0.0, drag = 0.0;
      for (int g = 0; g < 3; g++) {
        cell.group_drag_n[g] /= readings;
        cell.group_down_n[g] /= readings;
        down += cell.group_down_n[g];
        drag += cell.group_drag_n[g];
      }
      cell.down_kg = down / 9.81;
      cell.drag_n = drag;
      cell.efficiency = down / (drag > 1.0 ? drag : 1.0);
      cell.order = k;
      cell.readings = readings;
      out[(size_t)i * s->n_rear + j] = cell;
    }
  }
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
  uint64_t v = ((uint64_t)b->bx << 32) ^ ((uint64_t)b->by << 48);
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
  for (int k = 0; k < n; k++) {
    const bool last = (k == n - 1);
    cudaError_t e = launch_batch_step(b->storage, (k & 1) == 0, last, block, b->total_blocks, b->d_args, b->d_tiles,
                                      count, pending, s);
    if (e != cudaSuccess) return e;
    pending++;
    if (pending == b->pending_cap || last) {
      e = launch_force_reduce(b->d_reduce, count, pending, last, s);
      if (e != cudaSuccess) return e;
      pending = 0;
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
      cudaMalloc((void**)&b->d_reduce, count * sizeof(ReduceArgs)) != cudaSuccess) {
    b->err = "wt_batch_create: device tables";
    return cleanup(WT_ERR_NOMEM);
  }
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
  for (auto& sh : kShapes) {
    b->bx = sh[0];
    b->by = sh[1];
    const float ms = time_steps(b->stream, [&](int n) { return wt_batch_step(b, n, 0, 0.0f); });
    if (ms > 0.0f && ms < best) {
      best = ms;
      bbx = b->bx;
      bby = b->by;
    }
  }
  b->bx = bbx;
  b->by = bby;
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

const char* wt_batch_last_error(const wt_batch* b) { return b ? b->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

// ---------------------------------------------------------------- renderer
struct wt_renderer {
  wt_ctx* c = nullptr;
  uint32_t w = 0, h = 0, hw = 0, hh = 0;
  ushort4* scene = nullptr;
  ushort4* hist[2] = {nullptr, nullptr};
  ushort4* glow = nullptr;
  ushort4* bloom_a = nullptr;
  ushort4* bloom_b = nullptr;
  uchar4* out = nullptr;
  ushort4* g_albedo = nullptr;        // car G-buffer (engine.ts:297-303)
  ushort4* g_normal = nullptr;
  uchar4* g_material = nullptr;
  unsigned long long* acc = nullptr;  // glow fixed-point sums, w*h*4
  float4* staging = nullptr;          // host particle / line data copied for a draw
  size_t staging_bytes = 0;
  // mesh pass scratch, made on the first wt_render_mesh: depth, visibility keys,
  // decal counts / offsets / cursors (w*h each), grown buffers below
  float* m_depth = nullptr;
  unsigned long long* m_keys = nullptr;
  uint32_t* m_dcount = nullptr;
  uint32_t* m_doff = nullptr;
  uint32_t* m_dcur = nullptr;
  unsigned long long* m_nbig = nullptr;
  uint32_t* m_dslots = nullptr;
  size_t m_slots_cap = 0;
  float4* m_corners = nullptr;
  size_t m_corners_cap = 0;
  uint4* m_big = nullptr;
  size_t m_big_cap = 0;
  void* m_scan = nullptr;
  size_t m_scan_bytes = 0;
  wt::MeshDraw* m_draws = nullptr;
  size_t m_draws_cap = 0;
  float4* m_rig = nullptr;
};

struct wt_mesh {
  wt_ctx* c = nullptr;
  uint32_t n_verts = 0, n_indices = 0;
  float4* verts = nullptr;
  uint32_t* indices = nullptr;
  uint8_t* tags = nullptr;
  std::vector<uint8_t*> tex_data;          // device: each texture's levels back to back
  std::vector<wtx::Level> levels;          // every level of every texture (device pointers)
  std::vector<wt::MeshTex> texs;
  wtx::Level* d_levels = nullptr;          // device copies of the two tables
  wt::MeshTex* d_texs = nullptr;
  std::vector<wt_mesh_draw> draws;
};

namespace {
F3 f3(const float* v) { return F3{v[0], v[1], v[2]}; }
F3 f3n(float x, float y, float z) {  // normalize(e) = e / length(e), IEEE operations
  const float l = sqrtf(x * x + y * y + z * z);
  return F3{x / l, y / l, z / l};
}
int render_check(wt_renderer* r) {
  if (!r || !r->c) return WT_ERR_ARG;  // also: its context was destroyed
  return check_ctx(r->c);
}
void release_renderer_buffers(wt_renderer* r) {
  void* bufs[] = {r->scene,    r->hist[0],  r->hist[1],  r->glow,    r->bloom_a,   r->bloom_b, r->out,
                  r->acc,      r->staging,  r->g_albedo, r->g_normal, r->g_material, r->m_depth, r->m_keys,
                  r->m_dcount, r->m_doff,   r->m_dcur,   r->m_nbig,  r->m_dslots,  r->m_corners, r->m_big,
                  r->m_scan,   r->m_draws,  r->m_rig};
  for (void* b : bufs)
    if (b) cudaFree(b);
  r->m_depth = nullptr;
  r->m_keys = nullptr;
  r->m_dcount = r->m_doff = r->m_dcur = r->m_dslots = nullptr;
  r->m_nbig = nullptr;
  r->m_corners = nullptr;
  r->m_big = nullptr;
  r->m_scan = nullptr;
  r->m_draws = nullptr;
  r->m_rig = nullptr;
  r->m_slots_cap = r->m_corners_cap = r->m_big_cap = r->m_scan_bytes = r->m_draws_cap = 0;
  r->scene = r->hist[0] = r->hist[1] = r->glow = r->bloom_a = r->bloom_b = r->g_albedo = r->g_normal = nullptr;
  r->out = r->g_material = nullptr;
  r->acc = nullptr;
  r->staging = nullptr;
  r->staging_bytes = 0;
  r->c = nullptr;
}
void* target_ptr(wt_renderer* r, int t, size_t* bytes) {
  const size_t full = (size_t)r->w * r->h, half = (size_t)r->hw * r->hh;
  switch (t) {
    case WT_TARGET_SCENE: *bytes = full * 8; return r->scene;
    case WT_TARGET_HIST0: *bytes = full * 8; return r->hist[0];
    case WT_TARGET_HIST1: *bytes = full * 8; return r->hist[1];
    case WT_TARGET_GLOW: *bytes = full * 8; return r->glow;
    case WT_TARGET_BLOOM_A: *bytes = half * 8; return r->bloom_a;
    case WT_TARGET_BLOOM_B: *bytes = half * 8; return r->bloom_b;
    case WT_TARGET_OUTPUT: *bytes = full * 4; return r->out;
    case WT_TARGET_GALBEDO: *bytes = full * 8; return r->g_albedo;
    case WT_TARGET_GNORMAL: *bytes = full * 8; return r->g_normal;
    case WT_TARGET_GMATERIAL: *bytes = full * 4; return r->g_material;
    default: *bytes = 0; return nullptr;
  }
}
// Device copy of caller data for a draw: the pointer itself, or host data staged
// into the renderer's buffer (region `slot` of two, each `bytes` long).
int draw_source(wt_renderer* r, const float* p, int on_device, size_t bytes, size_t offset, const float4** out) {
  wt_ctx* c = r->c;
  if (on_device) {
    *out = reinterpret_cast<const float4*>(p);
    return WT_OK;
  }
  WT_CUDA(c, cudaMemcpyAsync(reinterpret_cast<char*>(r->staging) + offset, p, bytes, cudaMemcpyHostToDevice, c->stream));
  *out = reinterpret_cast<const float4*>(reinterpret_cast<char*>(r->staging) + offset);
  return WT_OK;
}
}  // namespace

void wt_render_destroy(wt_renderer* r) {
  if (!r) return;
  if (wt_ctx* c = r->c) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (size_t i = 0; i < c->renderers.size(); i++)
      if (c->renderers[i] == r) {
        c->renderers.erase(c->renderers.begin() + (long)i);
        break;
      }
    release_renderer_buffers(r);
  }
  delete r;
}

int wt_render_create(wt_ctx* c, uint32_t width, uint32_t height, wt_renderer** out) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!out) return fail(c, WT_ERR_ARG, "wt_render_create: null output");
  *out = nullptr;
  if (width == 0 || height == 0 || width > 16384 || height > 16384)
    return fail(c, WT_ERR_ARG, "wt_render_create: width and height must be 1..16384");
  wt_renderer* r = new wt_renderer;
  r->c = c;
  r->w = width;
  r->h = height;
  r->hw = width >> 1 ? width >> 1 : 1;   // engine.ts:291: max(1, w >> 1)
  r->hh = height >> 1 ? height >> 1 : 1;
  const size_t full = (size_t)width * height, half = (size_t)r->hw * r->hh;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, c->stream);
  };
  alloc((void**)&r->scene, full * 8);
  alloc((void**)&r->hist[0], full * 8);
  alloc((void**)&r->hist[1], full * 8);
  alloc((void**)&r->glow, full * 8);
  alloc((void**)&r->bloom_a, half * 8);
  alloc((void**)&r->bloom_b, half * 8);
  alloc((void**)&r->out, full * 4);
  alloc((void**)&r->acc, full * 32);
  alloc((void**)&r->g_albedo, full * 8);
  alloc((void**)&r->g_normal, full * 8);
  alloc((void**)&r->g_material, full * 4);
  if (e != cudaSuccess) {
    release_renderer_buffers(r);
    delete r;
    return fail(c, e == cudaErrorMemoryAllocation ? WT_ERR_NOMEM : WT_ERR_CUDA,
                std::string("wt_render_create: ") + cudaGetErrorString(e));
  }
  c->renderers.push_back(r);
  *out = r;
  return WT_OK;
}

int wt_render_scene(wt_renderer* r, const wt_cam* cam, const wt_look* look, const wt_view* view) {
  int rc = render_check(r);
  if (rc) return rc;
  wt_ctx* c = r->c;
  if (!cam || !look || !view) return fail(c, WT_ERR_ARG, "wt_render_scene: null argument");
  SceneArgs a;
  a.shape = c->shape;
  a.car = car_view(c);
  a.g = field_grid(c);
  a.view = view_args(view);
  a.pos = f3(cam->pos); a.fwd = f3(cam->fwd); a.right = f3(cam->right); a.up = f3(cam->up);
  a.tan_half = cam->tan_half; a.aspect = cam->aspect; a.time = cam->time; a.road_speed = cam->road_speed;
  a.jitter_x = cam->jitter[0]; a.jitter_y = cam->jitter[1];
  a.bmin = f3(look->bmin); a.bmax = f3(look->bmax);
  // toLinear (render-wgsl.ts:40) of the livery colours, once per frame: the same
  // function the shader evaluates per hit, so the same bits
  a.paint_lin = F3{wtm::powf(look->paint[0], 2.2f), wtm::powf(look->paint[1], 2.2f), wtm::powf(look->paint[2], 2.2f)};
  a.accent_lin = F3{wtm::powf(look->accent[0], 2.2f), wtm::powf(look->accent[1], 2.2f), wtm::powf(look->accent[2], 2.2f)};
  a.surf_mode = look->surf_mode; a.palette = look->palette; a.carbon_body = look->carbon_body; a.is_f1 = look->is_f1;
  a.slice_axis = look->slice_axis; a.show_flow = look->show_flow;
  a.slice_pos = look->slice_pos; a.slice_alpha = look->slice_alpha;
  a.mesh_mode = look->mesh_mode; a.cooling = look->cooling;
  a.g_albedo = r->g_albedo; a.g_normal = r->g_normal; a.g_material = r->g_material;
  a.key = f3n(-0.32f, 0.90f, 0.30f);    // KEY (render-wgsl.ts:38)
  a.fill_a = f3n(0.6f, 0.35f, -0.7f);   // shadeSurface fill lights (render-wgsl.ts:265)
  a.fill_b = f3n(0.6f, 0.35f, 0.7f);
  a.w = r->w; a.h = r->h;
  a.scene = r->scene;
  WT_CUDA(c, launch_render_scene(a, c->stream));
  return WT_OK;
}

int wt_render_taa(wt_renderer* r, const wt_taa* t, int cur) {
  int rc = render_check(r);
  if (rc) return rc;
  wt_ctx* c = r->c;
  if (!t || (cur != 0 && cur != 1)) return fail(c, WT_ERR_ARG, "wt_render_taa: null uniform or cur not 0/1");
  TaaArgs a;
  for (int i = 0; i < 16; i++) a.m[i] = t->prev_view_proj[i];
  a.cam_pos = f3(t->cam_pos); a.fwd = f3(t->fwd); a.right = f3(t->right); a.up = f3(t->up);
  a.tan_half = t->tan_half; a.aspect = t->aspect; a.blend = t->blend;
  a.w = r->w; a.h = r->h;
  a.cur = r->scene;
  a.hist = r->hist[1 - cur];
  a.out = r->hist[cur];
  WT_CUDA(c, launch_taa(a, c->stream));
  return WT_OK;
}

int wt_render_glow(wt_renderer* r, const float* parts, int parts_on_device, const wt_pdraw* pd, const float* pts,
                   int pts_on_device, const wt_sdraw* sd) {
  int rc = render_check(r);
  if (rc) return rc;
  wt_ctx* c = r->c;
  if ((parts && !pd) || (pts && !sd)) return fail(c, WT_ERR_ARG, "wt_render_glow: draw data without its uniform");
  if (pts && sd->steps < 2) return fail(c, WT_ERR_ARG, "wt_render_glow: streamlines need steps >= 2");
  const size_t texels = (size_t)r->w * r->h;
  const size_t pbytes = parts ? (size_t)pd->count * 32 : 0, sbytes = pts ? (size_t)sd->lines * sd->steps * 16 : 0;
  const uint64_t pinst = parts ? 2ull * pd->count : 0, sinst = pts ? (uint64_t)sd->lines * 2ull * (sd->steps - 1u) : 0;
  if (pinst >= (1ull << 31) || sinst >= (1ull << 31)) return fail(c, WT_ERR_ARG, "wt_render_glow: too many instances");
  const size_t need = (parts_on_device ? 0 : pbytes) + (pts_on_device ? 0 : sbytes);
  if (need > r->staging_bytes) {
    WT_CUDA(c, cudaStreamSynchronize(c->stream));
    if (r->staging) cudaFree(r->staging);
    r->staging = nullptr;
    r->staging_bytes = 0;
    WT_CUDA(c, cudaMalloc((void**)&r->staging, need));
    r->staging_bytes = need;
  }
  WT_CUDA(c, cudaMemsetAsync(r->acc, 0, texels * 32, c->stream));
  auto base = [&](DrawArgs& d) {
    d.w = r->w; d.h = r->h;
    d.scene = r->scene;
    d.acc = r->acc;
  };
  size_t off = 0;
  if (parts && pinst) {
    DrawArgs d{};
    base(d);
    d.kind = 0;
    for (int i = 0; i < 16; i++) d.m[i] = pd->view_proj[i];
    d.cam_pos = f3(pd->cam_pos);
    d.width = pd->width; d.res_x = pd->res[0]; d.res_y = pd->res[1];
    d.trail = pd->trail; d.alpha = pd->alpha; d.fade_in = pd->fade_in;
    d.count = pd->count; d.palette = pd->palette;
    d.instances = (uint32_t)pinst;
    if ((rc = draw_source(r, parts, parts_on_device, pbytes, off, &d.data))) return rc;
    if (!parts_on_device) off += pbytes;
    WT_CUDA(c, launch_glow_draw(d, c->stream));
  }
  if (pts && sinst) {
    DrawArgs d{};
    base(d);
    d.kind = 1;
    for (int i = 0; i < 16; i++) d.m[i] = sd->view_proj[i];
    d.cam_pos = f3(sd->cam_pos);
    d.width = sd->width; d.res_x = sd->res[0]; d.res_y = sd->res[1];
    d.time = sd->time; d.intensity = sd->intensity; d.pulse = sd->pulse;
    d.lines = sd->lines; d.steps = sd->steps; d.palette = sd->palette;
    d.instances = (uint32_t)sinst;
    if ((rc = draw_source(r, pts, pts_on_device, sbytes, off, &d.data))) return rc;
    WT_CUDA(c, launch_glow_draw(d, c->stream));
  }
  WT_CUDA(c, launch_glow_resolve(r->acc, r->glow, (uint32_t)texels, c->stream));
  return WT_OK;
}

int wt_render_bloom(wt_renderer* r) {
  int rc = render_check(r);
  if (rc) return rc;
  wt_ctx* c = r->c;
  BlurArgs a;
  for (int k = -6; k <= 6; k++) a.wk[k + 6] = wtm::expf(-(float)(k * k) / 14.0f);
  a.gain = 1.0f;
  // engine.ts:316: glow (full size) -> bloom A (half size), dir (1, 0), spacing 3
  a.dir_x = 1.0f; a.dir_y = 0.0f; a.spacing = 3.0f;
  a.sw = r->w; a.sh = r->h; a.dw = r->hw; a.dh = r->hh;
  a.src = r->glow; a.dst = r->bloom_a;
  WT_CUDA(c, launch_blur(a, c->stream));
  // engine.ts:317: bloom A -> bloom B, dir (0, 1), spacing 1.5
  a.dir_x = 0.0f; a.dir_y = 1.0f; a.spacing = 1.5f;
  a.sw = r->hw; a.sh = r->hh;
  a.src = r->bloom_a; a.dst = r->bloom_b;
  WT_CUDA(c, launch_blur(a, c->stream));
  return WT_OK;
}

int wt_render_present(wt_renderer* r, const wt_post* post, int cur) {
  int rc = render_check(r);
  if (rc) return rc;
  wt_ctx* c = r->c;
  if (!post || (cur != 0 && cur != 1)) return fail(c, WT_ERR_ARG, "wt_render_present: null uniform or cur not 0/1");
  PresentArgs a;
  a.bloom = post->bloom; a.exposure = post->exposure;
  a.w = r->w; a.h = r->h; a.gw = r->w; a.gh = r->h; a.bw = r->hw; a.bh = r->hh;
  a.scene = r->hist[cur];
  a.glow = r->glow;
  a.bloom_tex = r->bloom_b;
  a.out = r->out;
  WT_CUDA(c, launch_present(a, c->stream));
  return WT_OK;
}

int wt_render_read(wt_renderer* r, int target, void* host) {
  int rc = render_check(r);
  if (rc) return rc;
  wt_ctx* c = r->c;
  size_t bytes = 0;
  void* p = target_ptr(r, target, &bytes);
  if (!p || !host) return fail(c, WT_ERR_ARG, "wt_render_read: unknown target or null buffer");
  WT_CUDA(c, cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

int wt_render_write(wt_renderer* r, int target, const void* host) {
  int rc = render_check(r);
  if (rc) return rc;
  wt_ctx* c = r->c;
  size_t bytes = 0;
  void* p = target_ptr(r, target, &bytes);
  if (!p || !host) return fail(c, WT_ERR_ARG, "wt_render_write: unknown target or null buffer");
  WT_CUDA(c, cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  return WT_OK;
}

namespace {
void release_mesh_buffers(wt_mesh* m) {
  void* bufs[] = {m->verts, m->indices, m->tags, m->d_levels, m->d_texs};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (uint8_t* t : m->tex_data) cudaFree(t);
  m->verts = nullptr;
  m->indices = nullptr;
  m->tags = nullptr;
  m->d_levels = nullptr;
  m->d_texs = nullptr;
  m->tex_data.clear();
  m->levels.clear();
  m->texs.clear();
  m->c = nullptr;
}
int mesh_check(wt_mesh* m) {
  if (!m || !m->c) return WT_ERR_ARG;  // also: its context was destroyed
  return check_ctx(m->c);
}
// halveRgba (mesh-car.ts:30-44): the next mip level, a rounded 2 x 2 box
std::vector<uint8_t> halve_rgba(const std::vector<uint8_t>& src, uint32_t w, uint32_t h, uint32_t* ow, uint32_t* oh) {
  const uint32_t nw = w >> 1 ? w >> 1 : 1, nh = h >> 1 ? h >> 1 : 1;
  std::vector<uint8_t> out((size_t)nw * nh * 4);
  for (uint32_t y = 0; y < nh; y++) {
    const size_t y0 = std::min(h - 1, y * 2), y1 = std::min(h - 1, y * 2 + 1);
    for (uint32_t x = 0; x < nw; x++) {
      const size_t x0 = std::min(w - 1, x * 2), x1 = std::min(w - 1, x * 2 + 1);
      for (int k = 0; k < 4; k++) {
        const unsigned sum = src[(y0 * w + x0) * 4 + k] + src[(y0 * w + x1) * 4 + k] + src[(y1 * w + x0) * 4 + k] +
                             src[(y1 * w + x1) * 4 + k] + 2u;
        out[((size_t)y * nw + x) * 4 + k] = (uint8_t)(sum >> 2);
      }
    }
  }
  *ow = nw;
  *oh = nh;
  return out;
}
// grow a device buffer to at least `need` elements (contents not kept)
template <class T>
cudaError_t grow(T** p, size_t* cap, size_t need) {
  if (*cap >= need && *p) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t n = need > 0 ? need : 1;
  const cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e == cudaSuccess) *cap = n;
  return e;
}
}  // namespace

int wt_png_unfilter(const uint8_t* filtered, uint32_t rows, uint32_t row_bytes, uint32_t bpp, uint8_t* out) {
  if (!filtered || !out || bpp == 0 || bpp > 8) return WT_ERR_ARG;
  const uint8_t* src = filtered;
  for (uint32_t y = 0; y < rows; y++, src += (size_t)row_bytes + 1) {
    const uint8_t type = src[0];
    const uint8_t* f = src + 1;
    uint8_t* o = out + (size_t)y * row_bytes;
    const uint8_t* up = y ? o - row_bytes : nullptr;
    for (uint32_t i = 0; i < row_bytes; i++) {
      const int a = i >= bpp ? o[i - bpp] : 0;  // left, above, above-left (0 outside the image)
      const int b = up ? up[i] : 0;
      const int c = (up && i >= bpp) ? up[i - bpp] : 0;
      int pred;
      switch (type) {
        case 0: pred = 0; break;
        case 1: pred = a; break;
        case 2: pred = b; break;
        case 3: pred = (a + b) >> 1; break;
        case 4: {  // Paeth: the neighbour closest to a + b - c, ties to a, then b
          const int p = a + b - c, pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
          pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
          break;
        }
        default: return WT_ERR_ARG;
      }
      o[i] = (uint8_t)(f[i] + pred);
    }
  }
  return WT_OK;
}

int wt_mesh_create(wt_ctx* c, const float* verts, uint32_t n_verts, const uint32_t* indices, uint32_t n_indices,
                   const uint8_t* tags, wt_mesh** out) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!out) return fail(c, WT_ERR_ARG, "wt_mesh_create: null output");
  *out = nullptr;
  if (!verts || !indices || !tags || n_verts == 0 || n_indices == 0)
    return fail(c, WT_ERR_ARG, "wt_mesh_create: empty or null vertex, index or tag buffer");
  for (uint32_t i = 0; i < n_indices; i++)
    if (indices[i] >= n_verts)
      return fail(c, WT_ERR_ARG, "wt_mesh_create: index " + std::to_string(i) + " out of range");
  wt_mesh* m = new wt_mesh;
  m->c = c;
  m->n_verts = n_verts;
  m->n_indices = n_indices;
  cudaError_t e = cudaMalloc((void**)&m->verts, (size_t)n_verts * 32);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->indices, (size_t)n_indices * 4);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->tags, n_verts);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->verts, verts, (size_t)n_verts * 32, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->indices, indices, (size_t)n_indices * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->tags, tags, n_verts, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    release_mesh_buffers(m);
    delete m;
    return fail(c, e == cudaErrorMemoryAllocation ? WT_ERR_NOMEM : WT_ERR_CUDA,
                std::string("wt_mesh_create: ") + cudaGetErrorString(e));
  }
  c->meshes.push_back(m);
  *out = m;
  return WT_OK;
}

void wt_mesh_destroy(wt_mesh* m) {
  if (!m) return;
  if (wt_ctx* c = m->c) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (size_t i = 0; i < c->meshes.size(); i++)
      if (c->meshes[i] == m) {
        c->meshes.erase(c->meshes.begin() + (long)i);
        break;
      }
    release_mesh_buffers(m);
  }
  delete m;
}

int wt_mesh_add_texture(wt_mesh* m, uint32_t width, uint32_t height, const uint8_t* rgba, int32_t* index) {
  int rc = mesh_check(m);
  if (rc) return rc;
  wt_ctx* c = m->c;
  if (!rgba || !index || width == 0 || height == 0 || width > 16384 || height > 16384)
    return fail(c, WT_ERR_ARG, "wt_mesh_add_texture: null buffer or size not 1..16384");
  // levels: floor(log2(max(w, h))) + 1 (mesh-car.ts:115)
  uint32_t big = width > height ? width : height, n_levels = 0;
  while (big) {
    n_levels++;
    big >>= 1;
  }
  std::vector<std::vector<uint8_t>> lv(1, std::vector<uint8_t>(rgba, rgba + (size_t)width * height * 4));
  std::vector<uint32_t> ws{width}, hs{height};
  size_t total = lv[0].size();
  for (uint32_t l = 1; l < n_levels; l++) {
    uint32_t nw, nh;
    lv.push_back(halve_rgba(lv.back(), ws.back(), hs.back(), &nw, &nh));
    ws.push_back(nw);
    hs.push_back(nh);
    total += lv.back().size();
  }
  uint8_t* d = nullptr;
  WT_CUDA(c, cudaMalloc((void**)&d, total));
  m->tex_data.push_back(d);
  size_t off = 0;
  wt::MeshTex t{(uint32_t)m->levels.size(), n_levels};
  for (uint32_t l = 0; l < n_levels; l++) {
    WT_CUDA(c, cudaMemcpyAsync(d + off, lv[l].data(), lv[l].size(), cudaMemcpyHostToDevice, c->stream));
    m->levels.push_back(wtx::Level{d + off, (int)ws[l], (int)hs[l]});
    off += lv[l].size();
  }
  m->texs.push_back(t);
  // the tables, copied whole (they are small)
  if (m->d_levels) cudaFree(m->d_levels);
  if (m->d_texs) cudaFree(m->d_texs);
  m->d_levels = nullptr;
  m->d_texs = nullptr;
  WT_CUDA(c, cudaMalloc((void**)&m->d_levels, m->levels.size() * sizeof(wtx::Level)));
  WT_CUDA(c, cudaMalloc((void**)&m->d_texs, m->texs.size() * sizeof(wt::MeshTex)));
  WT_CUDA(c, cudaMemcpyAsync(m->d_levels, m->levels.data(), m->levels.size() * sizeof(wtx::Level),
                             cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaMemcpyAsync(m->d_texs, m->texs.data(), m->texs.size() * sizeof(wt::MeshTex), cudaMemcpyHostToDevice,
                             c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  *index = (int32_t)m->texs.size() - 1;
  return WT_OK;
}

int wt_mesh_add_draw(wt_mesh* m, const wt_mesh_draw* d) {
  int rc = mesh_check(m);
  if (rc) return rc;
  wt_ctx* c = m->c;
  if (!d) return fail(c, WT_ERR_ARG, "wt_mesh_add_draw: null draw");
  if ((uint64_t)d->first_index + d->count > m->n_indices)
    return fail(c, WT_ERR_ARG, "wt_mesh_add_draw: index range beyond the index buffer");
  if (d->has_tex > 0.5f && (d->texture < 0 || d->texture >= (int32_t)m->texs.size()))
    return fail(c, WT_ERR_ARG, "wt_mesh_add_draw: has_tex set without a valid texture");
  m->draws.push_back(*d);
  return WT_OK;
}

int wt_render_mesh(wt_renderer* r, wt_mesh* m, const wt_mesh_cam* cam, const wt_rig* rig, int optional) {
  int rc = render_check(r);
  if (rc) return rc;
  wt_ctx* c = r->c;
  if (!m || m->c != c) return fail(c, WT_ERR_ARG, "wt_render_mesh: mesh missing or made on another context");
  if (!cam || !rig) return fail(c, WT_ERR_ARG, "wt_render_mesh: null camera or rig");
  // the draws of this frame in record order, with their corner and triangle bases
  std::vector<wt::MeshDraw> dl;
  uint64_t corners = 0, tris = 0;
  for (const wt_mesh_draw& d : m->draws) {
    if (d.optional && !optional) continue;
    wt::MeshDraw x{};
    for (int k = 0; k < 4; k++) x.color[k] = d.color[k];
    x.metal = d.metal; x.rough = d.rough; x.coat = d.coat; x.alpha_cut = d.alpha_cut;
    x.emissive = d.emissive; x.has_tex = d.has_tex; x.is_body = d.is_body;
    x.first_index = d.first_index;
    x.count = d.count - d.count % 3u;
    x.tex = d.has_tex > 0.5f ? d.texture : -1;
    x.blend = d.blend ? 1u : 0u;
    x.corner_base = (uint32_t)corners;
    x.tri_base = (uint32_t)tris;
    corners += x.count;
    tris += x.count / 3u;
    dl.push_back(x);
  }
  if (tris >= 0x7fffffffull || corners >= 0xffffffffull)
    return fail(c, WT_ERR_ARG, "wt_render_mesh: more than 2^31 - 1 triangles");
  const size_t px = (size_t)r->w * r->h;
  if (!r->m_depth) {  // per-pixel scratch, once per renderer
    WT_CUDA(c, cudaMalloc((void**)&r->m_depth, px * 4));
    WT_CUDA(c, cudaMalloc((void**)&r->m_keys, px * 8));
    WT_CUDA(c, cudaMalloc((void**)&r->m_dcount, px * 4));
    WT_CUDA(c, cudaMalloc((void**)&r->m_doff, px * 4));
    WT_CUDA(c, cudaMalloc((void**)&r->m_dcur, px * 4));
    WT_CUDA(c, cudaMalloc((void**)&r->m_nbig, 8));
  }
  WT_CUDA(c, grow(&r->m_corners, &r->m_corners_cap, (size_t)corners * 3));
  WT_CUDA(c, grow(&r->m_big, &r->m_big_cap, (size_t)tris * 2));
  WT_CUDA(c, grow(&r->m_draws, &r->m_draws_cap, dl.size()));
  if (!dl.empty())  // pageable source: copied before the call returns
    WT_CUDA(c, cudaMemcpyAsync(r->m_draws, dl.data(), dl.size() * sizeof(wt::MeshDraw), cudaMemcpyHostToDevice,
                               c->stream));
  wt::MeshArgs a{};
  a.verts = m->verts; a.indices = m->indices; a.tags = m->tags;
  a.levels = m->d_levels; a.texs = m->d_texs;
  a.draws = r->m_draws; a.n_draws = (uint32_t)dl.size();
  for (int k = 0; k < 16; k++) a.vp[k] = cam->view_proj[k];
  for (int k = 0; k < 3; k++) a.cam_pos[k] = cam->cam_pos[k];
  a.ride_h = cam->ride_h; a.jitter[0] = cam->jitter[0]; a.jitter[1] = cam->jitter[1];
  a.rake = cam->rake; a.base_ride = cam->base_ride;
  // the mesh's rig travels in its own copy so the scene's car model stays as set
  if (!r->m_rig) WT_CUDA(c, cudaMalloc((void**)&r->m_rig, sizeof(wt_rig)));
  WT_CUDA(c, cudaMemcpyAsync(r->m_rig, rig, sizeof(wt_rig), cudaMemcpyHostToDevice, c->stream));
  a.rig = r->m_rig;
  a.w = r->w; a.h = r->h;
  a.cpos = r->m_corners;
  a.cattr = r->m_corners + corners;
  a.depth = r->m_depth; a.keys = r->m_keys;
  a.big = r->m_big; a.big_count = r->m_nbig; a.big_cap = (uint32_t)std::min<size_t>(r->m_big_cap, 0xffffffffu);
  a.g_albedo = r->g_albedo; a.g_normal = r->g_normal; a.g_material = r->g_material;
  a.dcount = r->m_dcount; a.doff = r->m_doff; a.dcur = r->m_dcur; a.dslots = r->m_dslots;
  WT_CUDA(c, launch_mesh_clear(a, c->stream));
  WT_CUDA(c, launch_mesh_vertex(a, (uint32_t)corners, c->stream));
  for (size_t i = 0; i < dl.size();) {  // runs of opaque draws and runs of decals
    size_t j = i;
    while (j < dl.size() && dl[j].blend == dl[i].blend) j++;
    const uint32_t tri0 = dl[i].tri_base, tri1 = dl[j - 1].tri_base + dl[j - 1].count / 3u;
    if (!dl[i].blend) {
      WT_CUDA(c, launch_mesh_opaque(a, (uint32_t)i, (uint32_t)j, tri0, tri1, c->stream));
    } else if (tri1 > tri0) {
      WT_CUDA(c, launch_mesh_decal_count(a, (uint32_t)i, (uint32_t)j, tri0, tri1, c->stream));
      size_t need = 0;
      WT_CUDA(c, launch_mesh_decal_scan(a, nullptr, &need, c->stream));
      WT_CUDA(c, grow((uint8_t**)&r->m_scan, &r->m_scan_bytes, need));
      WT_CUDA(c, launch_mesh_decal_scan(a, r->m_scan, &need, c->stream));
      uint32_t last[2] = {0, 0};
      WT_CUDA(c, cudaMemcpyAsync(&last[0], r->m_doff + px - 1, 4, cudaMemcpyDeviceToHost, c->stream));
      WT_CUDA(c, cudaMemcpyAsync(&last[1], r->m_dcount + px - 1, 4, cudaMemcpyDeviceToHost, c->stream));
      WT_CUDA(c, cudaStreamSynchronize(c->stream));
      WT_CUDA(c, grow(&r->m_dslots, &r->m_slots_cap, (size_t)last[0] + last[1]));
      a.dslots = r->m_dslots;
      WT_CUDA(c, launch_mesh_decal_blend(a, (uint32_t)i, (uint32_t)j, tri0, tri1, c->stream));
    }
    i = j;
  }
  return WT_OK;
}
