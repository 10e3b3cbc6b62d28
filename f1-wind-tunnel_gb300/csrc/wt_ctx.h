// Host-side state of libwt's C ABI, shared by its translation units: the
// lattice context (wt_ctx), the batch (wt_batch), and the helpers the API units
// call on them (error reporting, device allocation, the step sequence and its
// CUDA graphs, force reduction, block geometry).  Not installed.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "wt_fields.h"
#include "wt_internal.h"

#define WT_ASYNC_SLOTS 16  // force readbacks in flight per context

struct wt_renderer;
struct wt_mesh;

struct wt_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  wt_grid grid{};
  wt_sim sim{};
  uint32_t nx = 0, ny = 0, nz = 0;
  uint64_t n = 0, np = 0;
  size_t elem = 4;
  wt::StepGeom geom{};
  uint32_t sm_count = 0;
  uint64_t l2_bytes = 0;        // the device's L2 size
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
  wt::ForceSlot* slots = nullptr;
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
  wt::ReduceArgs* d_reduce = nullptr;          // device: this lattice's reduction record
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
  wt::StepArgs* d_args = nullptr;
  wt::BatchTiles* d_tiles = nullptr;
  wt::ReduceArgs* d_reduce = nullptr;
  uint32_t total_blocks = 0;
  uint32_t pending_cap = 1;
  // persistent launch (batch_persist_kernel): on/off, its grid, the grid
  // barrier's device words and the pinned copy of the barrier's expiry flag
  bool persist = false;
  uint32_t persist_grid = 0;
  unsigned int* d_sync = nullptr;
  unsigned int* h_flag = nullptr;
  uint64_t version = ~0ull;                // sum of member versions the device tables were built for
  std::vector<wt_ctx::Graph> graphs;
  std::string err;
};

namespace wt {
namespace api {

// error text of the last failed wt_create / wt_batch_create on this thread
extern thread_local std::string g_create_error;
// records msg as the context's (or the thread's creation) error, returns code
int fail(wt_ctx* c, int code, const std::string& msg);

#define WT_CUDA(c, call)                                                                       \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return fail((c), e_ == cudaErrorMemoryAllocation ? WT_ERR_NOMEM : WT_ERR_CUDA,           \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                         \
  } while (0)

template <class T>
int dalloc(wt_ctx* c, T** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) return fail(c, WT_ERR_NOMEM, std::string("cudaMalloc ") + std::to_string(bytes) + " B: " + cudaGetErrorString(e));
  c->device_bytes += bytes;
  return WT_OK;
}

bool valid_storage(uint32_t s);
// x-dependent base relaxation time (wgsl.ts:260) and its admissibility
float tau0_at(const wt_sim& s, uint32_t nx, uint32_t x);
bool valid_tau(const wt_sim& s, uint32_t nx);
int apply_sim(wt_ctx* c);
uint32_t warps_per_block(const StepGeom& g);
ReduceArgs reduce_args(const wt_ctx* c);
int flush_forces(wt_ctx* c);
int rebuild_links(wt_ctx* c);
StepArgs step_args(const wt_ctx* c);
cudaError_t enqueue_heat(wt_ctx* c, int heat_passes, float dt, cudaStream_t s);
cudaError_t enqueue_frame(wt_ctx* c, int n, int heat_passes, float dt, uint32_t pending0, cudaStream_t s);
int set_geometry(wt_ctx* c, uint32_t bx, uint32_t by);
int check_ctx(wt_ctx* c);
// New lattice; `ext` (may be null) is a stream owned by the caller, e.g. a batch.
int create_ctx(const wt_grid* grid, const wt_sim* sim, cudaStream_t ext, wt_ctx** out);
// the context's W17 model, field and view arguments as the kernels take them
CarView car_view(const wt_ctx* c);
FieldGrid field_grid(const wt_ctx* c);
ViewArgs view_args(const wt_view* v);
// device buffers of a renderer / mesh whose lattice is being destroyed
void release_renderer_buffers(wt_renderer* r);
void release_mesh_buffers(wt_mesh* m);

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

}  // namespace api
}  // namespace wt
