// The C ABI of the field consumers (sampleFlow / vorticityAt, the particle and
// streamline passes: src/engine/wgsl.ts:324-366,516-594,
// src/engine/render-wgsl.ts:520-576), the body-coefficient averaging
// (src/main.ts:590-596) and the aero-map sweep loop (src/ui/aeromap.ts:73-114).
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

FieldGrid wt::api::field_grid(const wt_ctx* c) {
  FieldGrid g;
  g.nx = c->nx; g.ny = c->ny; g.nz = c->nz;
  g.ox = c->grid.origin[0]; g.oy = c->grid.origin[1]; g.oz = c->grid.origin[2];
  g.h = c->grid.h;
  g.fields = c->fields;
  g.temps = c->tA;
  return g;
}
ViewArgs wt::api::view_args(const wt_view* v) {
  ViewArgs a;
  a.uIn = v->u_in; a.vReal = v->v_real; a.cpMin = v->cp_min; a.cpMax = v->cp_max;
  a.tMin = v->t_min; a.tMax = v->t_max; a.speedMax = v->speed_max; a.vortMax = v->vort_max;
  return a;
}

extern "C" {

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

}  // extern "C"
