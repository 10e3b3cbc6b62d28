// The C ABI of the render passes (src/engine/render-wgsl.ts, engine.ts:290-327,
// 714-725) and of the car mesh G-buffer pass (render-wgsl.ts:647-760,
// src/engine/mesh-car.ts), into headless render targets.
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
}  // namespace

void wt::api::release_renderer_buffers(wt_renderer* r) {
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

namespace {
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
}  // namespace

void wt::api::release_mesh_buffers(wt_mesh* m) {
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

namespace {
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
