// TEST INFRASTRUCTURE ONLY - C entry points of the oracle (wt_oracle.hpp) for
// the Python tests and the benchmark's CPU-baseline leg.  Mirrors the engine
// calls of src/engine/engine.ts: reset (:371), setShape/voxelize (:426-470),
// the frame's LBM and heat dispatches (:708-712), force readout (:739-761) and
// debugRead (:763-768).
#include "wt_oracle.hpp"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {
struct Handle {
  int fp64;
  wto::Lattice<float>* f;
  wto::Lattice<double>* d;
};
template <class Fn> void with(void* h, Fn fn) {
  Handle* H = (Handle*)h;
  if (H->fp64) fn(*H->d); else fn(*H->f);
}
}  // namespace

extern "C" {

void* wto_new(int nx, int ny, int nz, float ox, float oy, float oz, float h, int fp64) {
  float o[3] = {ox, oy, oz};
  Handle* H = new Handle();
  H->fp64 = fp64;
  H->f = fp64 ? nullptr : new wto::Lattice<float>(nx, ny, nz, o, h);
  H->d = fp64 ? new wto::Lattice<double>(nx, ny, nz, o, h) : nullptr;
  return H;
}
void wto_free(void* h) {
  Handle* H = (Handle*)h;
  delete H->f; delete H->d; delete H;
}
// p: uIn, tau0, smag, sponge_cells, sponge_amp, inlet_cells, inlet_amp, cool, diffuse, src_mix
void wto_set_params(void* h, const float* p) {
  with(h, [&](auto& L) {
    L.prm.uIn = p[0]; L.prm.tau0 = p[1]; L.prm.smag = p[2]; L.prm.sponge_cells = p[3];
    L.prm.sponge_amp = p[4]; L.prm.inlet_cells = p[5]; L.prm.inlet_amp = p[6];
    L.prm.cool = p[7]; L.prm.diffuse = p[8]; L.prm.src_mix = p[9];
  });
}
void wto_reset(void* h) { with(h, [&](auto& L) { L.reset(); }); }
// shape: 30 32-bit words, the wt_shape layout (24 Shape words + box centre + box half size)
void wto_voxelize(void* h, const void* shape) {
  wto::Shape s;
  memcpy(&s, shape, sizeof(s));
  with(h, [&](auto& L) { L.voxelize(s); });
}
// The scene SDF at n points (xyz): out[2k] distance, out[2k+1] material.
void wto_scene_sdf(const void* shape, const float* pts, uint32_t n, float* out) {
  wto::Shape s;
  memcpy(&s, shape, sizeof(s));
  wto::Sdf sdf(s);
  for (uint32_t k = 0; k < n; k++) {
    const wto::F2 r = sdf.scene(wto::f3(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]));
    out[2 * k] = r.x;
    out[2 * k + 1] = r.y;
  }
}
void wto_set_solid(void* h, const uint32_t* solid, const float* emit) {
  with(h, [&](auto& L) {
    memcpy(L.solid.data(), solid, L.n * 4);
    memcpy(L.emit.data(), emit, L.n * 4);
  });
}
void wto_steps(void* h, int n) { with(h, [&](auto& L) { L.steps(n); }); }
void wto_heat(void* h, float dt) { with(h, [&](auto& L) { L.heat(dt); }); }

// fields (4n), solid (n), emit (n), temps (n), populations of the current buffer (19n),
// forces i32[12], forces64[9]; any pointer may be null.  Float outputs are converted from
// the lattice's precision.
void wto_read(void* h, float* fields, uint32_t* solid, float* emit, float* temps, float* f, int32_t* forces,
              double* forces64, int reset_forces) {
  with(h, [&](auto& L) {
    size_t n = L.n;
    if (fields) for (size_t i = 0; i < 4 * n; i++) fields[i] = (float)L.fields[i];
    if (solid) memcpy(solid, L.solid.data(), n * 4);
    if (emit) memcpy(emit, L.emit.data(), n * 4);
    if (temps) memcpy(temps, L.ta.data(), n * 4);
    if (f) { const auto& c = L.cur(); for (size_t i = 0; i < 19 * n; i++) f[i] = (float)c[i]; }
    if (forces) memcpy(forces, L.forces, sizeof(L.forces));
    if (forces64) memcpy(forces64, L.forces64, sizeof(L.forces64));
    if (reset_forces) { memset(L.forces, 0, sizeof(L.forces)); memset(L.forces64, 0, sizeof(L.forces64)); }
  });
}
// Double-precision copies for the FP64 model (fields 4n, populations 19n).
void wto_read64(void* h, double* fields, double* f) {
  with(h, [&](auto& L) {
    size_t n = L.n;
    if (fields) for (size_t i = 0; i < 4 * n; i++) fields[i] = (double)L.fields[i];
    if (f) { const auto& c = L.cur(); for (size_t i = 0; i < 19 * n; i++) f[i] = (double)c[i]; }
  });
}
// Overwrite the current populations / fields / temps (for injected states).
void wto_write_state(void* h, const float* f, const float* fields, const float* temps) {
  with(h, [&](auto& L) {
    size_t n = L.n;
    auto& c = L.cur_a ? L.fa : L.fb;
    if (f) for (size_t i = 0; i < 19 * n; i++) c[i] = f[i];
    if (fields) for (size_t i = 0; i < 4 * n; i++) L.fields[i] = fields[i];
    if (temps) memcpy(L.ta.data(), temps, n * 4);
  });
}
// Per-cell link words: bits 1..18 bounce-back links, bit 19 belt contact (floorU = 0).
void wto_link_mask(void* h, uint32_t* out) {
  with(h, [&](auto& L) {
    for (int z = 0; z < L.nz; z++)
      for (int y = 0; y < L.ny; y++)
        for (int x = 0; x < L.nx; x++) {
          size_t idx = (size_t)x + (size_t)L.nx * ((size_t)y + (size_t)L.ny * z);
          uint32_t m = L.link_mask(x, y, z);
          if (!L.solid[idx] && L.belt_contact(x, y, z)) m |= 1u << 19;
          out[idx] = m;
        }
  });
}
uint64_t wto_guarded(void* h) {
  uint64_t g = 0;
  with(h, [&](auto& L) { g = L.guarded; });
  return g;
}
// The project's math functions (wt_fmath.h) on an array, for accuracy tests:
// which 0 sin, 1 cos, 2 atan, 3 exp, 4 exp2, 5 log2.
void wto_fmath(int which, const float* x, float* y, int n) {
  for (int i = 0; i < n; i++) {
    const float v = x[i];
    y[i] = which == 0 ? wtm::sinf(v) : which == 1 ? wtm::cosf(v) : which == 2 ? wtm::atanf(v)
         : which == 3 ? wtm::expf(v) : which == 4 ? wtm::exp2f(v) : wtm::log2f(v);
  }
}
// Two-argument functions: which 0 pow(x, y), 1 atan2(x, y) (x = the ordinate).
void wto_fmath2(int which, const float* x, const float* y, float* out, int n) {
  for (int i = 0; i < n; i++) out[i] = which == 0 ? wtm::powf(x[i], y[i]) : wtm::atan2f(x[i], y[i]);
}
int wto_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void wto_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

}  // extern "C"
