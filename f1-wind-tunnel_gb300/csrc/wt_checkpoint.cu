// Checkpoint and resume of one lattice: wt_save writes the whole simulation
// state of a context to a file, wt_load puts it back into a context of the same
// size and storage format, after which the run continues bit for bit as if it
// had never stopped.  The reference keeps its state only in GPU buffers
// (src/engine/engine.ts:234-260) and has no counterpart; long FP32 reference
// runs and warm-start data reuse it.
//
// File layout (little-endian, both build machines are):
//   header     "WTCKPT01", u32 version (1), u32 nx, ny, nz, storage,
//              u32 sizeof(wt_sim), sizeof(wt_shape), the two structs,
//              u64 steps_total, steps_since_read
//   pop        19 arrays of n cells in the storage format's own bits, in the
//              canonical AA state (pop[opp(j)][x] holds f*_j(x), the state after
//              every wt_step call), so f16 / bf16 round-trip exactly
//   solid      n u8 groups;  emit n f32;  temperatures n f32;
//   fields     n x 4 f32 (u, rho of the last step);  outlet ny * nz x 4 f32
//   readout    18 f64 accumulators (force sums, mass), 12 i32 fixed-point
//              sums, u32 guard count
//   checksum   u64 FNV-1a over every byte before it
// Not stored: the per-step force history (it restarts at the load), the block
// shape (a tuning choice of the loading context), the W17 model buffers (the
// voxel flags are stored; re-voxelizing a W17 shape after a load needs
// wt_set_car_model again).
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "wt_ctx.h"

using namespace wt;
using namespace wt::api;

namespace {

constexpr char kMagic[8] = {'W', 'T', 'C', 'K', 'P', 'T', '0', '1'};
constexpr uint32_t kVersion = 1;

struct Fnv {
  uint64_t h = 1469598103934665603ull;
  void add(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
  }
};

struct Writer {
  FILE* f;
  Fnv sum;
  bool ok = true;
  void put(const void* p, size_t n) {
    if (ok && n && fwrite(p, 1, n, f) != n) ok = false;
    sum.add(p, n);
  }
  template <class T> void val(const T& v) { put(&v, sizeof(v)); }
};

struct Reader {
  FILE* f;
  Fnv sum;
  bool ok = true;
  void get(void* p, size_t n) {
    if (ok && n && fread(p, 1, n, f) != n) ok = false;
    if (ok) sum.add(p, n);
  }
  template <class T> T val() {
    T v{};
    get(&v, sizeof(v));
    return v;
  }
};

// device -> file (or file -> device) through one host buffer per section
int save_dev(wt_ctx* c, Writer& w, const void* dev, size_t bytes, std::vector<unsigned char>& buf) {
  buf.resize(bytes);
  WT_CUDA(c, cudaMemcpyAsync(buf.data(), dev, bytes, cudaMemcpyDeviceToHost, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  w.put(buf.data(), bytes);
  return WT_OK;
}

int load_dev(wt_ctx* c, Reader& r, void* dev, size_t bytes, std::vector<unsigned char>& buf) {
  buf.resize(bytes);
  r.get(buf.data(), bytes);
  if (!r.ok) return WT_OK;  // the caller reports the short file
  WT_CUDA(c, cudaMemcpyAsync(dev, buf.data(), bytes, cudaMemcpyHostToDevice, c->stream));
  WT_CUDA(c, cudaStreamSynchronize(c->stream));  // buf is reused by the next section
  return WT_OK;
}

}  // namespace

extern "C" {

int wt_save(wt_ctx* c, const char* path) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!path) return fail(c, WT_ERR_ARG, "wt_save: null path");
  if ((rc = flush_forces(c))) return rc;  // pending force records into the accumulators
  WT_CUDA(c, cudaStreamSynchronize(c->stream));
  FILE* f = fopen(path, "wb");
  if (!f) return fail(c, WT_ERR_IO, std::string("wt_save: cannot open ") + path + " for writing");
  Writer w{f};
  std::vector<unsigned char> buf;
  w.put(kMagic, 8);
  w.val(kVersion);
  w.val(c->nx);
  w.val(c->ny);
  w.val(c->nz);
  w.val(c->sim.storage);
  w.val((uint32_t)sizeof(wt_sim));
  w.val((uint32_t)sizeof(wt_shape));
  w.val(c->sim);
  w.val(c->shape);
  w.val(c->steps_total);
  w.val(c->steps_since_read);
  const size_t n = c->n;
  for (int i = 0; i < 19 && rc == WT_OK; i++)
    rc = save_dev(c, w, static_cast<const char*>(c->pop) + (size_t)i * c->np * c->elem, n * c->elem, buf);
  if (rc == WT_OK) rc = save_dev(c, w, c->solid, n, buf);
  if (rc == WT_OK) rc = save_dev(c, w, c->emit, n * 4, buf);
  if (rc == WT_OK) rc = save_dev(c, w, c->tA, n * 4, buf);
  if (rc == WT_OK) rc = save_dev(c, w, c->fields, n * 16, buf);
  if (rc == WT_OK) rc = save_dev(c, w, c->outlet_u, (size_t)c->ny * c->nz * 16, buf);
  if (rc == WT_OK) rc = save_dev(c, w, c->totals, 18 * 8, buf);
  if (rc == WT_OK) rc = save_dev(c, w, c->raw_totals, 12 * 4, buf);
  if (rc == WT_OK) rc = save_dev(c, w, c->counters, 4, buf);
  const uint64_t sum = w.sum.h;
  if (rc == WT_OK) w.put(&sum, 8);
  const bool closed = fclose(f) == 0;
  if (rc != WT_OK) return rc;
  if (!w.ok || !closed) return fail(c, WT_ERR_IO, std::string("wt_save: write to ") + path + " failed");
  return WT_OK;
}

int wt_load(wt_ctx* c, const char* path) {
  int rc = check_ctx(c);
  if (rc) return rc;
  if (!path) return fail(c, WT_ERR_ARG, "wt_load: null path");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(c, WT_ERR_IO, std::string("wt_load: cannot open ") + path);
  Reader r{f};
  char magic[8] = {0};
  r.get(magic, 8);
  const uint32_t version = r.val<uint32_t>();
  const uint32_t nx = r.val<uint32_t>(), ny = r.val<uint32_t>(), nz = r.val<uint32_t>();
  const uint32_t storage = r.val<uint32_t>();
  const uint32_t sim_bytes = r.val<uint32_t>(), shape_bytes = r.val<uint32_t>();
  auto bad = [&](int code, const std::string& m) {
    fclose(f);
    return fail(c, code, "wt_load: " + std::string(path) + ": " + m);
  };
  if (!r.ok || memcmp(magic, kMagic, 8) != 0) return bad(WT_ERR_IO, "not a libwt checkpoint");
  if (version != kVersion || sim_bytes != sizeof(wt_sim) || shape_bytes != sizeof(wt_shape))
    return bad(WT_ERR_IO, "checkpoint version " + std::to_string(version) + " is not readable by this build");
  if (nx != c->nx || ny != c->ny || nz != c->nz)
    return bad(WT_ERR_ARG, "lattice " + std::to_string(nx) + "x" + std::to_string(ny) + "x" + std::to_string(nz) +
                               " does not match the context's " + std::to_string(c->nx) + "x" + std::to_string(c->ny) +
                               "x" + std::to_string(c->nz));
  if (storage != c->sim.storage) return bad(WT_ERR_ARG, "storage format differs from the context's");
  const wt_sim sim = r.val<wt_sim>();
  const wt_shape shape = r.val<wt_shape>();
  const uint64_t steps_total = r.val<uint64_t>(), since = r.val<uint64_t>();
  if (!r.ok) return bad(WT_ERR_IO, "file ends inside the header");
  if (!valid_tau(sim, c->nx)) return bad(WT_ERR_IO, "stored relaxation times are not valid");
  // Sections go straight to the device; the context is left in a defined state
  // (its old one, overwritten in part) if the file turns out short or damaged.
  if ((rc = flush_forces(c))) { fclose(f); return rc; }
  std::vector<unsigned char> buf;
  const size_t n = c->n;
  for (int i = 0; i < 19 && rc == WT_OK; i++)
    rc = load_dev(c, r, static_cast<char*>(c->pop) + (size_t)i * c->np * c->elem, n * c->elem, buf);
  if (rc == WT_OK) rc = load_dev(c, r, c->solid, n, buf);
  if (rc == WT_OK) rc = load_dev(c, r, c->emit, n * 4, buf);
  if (rc == WT_OK) rc = load_dev(c, r, c->tA, n * 4, buf);
  if (rc == WT_OK) rc = load_dev(c, r, c->fields, n * 16, buf);
  if (rc == WT_OK) rc = load_dev(c, r, c->outlet_u, (size_t)c->ny * c->nz * 16, buf);
  if (rc == WT_OK) rc = load_dev(c, r, c->totals, 18 * 8, buf);
  if (rc == WT_OK) rc = load_dev(c, r, c->raw_totals, 12 * 4, buf);
  if (rc == WT_OK) rc = load_dev(c, r, c->counters, 4, buf);
  if (rc != WT_OK) { fclose(f); return rc; }
  const uint64_t expect = r.sum.h;
  uint64_t stored = 0;
  Reader tail{f};
  tail.get(&stored, 8);
  char extra;
  const bool at_end = fread(&extra, 1, 1, f) == 0;
  fclose(f);
  if (!r.ok || !tail.ok) return fail(c, WT_ERR_IO, "wt_load: " + std::string(path) + ": file is truncated");
  if (stored != expect || !at_end)
    return fail(c, WT_ERR_IO, "wt_load: " + std::string(path) + ": checksum mismatch (damaged checkpoint)");
  // parameters, flags and the host-side counters of the stored run
  c->sim = sim;
  if ((rc = apply_sim(c))) return rc;
  c->shape = shape;
  c->steps_total = steps_total;
  c->steps_since_read = since;
  c->steps_recorded = 0;  // the force history restarts here
  c->pending = 0;
  c->mass_pending = false;
  WT_CUDA(c, cudaMemsetAsync(c->hist_pos, 0, 8, c->stream));
  WT_CUDA(c, cudaMemsetAsync(c->counters + 1, 0, 4, c->stream));  // reduction counter: idle
  WT_CUDA(c, cudaMemcpyAsync(c->tB, c->tA, n * 4, cudaMemcpyDeviceToDevice, c->stream));
  return rebuild_links(c);  // cell words, heat sources, force blocks from the loaded flags
}

}  // extern "C"
