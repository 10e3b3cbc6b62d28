/*
 * libwt - GB300 (sm_103a) wind-tunnel simulation core, C ABI.
 *
 * Drop-in for the simulation half of the reference engine class
 * `AeroEngine` (src/engine/engine.ts:159-769).  A TypeScript host binds these
 * entry points through N-API/FFI in place of its WGSL dispatches; every other
 * caller (Python ctypes, C, C++) uses them the same way.
 *
 * Conventions (all entry points):
 *   - return 0 (WT_OK) on success, a negative WT_ERR_* code on failure;
 *     wt_last_error(ctx) gives a one-line message for the last failure;
 *   - the library owns all device memory of a context; callers pass plain
 *     host structs and host buffers of the documented sizes;
 *   - one context = one CUDA stream on the current device; calls on one context
 *     must be serialised by the caller, different contexts are independent;
 *   - there is no CPU fallback: without a usable sm_103a device wt_create fails.
 *
 * Lattice layout and conventions follow the reference shaders
 * (src/engine/wgsl.ts:123-139): D3Q19 velocity order
 *   0 rest; 1,2 +-x; 3,4 +-y; 5,6 +-z; 7..10 xy diagonals (1,1),(-1,-1),(1,-1),(-1,1);
 *   11..14 xz; 15..18 yz;
 * cell index idx = x + nx*(y + ny*z); x streamwise, y up (moving floor at y=0),
 * z lateral with the symmetry plane at z=0 (half tunnel, z >= 0).
 */
#ifndef WT_H
#define WT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WT_OK 0
#define WT_ERR_ARG (-1)         /* invalid argument or size */
#define WT_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define WT_ERR_NOMEM (-3)       /* device allocation failed */
#define WT_ERR_UNSUPPORTED (-4) /* scene kind or option not built */
#define WT_ERR_STATE (-5)       /* call not valid in the current state */
#define WT_ERR_DEVICE (-6)      /* no sm_103a device / wrong architecture */
#define WT_ERR_IO (-8)          /* checkpoint file not writable / readable, damaged or of another build */

/* Population storage format (see wt_sim.storage). */
#define WT_STORE_F32 0u  /* f_i as float: 19*4 B per cell */
#define WT_STORE_F16 1u  /* f_i - w_i as IEEE half: 19*2 B per cell */
#define WT_STORE_BF16 2u /* f_i - w_i as bfloat16: 19*2 B per cell */

/* Scene kinds, Shape.kind of src/engine/engine.ts:30 plus one build extension. */
#define WT_KIND_F1 0u     /* analytic generic F1, src/engine/f1.ts:283-320 */
#define WT_KIND_SPHERE 1u /* wgsl.ts:104 */
#define WT_KIND_CUBE 2u   /* wgsl.ts:105, 1 m rounded cube at (2.6, 1.0, 0) */
#define WT_KIND_WING 3u   /* wgsl.ts:106 */
#define WT_KIND_W17 5u    /* baked W17 model, src/engine/f1.ts:322-381; needs wt_set_car_model */
#define WT_KIND_EMPTY 6u  /* wgsl.ts:108 */
#define WT_KIND_BOX 7u    /* build extension: axis-aligned box box_center +- box_half */

/* Grid of one lattice: AeroEngine constructor fields dims/h/origin (engine.ts:226-231). */
typedef struct wt_grid {
  uint32_t nx, ny, nz; /* cells; nx >= 8, ny >= 2, nz >= 2 */
  float origin[3];     /* world position of the corner of cell (0,0,0), metres */
  float h;             /* cell size, metres */
} wt_grid;

/* Simulation parameters: the Sim uniform (wgsl.ts:158, engine.ts:249) plus the
 * constants the reference hard-codes in its collision and heat shaders. */
typedef struct wt_sim {
  float u_in;          /* inlet speed, lattice units (engine.ts:110: 0.0925) */
  float tau0;          /* base relaxation time (engine.ts:249: 0.508) */
  float smag;          /* Smagorinsky constant Cs (engine.ts:249: 0.17) */
  float sponge_cells;  /* outlet sponge ramp smoothstep(nx-cells, nx-1, x) (wgsl.ts:260: 18) */
  float sponge_amp;    /* tau added at the outlet (0.4) */
  float inlet_cells;   /* inlet ramp smoothstep(0, cells, x) (10) */
  float inlet_amp;     /* tau added at the inlet (0.25) */
  float heat_cool;     /* heat uniform cool (engine.ts:263: 0.004) */
  float heat_diffuse;  /* heat uniform diffuse (0.04) */
  float heat_src_mix;  /* source blend (wgsl.ts:508: 0.35) */
  uint32_t storage;    /* WT_STORE_* (fixed at wt_create) */
  uint32_t reserved;   /* must be 0 */
} wt_sim;

/* Scene description: the Shape uniform (wgsl.ts:9-18) word for word, angles in
 * radians as engine.ts:429-448 packs them, followed by the box extension. */
typedef struct wt_shape {
  uint32_t kind, profile_mode, pw, ph;
  float front_flap, rear_main, rear_flap, ride_h;
  float aoa, width, axis_y, p_scale;
  float p_origin[2], heat_brakes, heat_engine;
  float heat_rad, front_wing, rear_wing, sidepod;
  float cover, nose, rear_ride, duct;
  float box_center[3], box_half[3]; /* WT_KIND_BOX only */
} wt_shape;

/* Force readout (engine.ts:739-761 maybeReadForces).  Groups g: 0 body, 1 front
 * wing, 2 rear wing (solid flag values 1, 2, 3). */
typedef struct wt_forces {
  int32_t raw[12];     /* the reference's i32 accumulator, bit-compatible: raw[3g+0] = x,
                          raw[3g+1] = y of round(1e4 * per-cell force), summed with wrap */
  double sum[9];       /* the same per-cell forces summed in FP64 on the device:
                          sum[3g+c], c = x, y, z (lattice units, momentum per step) */
  double mass;         /* FP64 sum of rho over fluid cells after the last step */
  uint64_t steps;      /* LBM steps accumulated since the last reset of the readout */
  uint64_t guarded;    /* cells reset by the divergence guard since that reset */
} wt_forces;

/* Sizes and state of a context. */
typedef struct wt_info {
  uint64_t cells;          /* nx*ny*nz */
  uint64_t device_bytes;   /* device memory held by the context */
  uint64_t steps_total;    /* LBM steps since wt_reset */
  uint32_t storage;        /* WT_STORE_* */
  uint32_t fluid_cells;    /* after the last voxelization */
  uint32_t solid_cells[3]; /* per group */
  uint32_t boundary_blocks;/* step-kernel blocks that carry bounce-back links */
  uint32_t history_capacity; /* per-step force records kept (ring) */
  uint32_t sm_count;
} wt_info;

typedef struct wt_ctx wt_ctx;

/* new AeroEngine(...) (engine.ts:226-345): allocate one lattice on the current device.
 * The lattice starts in the reset state with an empty scene. */
int wt_create(const wt_grid* grid, const wt_sim* sim, wt_ctx** out);

/* Release everything the context holds.  Safe on NULL. */
int wt_destroy(wt_ctx* ctx);

/* syncSim (engine.ts:497-501): update the simulation parameters between steps.
 * sim->storage must equal the value given to wt_create. */
int wt_set_sim(wt_ctx* ctx, const wt_sim* sim);

/* reset() (engine.ts:371-381, LBM_INIT wgsl.ts:147-155): populations to
 * feq(1, (u_in,0,0)), fields to (u_in,0,0,1), temperatures to 0.  Keeps the scene. */
int wt_reset(wt_ctx* ctx);

/* Rig uniform of the baked W17 model (src/engine/car-model.ts:60-69): the
 * articulated wing elements' hinges, angles, extras and part grids. */
typedef struct wt_rig {
  float front[71][4];  /* front flap hinges along |z| in 1 cm bins: flap A xy, flap B zw */
  float hinges[4];     /* rear main plane xy, rear flap zw */
  float angles[4];     /* front flap A, front flap B, rear flap, rear main plane (rad) */
  float extra[4];      /* rear tip twist (rad), flap chord scale, sidepod squeeze, unused */
  float fly[4];        /* fly-away progress front / rear, fitted front / rear (1 or 0) */
  float grids[12][4];  /* per part (6): origin xyz + cell size, dims xyz + atlas z offset */
} wt_rig;

/* setCarModel (engine.ts:410-421) plus the rig of setShape (engine.ts:450-462):
 * the W17 model that scene kind WT_KIND_W17 voxelizes and renders.  body_sdf:
 * 368 x 84 x 67 binary16 distances at 1.5 cm from (-0.3, 0, 0), x fastest;
 * parts: the atlas of per-part grids (partsAtlas, car-model.ts:176-193),
 * parts_dims[0] x [1] x [2] binary16, x fastest.  Copied to the device; a later
 * call replaces the model (call it again with a new rig when the wing settings
 * change).  Sampling is trilinear with clamp-to-edge, in f32. */
int wt_set_car_model(wt_ctx* ctx, const uint16_t* body_sdf, const uint16_t* parts, const uint32_t parts_dims[3],
                     const wt_rig* rig);

/* setShape() (engine.ts:426-470, VOXELIZE wgsl.ts:305-321): voxelize the scene
 * into solid flags, heat emission and bounce-back link masks.  Populations are
 * kept (re-voxelize semantics, engine.ts:469). */
int wt_voxelize(wt_ctx* ctx, const wt_shape* shape);

/* Load externally computed flags instead of a scene: solid[n] in {0,1,2,3} and
 * emit[n] (heat source in solid cells, negative marks a duct cell). */
int wt_set_solid(wt_ctx* ctx, const uint32_t* solid, const float* emit);

/* The compute pass of frame() (engine.ts:708-712): n_lbm_steps collide-stream
 * steps (must be even and >= 2, as engine.ts:585 makes them), then heat_passes
 * semi-Lagrangian heat passes (0 or an even number; engine.ts:711-712 issues 2)
 * with backtrace time heat_dt (engine.ts:659-660 uses n_lbm_steps/2; pass <= 0
 * for that default).  Asynchronous on the context stream. */
int wt_step(wt_ctx* ctx, int n_lbm_steps, int heat_passes, float heat_dt);

/* maybeReadForces (engine.ts:739-761): copy the force accumulators to *out and,
 * if reset != 0, zero them (engine.ts:747).  Synchronises the context stream. */
int wt_read_forces(wt_ctx* ctx, wt_forces* out, int reset);

/* maybeReadForces without waiting, as the reference maps its readback buffer
 * asynchronously (engine.ts:746-760): queue the pending force reduction, a copy
 * of the accumulators into one of the context's 16 pinned landing slots and, if
 * reset != 0, their zeroing; return at once with *ticket.  wt_forces_collect
 * waits for that copy and fills *out (the same fields as wt_read_forces).  A
 * ticket can be collected until 16 newer readbacks have been queued. */
int wt_read_forces_async(wt_ctx* ctx, int reset, uint64_t* ticket);
int wt_forces_collect(wt_ctx* ctx, uint64_t ticket, wt_forces* out);

/* Per-step FP64 force records of the last `count` steps, oldest first:
 * out[9*k + 3g + c].  count <= min(steps recorded, history_capacity). */
int wt_read_force_history(wt_ctx* ctx, double* out, uint32_t count);

/* debugRead() (engine.ts:763-768): any pointer may be NULL.
 *   u_rho[4n]  (ux, uy, uz, rho) after the last step (0 in solid cells)
 *   solid[n]   0 fluid, 1 body, 2 front wing, 3 rear wing
 *   temps[n]   heat scalar after the last heat pass
 *   emit[n]    heat source field from the voxelizer
 *   links[n]   bit i (1..18) set when direction i of a fluid cell bounces back
 *              off a solid neighbour (the branch wgsl.ts:221 takes), bit 19 set
 *              for floor cells under a belt contact patch (wgsl.ts:192-197). */
int wt_read_fields(wt_ctx* ctx, float* u_rho, uint32_t* solid, float* temps, float* emit, uint32_t* links);

/* Post-collision populations in the reference's buffer order f[i*n + idx]
 * (what fA holds after an even number of steps), converted to float. */
int wt_read_populations(wt_ctx* ctx, float* f);

/* Replace the state: populations f[19n] (post-collision, reference order),
 * optional u_rho[4n] (fields, also the outlet's previous velocity) and temps[n]. */
int wt_write_state(wt_ctx* ctx, const float* f, const float* u_rho, const float* temps);

/* Checkpoint and resume (no reference counterpart: the reference keeps its state
 * only in GPU buffers, src/engine/engine.ts:234-260).  wt_save writes the whole
 * simulation state to `path`: populations in the storage format's own bits,
 * solid flags, emission, temperatures, fields, the outlet column's velocities,
 * the force readout accumulators, the step counters, the simulation parameters
 * and the voxelized shape, with a checksum.  wt_load restores it into a context
 * of the same lattice size and storage format (WT_ERR_ARG otherwise); the run
 * then continues bit for bit as if it had not stopped.  Not stored: the
 * per-step force history (wt_read_force_history sees only steps after the load),
 * the block shape, and the W17 model (voxel flags are stored; re-voxelizing a W17
 * shape after a load needs wt_set_car_model).  Damaged, truncated or foreign
 * files give WT_ERR_IO; a failed load may leave the context partly overwritten. */
int wt_save(wt_ctx* ctx, const char* path);
int wt_load(wt_ctx* ctx, const char* path);

/* Warm start: set populations to feq(rho, u) of a coarse (ux,uy,uz,rho) field
 * u_rho[4*cx*cy*cz] trilinearly resampled to the lattice; fields likewise. */
int wt_reset_from(wt_ctx* ctx, const float* u_rho, uint32_t cx, uint32_t cy, uint32_t cz);

/* Box average of the fluid cells' (ux, uy, uz, rho) of the last wt_step call's
 * fields onto a cx x cy x cz grid (fine cell i of an axis falls in coarse cell
 * i * c / n; boxes without fluid give (0, 0, 0, 1)); u_rho receives
 * cx*cy*cz*4 floats, x fastest.  The training target of the warm start and the
 * inverse direction of wt_reset_from. */
int wt_read_coarse(wt_ctx* ctx, uint32_t cx, uint32_t cy, uint32_t cz, float* u_rho);

/* Scene distance (the first component of the reference's sceneSdf,
 * src/engine/wgsl.ts:101-116 / f1.ts:283-320) at the cell centres
 * origin + (i + 0.5) h of `grid`; out receives nx*ny*nz floats.  Needs no
 * context (uses the current device); the warm start's geometry input. */
int wt_sdf_sample(const wt_shape* shape, const wt_grid* grid, float* out);

/* ---- host-side averaging and the aero-map sweep (src/main.ts:586-596,
 * src/ui/aeromap.ts:73-114), so a host UI only displays results. */

/* Running body coefficients (main.ts:590-596): the first reading sets them, then
 * an exponential average with rate 0.15 for readings 1-19, 0.04 for 20-59 and
 * 0.011 from then on (about 12 s of readings). */
typedef struct wt_coef_ema {
  double cd, cl; /* drag and downforce over dynamic pressure, m^2 */
  uint32_t n;
} wt_coef_ema;
void wt_coef_ema_update(wt_coef_ema* e, double drag_n, double down_n, double q);

/* Aero-map sweep on one lattice, as the reference runs it: the ride-height
 * points in serpentine order (front index i, rear index j reversed on odd i),
 * each re-voxelized into the running flow (populations kept), settled for
 * settle_steps, then measured over measure_steps with a force reading every
 * read_every steps (scaled to newtons as maybeReadForces does, engine.ts:750-759,
 * at `kmh`); cells get the mean downforce (kg), drag (N), efficiency
 * down / max(drag, 1) and the per-group means.  Steps are rounded up to even. */
typedef struct wt_sweep {
  uint32_t n_front, n_rear;
  const float* front; /* front ride heights, m (n_front) */
  const float* rear;  /* rear ride heights, m (n_rear) */
  uint32_t settle_steps, measure_steps, read_every;
  float kmh;
} wt_sweep;
typedef struct wt_sweep_cell {
  double down_kg, drag_n, efficiency;
  double group_down_n[3], group_drag_n[3]; /* body, front wing, rear wing */
  uint32_t order, readings;                /* position in the sweep; force readings averaged */
} wt_sweep_cell;
/* out: n_front * n_rear cells, [front][rear].  base: the shape whose ride_h and
 * rear_ride each point replaces. */
int wt_aeromap_sweep(wt_ctx* ctx, const wt_shape* base, const wt_sweep* s, wt_sweep_cell* out);

/* ---- field consumers: the reference's sampling, particle and streamline passes
 * as kernels into headless buffers.  They read the (u, rho) fields of the last
 * wt_step call and the temperatures; results are bit-identical to the
 * reference's shaders. */

/* View uniform (src/engine/wgsl.ts:431-434): colour scaling of fieldValue. */
typedef struct wt_view {
  float u_in, v_real, cp_min, cp_max, t_min, t_max, speed_max, vort_max;
} wt_view;

/* PSim uniform (wgsl.ts:517-521), as plain C fields. */
typedef struct wt_psim {
  uint32_t count, spawn_mode, color_mode, frame; /* spawn_mode 1 = rake; color_mode as fieldValue */
  float dt, life;
  uint32_t scatter, rake_rows, rake_cols, reserved;
  float spawn_min[3], spawn_max[3];
} wt_psim;

/* Stream uniform and emitters (src/engine/render-wgsl.ts:521-527). */
typedef struct wt_stream_params {
  uint32_t lines, steps, seed_mode, color_mode; /* seed_mode 1 = ring emitters */
  uint32_t rows, cols, per_emitter, emitters;
  float seed_min[3], seed_max[3];
  float step_len, time;
  float emitter[8][4]; /* centre x, y, z and radius */
} wt_stream_params;

/* sampleFlow (wgsl.ts:332-357) at n world points (pts: n*3 floats, host):
 * out receives n*6 floats (ux, uy, uz, rho, temperature, fluid weight); vort
 * (may be NULL) n floats of vorticityAt (wgsl.ts:359-366). */
int wt_sample_flow(wt_ctx* ctx, const float* pts, uint32_t n, float* out, float* vort);

/* One particle pass (PARTICLES_SIM cs_main, wgsl.ts:566-594): RK2 advection,
 * respawn and colour value of p->count particles.  parts: count*8 floats
 * (pos x, y, z, age, step x, y, z, colour), updated in place; host memory, or
 * device memory when parts_on_device != 0. */
int wt_particles_step(wt_ctx* ctx, float* parts, int parts_on_device, const wt_psim* p, const wt_view* v);

/* The streamline pass (STREAM_SIM cs_main, render-wgsl.ts:551-575): lines x
 * steps points (x, y, z, colour; colour -1 once a line has ended) into pts
 * (host, lines*steps*4 floats). */
int wt_streamlines(wt_ctx* ctx, const wt_stream_params* s, const wt_view* v, float* pts);

/* ---- render passes: the reference's frame graph into headless render targets
 * (src/engine/render-wgsl.ts; targets engine.ts:290-306, passes engine.ts:714-725).
 * The uniform structs below have the layouts of the WGSL uniforms they replace.
 * A renderer reads the fields and temperatures of its context's last step call
 * and the shape of its last wt_voxelize; its passes are queued on the
 * context's stream and return at once.  With look.mesh_mode != 0 the scene
 * pass takes the car's surfaces from the renderer's G-buffer (the targets
 * WT_TARGET_G*, written by wt_render_mesh or wt_render_write). */

/* Cam uniform (render-wgsl.ts:5-11). */
typedef struct wt_cam {
  float pos[3], tan_half;
  float fwd[3], aspect;
  float right[3], time;
  float up[3], road_speed;
  float jitter[2], pad0, pad1;
} wt_cam;

/* Look uniform (render-wgsl.ts:12-19); palette as fieldValue's colour field. */
typedef struct wt_look {
  float bmin[3]; uint32_t surf_mode;
  float bmax[3]; uint32_t palette;
  float paint[3]; uint32_t carbon_body;
  float accent[3]; uint32_t is_f1;
  uint32_t slice_axis; float slice_pos, slice_alpha; uint32_t show_flow;
  uint32_t mesh_mode, cooling, pad1, pad2;
} wt_look;

/* Taa uniform (render-wgsl.ts:457-463); matrices column-major. */
typedef struct wt_taa {
  float prev_view_proj[16];
  float cam_pos[3], tan_half;
  float fwd[3], aspect;
  float right[3], blend;
  float up[3], pad;
} wt_taa;

/* PDraw uniform (src/engine/wgsl.ts:598-603). */
typedef struct wt_pdraw {
  float view_proj[16];
  float cam_pos[3], width;
  float res[2], trail, alpha;
  uint32_t count, palette; float fade_in, pad;
} wt_pdraw;

/* SDraw uniform (render-wgsl.ts:579-584). */
typedef struct wt_sdraw {
  float view_proj[16];
  float cam_pos[3], width;
  float res[2], time, intensity;
  uint32_t lines, steps, palette; float pulse;
} wt_sdraw;

/* Post uniform (render-wgsl.ts:421). */
typedef struct wt_post {
  float bloom, exposure, pad0, pad1;
} wt_post;

/* Render targets, for wt_render_read / wt_render_write.  Float targets hold
 * RGBA binary16 (4 uint16 per texel); WT_TARGET_OUTPUT holds RGBA8. */
enum {
  WT_TARGET_SCENE = 0,   /* width x height, RENDER output (alpha: hit distance) */
  WT_TARGET_HIST0 = 1,   /* width x height, TAA history 0 */
  WT_TARGET_HIST1 = 2,   /* width x height, TAA history 1 */
  WT_TARGET_GLOW = 3,    /* width x height, particles and streamlines */
  WT_TARGET_BLOOM_A = 4, /* half size, horizontal blur */
  WT_TARGET_BLOOM_B = 5, /* half size, vertical blur */
  WT_TARGET_OUTPUT = 6,  /* width x height, presented RGBA8 */
  /* the car G-buffer (engine.ts:297-303), width x height; cleared to 0 at creation */
  WT_TARGET_GALBEDO = 7,  /* binary16: albedo rgb, roughness (or decal alpha) */
  WT_TARGET_GNORMAL = 8,  /* binary16: normal xyz, distance to the camera (0 = no car) */
  WT_TARGET_GMATERIAL = 9 /* RGBA8 unorm: metal, coat, emissive, 1 */
};

typedef struct wt_renderer wt_renderer;

/* Targets of one view: width x height (half-size bloom targets, at least 1x1). */
int wt_render_create(wt_ctx* ctx, uint32_t width, uint32_t height, wt_renderer** out);
void wt_render_destroy(wt_renderer* r);
/* RENDER pass (render-wgsl.ts:288-398) into WT_TARGET_SCENE; look->mesh_mode
 * selects the G-buffer composite (render-wgsl.ts:300-323), look->cooling the
 * louvres painted on the mesh (0 closed, 1 partly, 2 fully open). */
int wt_render_scene(wt_renderer* r, const wt_cam* cam, const wt_look* look, const wt_view* view);
/* TAA resolve (render-wgsl.ts:456-518): scene and history 1-cur into history cur. */
int wt_render_taa(wt_renderer* r, const wt_taa* taa, int cur);
/* Glow pass (engine.ts:719-722): clear, then the particle quads (parts: pd->count
 * particles of 8 floats, drawn twice, mirrored; NULL = no draw) and the
 * streamline quads (pts: sd->lines * sd->steps points of 4 floats, drawn
 * lines * 2 * (steps - 1) times; NULL = no draw).  Host memory, or device
 * memory when the matching *_on_device flag is set. */
int wt_render_glow(wt_renderer* r, const float* parts, int parts_on_device, const wt_pdraw* pd, const float* pts,
                   int pts_on_device, const wt_sdraw* sd);
/* Bloom (engine.ts:316-317): BLUR (1, 0) spacing 3 glow -> bloom A, then
 * (0, 1) spacing 1.5 bloom A -> bloom B, gain 1. */
int wt_render_bloom(wt_renderer* r);
/* PRESENT (render-wgsl.ts:442-454): history cur, glow and bloom B -> output. */
int wt_render_present(wt_renderer* r, const wt_post* post, int cur);
/* Copy a target to / from host memory (synchronous). */
int wt_render_read(wt_renderer* r, int target, void* host);
int wt_render_write(wt_renderer* r, int target, const void* host);

/* ---- the car mesh G-buffer pass: MESH_DRAW (render-wgsl.ts:647-760) over the
 * draws of MeshCar (mesh-car.ts:46-213), into the renderer's G-buffer
 * (engine.ts:297-303, 716).  The depth test, decal blending and texture
 * filtering rules are written out in wt_mesh.cu and wt_texfilter.h. */
typedef struct wt_mesh wt_mesh;

/* One draw (mesh-car.ts:134-175): the MeshMat uniform (render-wgsl.ts:653-657)
 * in its first 12 words, then the draw's index-list entries, texture and state. */
typedef struct wt_mesh_draw {
  float color[4];
  float metal, rough, coat, alpha_cut;
  float emissive, has_tex, is_body; uint32_t first_index;
  uint32_t count;    /* index-list entries drawn (count / 3 triangles) */
  int32_t texture;   /* wt_mesh_add_texture index; -1 = none (has_tex must be 0) */
  uint32_t blend;    /* decal (DECAL_BLEND): depth bias -4 / slope -1, 'less-equal', no
                        depth write, albedo blended, the other targets kept */
  uint32_t optional; /* drawn only when wt_render_mesh gets optional != 0 (the gurney) */
} wt_mesh_draw;

/* MeshCam uniform (render-wgsl.ts:648-652); view_proj column-major. */
typedef struct wt_mesh_cam {
  float view_proj[16];
  float cam_pos[3], ride_h;
  float jitter[2], rake, base_ride;
} wt_mesh_cam;

/* The vertex and index buffers of MeshCar.load (mesh-car.ts:63-95): verts n_verts
 * x 8 floats (x, y, z, u, nx, ny, nz, v in the car frame), indices n_indices
 * entries < n_verts, tags one byte per vertex (part in bits 0-2, assembly in
 * bits 3-7, car-model.ts:44-50).  Copied to the device. */
int wt_mesh_create(wt_ctx* ctx, const float* verts, uint32_t n_verts, const uint32_t* indices, uint32_t n_indices,
                   const uint8_t* tags, wt_mesh** out);
void wt_mesh_destroy(wt_mesh* m);
/* An rgba8unorm-srgb albedo texture, width x height RGBA8 texels from the top
 * row; its mip chain is made with halveRgba (mesh-car.ts:30-44).  *index
 * receives its number for wt_mesh_draw.texture. */
int wt_mesh_add_texture(wt_mesh* m, uint32_t width, uint32_t height, const uint8_t* rgba, int32_t* index);
/* Append a draw (record order = draw order; MeshCar sorts opaque before blended). */
int wt_mesh_add_draw(wt_mesh* m, const wt_mesh_draw* d);
/* The G-buffer pass (engine.ts:716): clear the G-buffer targets and the depth
 * buffer, then the mesh's draws in order (the optional ones when optional != 0)
 * with the camera and the Rig uniform (wt_set_car_model's rig).  Queued on the
 * context's stream; a frame with decals waits once for their fragment count. */
int wt_render_mesh(wt_renderer* r, wt_mesh* m, const wt_mesh_cam* cam, const wt_rig* rig, int optional);

/* Reverse the PNG scanline filters (None, Sub, Up, Average, Paeth) of an
 * inflated image: filtered holds rows x (1 + row_bytes) bytes (a filter-type
 * byte, then the row), bpp the bytes per pixel (1 for bit depths below 8).
 * out receives rows x row_bytes.  Host only; WT_ERR_ARG on an unknown filter.
 * For decoding the mesh's textures (the browser's image decoder in the
 * reference, main.ts:989-995). */
int wt_png_unfilter(const uint8_t* filtered, uint32_t rows, uint32_t row_bytes, uint32_t bpp, uint8_t* out);

int wt_info_get(wt_ctx* ctx, wt_info* out);

/* The context's cudaStream_t (as void*), for callers that time or order work. */
void* wt_stream(wt_ctx* ctx);

/* Block until all work queued on the context has finished. */
int wt_sync(wt_ctx* ctx);

/* Message of the last failure on ctx (or of the last failed wt_create if ctx is NULL). */
const char* wt_last_error(const wt_ctx* ctx);

/* Autotuner: time the collide-stream kernel under each candidate block shape
 * (cells along x by rows along y: 128x1, 64x2, 32x4, 256x1, 128x2, 64x4, 32x8)
 * and keep the fastest.  The simulation state is saved and restored, so the
 * lattice does not advance.  Outputs may be NULL. */
int wt_tune(wt_ctx* ctx, uint32_t* bx, uint32_t* by, float* ms_per_step);

/* ---- batches: many lattices advanced together (aero-map sweeps) -------------
 * No single reference function: the reference runs one lattice and sweeps the
 * aero map point by point (src/ui/aeromap.ts:73-114, re-voxelizing per point
 * through engine.ts:469).  A batch holds `count` lattices of any sizes with the
 * same simulation parameters; one kernel launch per LBM step covers every
 * lattice's blocks, and the launches of a wt_batch_step call are captured once
 * into a CUDA graph and replayed.  Each lattice is an ordinary wt_ctx
 * (wt_batch_lattice): voxelize, reset, read forces and fields with the single-
 * lattice calls; do not wt_destroy it. */
typedef struct wt_batch wt_batch;
int wt_batch_create(const wt_grid* grids, uint32_t count, const wt_sim* sim, wt_batch** out);
int wt_batch_destroy(wt_batch* batch);
uint32_t wt_batch_count(const wt_batch* batch);
wt_ctx* wt_batch_lattice(wt_batch* batch, uint32_t index);
/* n_lbm_steps / heat_passes / heat_dt as wt_step, for every lattice. */
int wt_batch_step(wt_batch* batch, int n_lbm_steps, int heat_passes, float heat_dt);
/* Autotuner over the block shapes for the whole batch, each timed with one
 * launch per LBM step and with the persistent launch (state saved and
 * restored).  The environment variable WT_BATCH_PERSIST=0/1, read at
 * wt_batch_create, fixes the launch kind instead. */
int wt_batch_tune(wt_batch* batch, uint32_t* bx, uint32_t* by, float* ms_per_step);
/* Grid of the batch's persistent launch (blocks resident at once), or 0 when the
 * batch launches its kernel once per LBM step.  In the persistent launch, one
 * cooperative kernel advances every lattice by up to 64 steps (the force-record
 * capacity), with a grid barrier between steps; the barrier's wait is bounded,
 * and an expired wait is reported as WT_ERR_CUDA by the next wt_batch_step. */
uint32_t wt_batch_persistent_grid(const wt_batch* batch);
void* wt_batch_stream(wt_batch* batch);
const char* wt_batch_last_error(const wt_batch* batch);

/* Library version, e.g. "libwt 0.1 sm_103a". */
const char* wt_version(void);

/* Forces of a population state without allocating any memory.  This entry
 * point has no counterpart in the reference.  It is for callers that cannot
 * call cudaMalloc: hosts that own every device buffer through their own
 * allocator or memory budget (or share the lattice through graphics interop
 * memory) and so cannot create a wt_ctx, and code that must not hit the device
 * synchronisation cudaMalloc can cause in the middle of a frame.
 *   f       device, 19*n floats: post-collision populations in the reference's
 *           order f[i*n + idx] (what wt_read_populations returns)
 *   solid   device, n u32 flags (0 fluid, 1..3 groups)
 *   emit    device, n floats (negative marks a duct cell whose links carry no
 *           force), or NULL
 *   fields  device, n x (ux, uy, uz, rho) floats of the previous step (what
 *           wt_read_fields returns); only the outlet column x = nx-1 is read,
 *           for its outflow equilibrium.  NULL takes (u_in, 0, 0) there.
 *   u_in    inlet speed (wt_sim.u_in): inlet and far-field equilibria, belt speed
 *   out     host; out->sum / out->raw get the force the next collide-stream step
 *           takes from this state, as wt_read_force_history / wt_read_forces
 *           report it: the same boundary precedence, and cells whose moments
 *           trip the divergence guard contribute nothing (their count is in
 *           out->guarded); out->steps = 1, out->mass = 0.
 * Scratch is a static device array of WT_NOALLOC_BLOCKS + 2 records
 * (98,496 B) that every GPU loading the library holds until exit.  The first
 * call on each device does that device's set-up: it looks up the array's
 * device address (with the device current) and keeps it for the process, which
 * assumes the device's primary context is not reset (cudaDeviceReset) between
 * calls.  Make that first call before any stream capture begins.  All calls
 * share the array and each keeps the previous call's contents except what it
 * clears: calls that overlap on the GPU race.  Every call synchronises `stream`
 * (a cudaStream_t, NULL = legacy default stream) before returning.  Lattices
 * above WT_NOALLOC_MAX_CELLS cells are rejected with WT_ERR_NOALLOC_LIMIT,
 * lattices below 8x3x3 with WT_ERR_ARG. */
#define WT_NOALLOC_BLOCKS 1024u
#define WT_NOALLOC_MAX_CELLS 134217728ull /* 2^27 */
#define WT_ERR_NOALLOC_LIMIT (-7)
int wt_forces_noalloc(const float* f, const uint32_t* solid, const float* emit, const float* fields, uint32_t nx,
                      uint32_t ny, uint32_t nz, float u_in, void* stream, wt_forces* out);

#ifdef __cplusplus
}
#endif

#endif /* WT_H */
