/*
 * si_cuda.h — C ABI of libsi_cuda, the GB300 (sm_103a) MLS-MPM substep behind ShaderIntel's MPM solver.
 *
 * The JavaScript `MPM` object (src/physics/mpm.js:82-680 of ShaderIntel v0.3.0) keeps its host logic
 * (option defaults, material validation, shape sampling, collider packing) and replaces its WebGPU
 * buffers and WGSL kernels with the calls below. Every entry point names the reference member it
 * replaces. Plain pointers and sizes only; all device memory belongs to the library.
 *
 * Units follow the reference: lattice units (dx = 1 cell), velocities in cells per substep.
 * Particle record = 32 floats (8 x vec4f, mpm.js:54-63):
 *   [0..3] x.xyz, material index (u32 bits)   [4..7]  v.xyz, J (fluid) / Jp (snow)
 *   [8..19] C columns c0,c1,c2 with tau00, tau11, tau22 in the .w lanes
 *   [20..31] F columns f0,f1,f2 with tau01, tau02, tau12 in the .w lanes
 * Grid node = 4 x i32 (fixed point 2^22: momentum xyz, mass) after P2G, re-read as vec4f(v, m)
 * after the grid update (mpm.js:428-470); node index x + X*(y + Y*z).
 *
 * Errors: every call returns SI_OK or a code; si_last_error() gives the message (thread-local).
 * Threading: every call takes its world's lock, so calls on one world from several threads (and a
 * server's rounds) are serialised. Work is ordered on the world's CUDA stream; reads synchronise it.
 */
#ifndef SI_CUDA_H
#define SI_CUDA_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes; the names mirror SIError codes (src/core/errors.js:1-11). */
#define SI_OK 0
#define SI_EINVAL 1      /* 'invalid-argument' */
#define SI_ENOMEM 2      /* device memory or the admission budget is exhausted */
#define SI_EDESTROYED 3  /* the object was destroyed (mpm.js:583 throws on step after destroy) */
#define SI_EDEVICE 4     /* CUDA error or no device ('no-device') */
#define SI_ETIMEOUT 5    /* a wait ran out */
#define SI_EBUSY 6       /* the world is driven by a server */

#define SI_MAX_MATERIALS 8   /* mpm.js:162 */
#define SI_MAX_COLLIDERS 16  /* mpm.js:280 */
#define SI_PARTICLE_FLOATS 32
#define SI_MATERIAL_FLOATS 12
#define SI_COLLIDER_FLOATS 12

typedef struct si_world si_world;   /* a CUDA stream + the scenes stepped together on it */
typedef struct si_mpm si_mpm;       /* one simulation (the reference's MPM object) */
typedef struct si_server si_server; /* continuous-batching request loop over one world */
typedef struct si_spatial si_spatial; /* a uniform-grid neighbour binning (SpatialGrid) */

/* Constructor options of `new MPM(ctx, o)`, mpm.js:89-109 (defaults by si_mpm_desc_default). */
typedef struct si_mpm_desc {
  int64_t max_particles; /* 262144 */
  int32_t grid;          /* cells along the longest axis, 64 */
  int32_t sort_every;    /* 4 */
  int32_t substeps;      /* 8 */
  int32_t ppc_axis;      /* 2 */
  double size[3];        /* world size, 1,1,1 */
  double origin[3];      /* 0,0,0 */
  double gravity[3];     /* m/s^2, 0,-9.81,0 */
  double time_scale;     /* 1 */
} si_mpm_desc;

/* Read-only properties of the MPM object (count, dims, dx, numNodes, substepDt, stepCount ...). */
typedef struct si_mpm_info {
  int64_t count, max_particles, step_count;
  int32_t dims[3];
  int32_t num_materials, num_colliders, sort_every, substeps, ppc_axis, bound;
  int64_t num_nodes;
  uint32_t num_blocks;
  double dx, substep_dt, time_scale;
  double origin[3], gravity[3];
  int64_t device_bytes; /* HBM held by this simulation */
} si_mpm_info;

const char* si_last_error(void);
const char* si_version(void);

/* ---------------------------------------------------------------- worlds */
/* A world owns one CUDA stream on the current device. si_world_step steps every scene of the
 * world together: one launch per phase covers all of them (the batched form). */
int si_world_create(si_world** out);
int si_world_destroy(si_world* w);                  /* destroys its scenes too; idempotent */
int si_world_step(si_world* w, int32_t K);          /* K substeps of every scene, each at its own dt */
int si_world_sync(si_world* w);
int si_world_set_graphs(si_world* w, int32_t enable); /* replay substeps from CUDA graphs (default 1) */
/* Snow and sand decompose F (svd3 of linalg.js:46-69: four Jacobi sweeps on F^T F) to a tolerance
 * instead of bit for bit: fused multiply-adds and the hardware reciprocal square root in place of
 * IEEE division and square root. Particle x, v, C, F and J stay within 1e-5 relative of the exact
 * path per substep from the same state; grid sums and binning remain exact integers of that state.
 * Default 0 (every field bit-identical to the CPU restatement of the reference). Worlds only; no
 * counterpart in the reference (its WGSL leaves the rounding of these operations open). */
int si_world_set_svd_tolerance(si_world* w, int32_t enable);
/* Per-phase GPU time in ms since the last reset: [sort, p2g, grid, g2p] — the labels
 * 'mpm sort' | 'mpm p2g' | 'mpm grid' | 'mpm g2p' of mpm.js:591-600. Timing is off until enabled. */
int si_world_profile(si_world* w, int32_t enable, double ms_out[4], int32_t reset);
/* Tuning knobs chosen by the autotuner (shaderintel_gb300/autotune.py): particles per CTA (256, 512
 * or 1024), the shared tile's capacity in nodes (a CTA whose stencils span more nodes uses the
 * global path) and the P2G flush strategy (0: shared tile, non-zero nodes flushed with global i32
 * atomics; 1: global i32 atomics per particle and node). Results are the same bits for every
 * setting. No counterpart in the reference, whose tile capacity follows the device limit. */
int si_world_set_tuning(si_world* w, int32_t particles_per_cta, int32_t tile_nodes, int32_t flush);
/* Timing on the world's own stream (the reference times regions with GPU timestamps,
 * src/core/context.js:168-181): si_world_mark records event `slot` (0..7); si_world_elapsed waits
 * for mark b and returns the GPU time from mark a to mark b in ms. */
int si_world_mark(si_world* w, int32_t slot);
int si_world_elapsed(si_world* w, int32_t a, int32_t b, double* ms);
/* Kernels this world has launched so far (graph replays count each kernel they contain). */
int si_world_launches(si_world* w, int64_t* count);

/* ---------------------------------------------------------------- the MPM object */
void si_mpm_desc_default(si_mpm_desc* d);
/* new MPM(ctx, o), mpm.js:89-127. world == NULL gives the scene a private world. */
int si_mpm_create(si_world* world, const si_mpm_desc* desc, si_mpm** out);
/* destroy(), mpm.js:262-267: frees the device memory; idempotent. The handle stays valid (every
 * later call but si_mpm_get_info/si_mpm_free returns SI_EDESTROYED) until si_mpm_free. */
int si_mpm_destroy(si_mpm* h);
void si_mpm_free(si_mpm* h);
int si_mpm_get_info(const si_mpm* h, si_mpm_info* out);

/* matBuf.write of _uploadMaterials, mpm.js:170-199: m <= 8 rows of 12 floats
 * [kind(u32 bits), mass, K|mu, lambda, visc, hardening, compression, stretch, DP alpha, 0, 0, 0]. */
int si_mpm_set_materials(si_mpm* h, const float* rows, int32_t m);
/* P.write(data, count*8) of add(), mpm.js:211-230: appends up to max_particles - count records;
 * *added (may be NULL) gets how many were taken. */
int si_mpm_add_particles(si_mpm* h, const float* records, int64_t n, int64_t* added);
/* clear(), mpm.js:238-242 (the host side forgets its materials itself). */
int si_mpm_clear(si_mpm* h);
/* P.write / P.read of raw records (tests, checkpoints), buffer.js:42-95, in current (sorted) order. */
int si_mpm_write_particles(si_mpm* h, const float* records, int64_t offset, int64_t n);
int si_mpm_read_particles(si_mpm* h, float* records, int64_t offset, int64_t n);
/* readPositions(), mpm.js:624-630: world xyz = x*dx + origin. */
/* The instance buffer of the sphere layer (spheres(), mpm.js:658-679, vertex stage of
 * src/render/spheres.js:50-60) without a renderer: per particle 8 floats — world x, y, z
 * (x * dx + origin in f32, as the shader), radius (dx / ppcAxis * 0.6 * size, 0 when the material
 * is not in mat_mask: the culled instance), world velocity (v * dx / dt in f32), material (u32 bits).
 * mat_mask = ~fluidMask() gives spheres({solidsOnly: true}). */
int si_mpm_read_instances(si_mpm* h, float* out, int64_t offset, int64_t n, uint32_t mat_mask, double size);
/* Read-only device views for zero-copy interop (the reference hands layers its GPU buffers, MPM.P /
 * MPM.grid): what = 0..7 particle stream k (float4 per particle: x, v, c0, c1, c2, f0, f1, f2 of the
 * record), 8 the grid of the last grid update (int4 / vec4f per node), 9 the block keys of the last
 * sort (u32, pre-sort order, as si_mpm_read_bins; SI_EINVAL for a scene admitted to a server), 10 the starts (u32, numBlocks + 1). *count = elements, *stride = bytes per element. Valid until the next
 * call that steps, sorts, adds or destroys; the caller orders its reads after si_mpm_sync. */
int si_mpm_device_ptr(si_mpm* h, int32_t what, const void** ptr, int64_t* count, int64_t* stride);
int si_mpm_read_positions(si_mpm* h, float* xyz, int64_t offset, int64_t n);
/* readPositions() as the reference's Promise (P.read, src/core/context.js:254-270): enqueues the
 * copy into `xyz` behind the work already queued and returns at once with a ticket (with pinned host
 * memory the copy runs while the host queues more steps); si_mpm_read_wait blocks until it landed. */
int si_mpm_read_positions_async(si_mpm* h, float* xyz, int64_t offset, int64_t n, uint64_t* ticket);
int si_mpm_read_wait(si_mpm* h, uint64_t ticket);
/* colBuf.writeOrdered of _uploadColliders, mpm.js:276-293: k <= 16 rows of 12 floats in lattice
 * units [kind(u32), center xyz, radius | half xyz | normal xyz, friction, velocity xyz (cells/substep), 0].
 * Taken by value; it reaches the device with the next step's parameters, ordered after the work
 * already queued, without waiting for it. */
int si_mpm_set_colliders(si_mpm* h, const float* rows, int32_t k);
/* gravity setter (m/s^2); applied as g*dt^2/dx per substep (mpm.js:588). */
int si_mpm_set_gravity(si_mpm* h, const double g[3]);
/* sortEvery setter, mpm.js:101. */
int si_mpm_set_sort_every(si_mpm* h, int32_t n);
/* substeps / timeScale setters, mpm.js:136-145: sets the substep length and rescales v and C
 * by k = dt_new / dt_old on the device (the retime kernel, mpm.js:405-413). */
int si_mpm_set_substep_dt(si_mpm* h, double dt);
int si_mpm_set_frame(si_mpm* h, int32_t substeps, double time_scale);
/* step(), mpm.js:582-604, generalised to step(dt, K): K substeps of length dt (dt <= 0 keeps the
 * current one; a new dt retimes first). K <= 0 steps one frame of `substeps` substeps. */
int si_mpm_step(si_mpm* h, double dt, int32_t K);
/* _sort(), mpm.js:614-621: Morton block counting sort, stable. */
int si_mpm_sort(si_mpm* h);
/* p2g(P, forceGlobal), mpm.js:607-612: clears the grid and scatters (tile or global atomics). */
int si_mpm_p2g(si_mpm* h, int32_t force_global);
/* gridK.run, mpm.js:593-595, and g2pK.run, mpm.js:598-600, one phase each (for parity tests). */
int si_mpm_grid_update(si_mpm* h);
int si_mpm_g2p(si_mpm* h);
/* grid.read(), the raw node words (4 x i32 per node). */
int si_mpm_read_grid(si_mpm* h, int32_t* nodes4);
/* key and blockCount of the last sort, mpm.js:122-124: keys in the pre-sort particle order,
 * starts = the exclusive scan of the block counts (num_blocks + 1 entries, last = count).
 * Either pointer may be NULL. A scene admitted to a server keeps no keys: keys must be NULL for it
 * (SI_EINVAL otherwise). */
int si_mpm_read_bins(si_mpm* h, uint32_t* keys, uint32_t* starts);
int si_mpm_sync(si_mpm* h);

/* Allocation-free block binning (no counterpart in the reference: its sort always runs on buffers
 * the MPM object allocated). For callers that must not allocate device memory themselves or through
 * this library: a host whose allocator owns all of the GPU's memory, a stream being recorded into a
 * CUDA graph, a frame loop that cannot take the device-wide synchronisation of cudaFree. Given n
 * positions on the device (x at x[i * stride_floats + 0..2]) and the grid dims, it writes, all on
 * the device: keys[n] (the block key of each particle, mpm.js:567-569), perm[n] (the stable sorted
 * order: entry d is the index of the particle that goes to slot d) and starts[numBlocks + 1] (the
 * exclusive scan of the block counts). Work is queued on `stream` (NULL: the default stream).
 * Its scratch is one fixed device array inside this library (about 4.3 MB per GPU that loads it,
 * kept until the process exits): n may be at most 262144, larger n fails with SI_EINVAL. Every
 * call uses the same array, so calls that overlap on the GPU (other streams, other threads) race:
 * order them. The first call on each device looks up the array's address; make that first call
 * before any stream capture. That address is kept for the life of the process: do not call this
 * after a cudaDeviceReset (or any other reset of the device's primary context), which reloads the
 * library's device code elsewhere. No part of the scratch needs to start at zero. */
int si_block_sort_noalloc(const float* x, int64_t stride_floats, int32_t n, const int32_t dims[3],
                          uint32_t* keys, uint32_t* perm, uint32_t* starts, void* stream);

/* ---------------------------------------------------------------- host helpers (no device)
 * The reference's host-side arithmetic, in f64 as JavaScript does it, so that every host that
 * drives this library builds bit-identical scenes. */
typedef struct si_material_def {
  int32_t kind;          /* 0 fluid, 1 jelly (Neo-Hookean), 2 snow, 3 sand */
  double density;        /* relative to water, (0, 50] */
  double stiffness;      /* fraction (0,1] of the max stable wave speed */
  double poisson, viscosity, hardening, compression, stretch, friction_deg;
} si_material_def;
/* MATERIALS presets, mpm.js:38-46: water oil honey jelly rubber snow sand. */
int si_material_preset(const char* name, si_material_def* out);
/* One row of _uploadMaterials, mpm.js:174-195, with the validation of _material, mpm.js:148-159. */
int si_material_row(const si_material_def* def, int32_t ppc_axis, float row[12]);
/* sampleShape, mpm.js:683-714: shape 0 box (a=lo, b=hi), 1 sphere (a=center, r), 2 cylinder
 * (a=center, r, h). Writes up to cap xyz triples (world units, f32) and returns the number in *n
 * (with out == NULL only counts). */
int si_sample_shape(int32_t shape, const double a[3], const double b[3], double r, double h,
                    double spacing, double jitter, uint32_t seed, float* out, int64_t cap, int64_t* n);
/* The per-particle conversion of add(), mpm.js:213-227: world points -> records. */
int si_make_records(const si_mpm* h, const float* xyz, int64_t n, int32_t material,
                    const double velocity[3], double substep_dt, float* records);
/* One row of _uploadColliders, mpm.js:280-291 (type 0 sphere, 1 box, 2 plane). */
int si_collider_row(const si_mpm* h, int32_t type, const double center[3], const double vec3[3],
                    double radius, double friction, const double velocity[3], double substep_dt,
                    float row[12]);

/* add(shape, opts) with the sampling on the device (mpm.js:207-232, sampleShape mpm.js:683-714):
 * shape 0 box (a = lo, b = hi), 1 sphere (a = centre, radius), 2 cylinder (a = centre, radius,
 * half_height), world units; lattice spacing dx / ppcAxis; xorshift32 jitter from `seed`
 * (0 -> 1); `material` is the slot of set_materials; truncated at maxParticles. The records equal,
 * bit for bit, si_sample_shape + si_make_records + si_mpm_add_particles. *added = particles added. */
int si_mpm_emit(si_mpm* h, int32_t shape, const double a[3], const double b[3], double radius, double half_height,
                double jitter, uint32_t seed, int32_t material, const double velocity[3], int64_t* added);

/* ---------------------------------------------------------------- fluid <-> rigid coupling
 * MPM.couple(world, o) / uncouple() (mpm.js:244-259, src/physics/coupling.js:62-222): rigid bodies
 * become moving boundaries of the grid. `bodies` is n records of 48 floats, the reference's Body
 * (src/physics/rigid-wgsl.js:20-33: x (w = bounding radius), q, v, w, x0, q0, y, qy, size (w = shape
 * 0 sphere / 1 box / 2 capsule), mass (x = m, 0 = static), props, info (4 u32 bit patterns: group,
 * mask, flags, user)), in world units. Every substep the pass runs after the grid update with the
 * bodies extrapolated by v (s + 0.5) dt, s the substep's index in its step() call
 * (coupling.substep, mpm.js:596). n = 0 uncouples. friction 0.2, band 0.5 cells, mask all bits and
 * density_scale 1 are the reference's defaults. */
int si_mpm_couple(si_mpm* h, const float* bodies, int32_t n, double friction, double band, uint32_t mask,
                  double density_scale);
/* The rigid world moved: new body records (same count) for the next substeps (the B buffer). The
 * table is copied before the call returns (into pinned staging memory), so the caller may reuse it
 * at once; the call does not wait for the GPU. */
int si_mpm_set_bodies(si_mpm* h, const float* bodies, int32_t n);
/* coupling.finish() (coupling.js:199-206, mpm-rigid-apply): the reaction impulses summed since the
 * last read, in world units, n x 8 floats (J xyz, 0, L xyz, 0) — what the reference adds to the
 * rigid world's external impulses; the sums restart from zero. */
int si_mpm_read_impulses(si_mpm* h, float* out, int32_t n);

/* ---------------------------------------------------------------- SpatialGrid (src/prims/grid.js)
 * Counting-sort binning of points into a uniform grid, the prim the MPM block sort specialises:
 * new SpatialGrid(ctx, {maxCount, min, max, cellSize}) (grid.js:25-55): dims = max(1,
 * ceil((max - min) / cellSize)) per axis, at most 2^26 cells. build(pos, count) (grid.js:69-76):
 * cell = gridIndex(gridCoord(p)) (grid.js:14-20, x fastest, clamped to the grid), order = point
 * indices sorted by cell, start = first sorted slot of every cell (numCells + 1 entries). Within a
 * cell the reference ranks by atomic arrival (any order); here by index (stable, deterministic).
 * Calls take the world's lock and run on its stream. */
int si_spatial_create(si_world* w, int64_t max_count, const double min[3], const double max[3], double cell_size,
                      si_spatial** out);
int si_spatial_destroy(si_spatial* g);
int si_spatial_info(const si_spatial* g, int32_t dims[3], int64_t* num_cells, int64_t* count);
/* pos: count x 4 floats (vec4f, xyz used), host memory */
int si_spatial_build(si_spatial* g, const float* pos, int64_t count);
/* the same over an MPM scene's current particle positions (lattice units), without a copy */
int si_spatial_build_mpm(si_spatial* g, const si_mpm* h);
/* order (count u32) and start (numCells + 1 u32) of the last build; either may be NULL */
int si_spatial_read(si_spatial* g, uint32_t* order, uint32_t* start);
/* gather(src, dst), grid.js:79-90: dst[k] = src[order[k]] for `width` floats per point, host arrays */
int si_spatial_gather(si_spatial* g, const float* src, float* dst, int32_t width);

/* ---------------------------------------------------------------- serving
 * A request loop that keeps every scene resident in HBM and runs step(dt, K) requests by
 * continuous batching: each tick is one substep of every scene with work left; requests that
 * arrive while others run join at the next tick. */
typedef struct si_server_stats {
  int64_t requests_done, substeps_done, particle_substeps, ticks;
  double p50_ms, p99_ms, mean_ms, max_ms; /* request latency, submit -> completion */
  double busy_s;                           /* wall time with work on the device */
  int64_t resident_bytes, budget_bytes;
  int32_t resident_scenes, queued_requests;
} si_server_stats;
/* The server steps `world` from its own thread until si_server_destroy; scenes already in the
 * world become resident. Edits of resident scenes stay allowed from any thread. Scenes created in
 * the world while it has a server keep one particle buffer instead of two (their sort substeps read
 * a gathered copy of the old state from the world's scratch) and no block keys (their sorts key the
 * positions as they start, so si_mpm_read_bins and si_mpm_device_ptr give their starts but refuse
 * their keys with SI_EINVAL); the gathered copy and the sort's scratch are held
 * below min(2 GiB, budget / 32) by running a tick's scenes in groups, and that reserve counts
 * against the budget (si_server_stats.resident_bytes includes it). */
int si_server_create(si_world* world, int64_t budget_bytes, si_server** out);
int si_server_destroy(si_server* s);
/* Admission by footprint: creates a resident scene if it fits the HBM budget, else SI_ENOMEM. The
 * footprint is 128 B x maxParticles (one particle buffer) + 32 B x grid nodes + 4 B x (numBlocks + 1)
 * + about 1.4 KB. */
int si_server_admit(si_server* s, const si_mpm_desc* desc, si_mpm** out);
/* Retires a scene (frees its HBM); pending requests on it complete with SI_EDESTROYED. */
int si_server_retire(si_server* s, si_mpm* h);
/* Queues step(dt, K) on a resident scene; returns a ticket. The scene keeps its collider table. */
int si_server_submit(si_server* s, si_mpm* h, double dt, int32_t K, uint64_t* ticket);
/* The same with the collider table that this step uploads (rows of si_collider_row, ncol <= 16
 * used; ncol = 0 clears the table, ncol < 0 keeps the scene's): the reference's step() uploads its
 * colliders first (mpm.js:586), and here the table travels with the request, so queued requests of
 * one scene each run with their own table. It is applied when the request's first substep is
 * enqueued, and submitting takes no lock that a running round holds. */
int si_server_submit_colliders(si_server* s, si_mpm* h, double dt, int32_t K, const float* rows, int32_t ncol,
                               uint64_t* ticket);
/* *done = 1 once the ticket's K substeps are on the device and finished; *status its result. */
int si_server_poll(si_server* s, uint64_t ticket, int32_t* done, int32_t* status);
int si_server_wait(si_server* s, uint64_t ticket, int32_t timeout_ms, int32_t* status);
int si_server_stats_get(si_server* s, si_server_stats* out, int32_t reset);
/* Runs fn(ctx) between two rounds, holding the world (several edits that must land together). */
int si_server_call(si_server* s, void (*fn)(void*), void* ctx);

#ifdef __cplusplus
}
#endif
#endif
