// si_device.h — structures shared by the host runtime (si_runtime.cpp) and the kernels (*.cu).
//
// HBM layout of one scene:
//   particles: two buffers (ping-pong for the sort), each 8 SoA streams of float4 with stride `cap`
//              (stream k = vec4 k of the reference record: x, v, c0, c1, c2, f0, f1, f2);
//   grid:      two node arrays of int4 (ping-pong: P2G of substep s+1 is fused into the G2P of
//              substep s and lands in the other array, which the grid update of s cleared);
//   keys:      u32 per particle (block key of the last sort, pre-sort order, mpm.js:569);
//   starts:    u32 x (num_blocks + 1) (mpm.js:122, after the scan);
//   box:       i32 x 2 x 8: for each grid array, the box of the particle bases whose P2G filled it.
//              A node outside the box of an array is zero there, so the grid update of a scene in
//              steady stepping visits only box_cur + box_next (+ the stencil reach), not the grid.
// A tick is one substep of every scene that has work. The host builds one TickScene per such
// scene; kernels map a flat chunk index to its scene by binary search over the chunk prefixes.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace si {

constexpr int kStreams = 8;           // float4 streams per particle
constexpr int kCtaThreads = 256;      // threads per CTA of the particle kernels
constexpr int kMaxPpt = 4;            // particles per thread in one chunk, at most
constexpr int kNodeChunk = 2048;      // grid nodes per work item of the grid kernel (small grids: fewer)
constexpr int kSortTile = 4096;       // keys per CTA of a radix pass (256 threads x 16)
constexpr int kRadixBits = 8;

// TickScene.flags
constexpr uint32_t F_P2G = 1u;        // run a standalone P2G into `grid` this substep
constexpr uint32_t F_GATHER = 2u;     // this substep sorts: G2P (or the reorder) reads P[perm] and writes Palt
constexpr uint32_t F_FUSE = 4u;       // G2P also scatters the new particle state into grid_next
constexpr uint32_t F_KEYS = 8u;       // G2P also writes the block key of the new position
constexpr uint32_t F_FORCE_GLOBAL = 16u; // P2G skips the shared-memory tile (mpm.js:380)
constexpr uint32_t F_NO_CLEAR_NEXT = 32u; // grid update leaves grid_next alone
constexpr uint32_t F_KEYS_NOW = 64u;  // compute the block keys of the current positions before the sort
constexpr uint32_t F_CLEAR = 128u;    // zero `grid` before the standalone P2G
constexpr uint32_t F_BOXED = 256u;    // grid update: nodes outside box_cur + box_next are zero in both arrays
constexpr uint32_t F_COUPLE = 512u;   // run the fluid <-> rigid coupling pass after the grid update
constexpr uint32_t F_PREGATHER = 1024u; // with F_GATHER, a scene with one particle buffer: the read streams were
                                        // gathered into the world's scratch in sorted order (k_pregather),
                                        // and the G2P reads them there and writes P in place
constexpr uint32_t F_KEYS_FROM_X = 2048u; // with F_GATHER, a scene without key buffers: the sort's first kernel
                                          // computes the block keys from the current positions

struct SceneParams {             // per scene, device resident, rewritten when a value changes
  float4 mats[24];               // 8 materials x 3 vec4 (mpm.js:116)
  float4 cols[48];               // 16 colliders x 3 vec4 (mpm.js:117)
  int32_t dims[3];
  int32_t ncol;
  float gravity[3];              // lattice units per substep^2 at the scene's dt
  float bound;                   // 3
  float floor_friction;          // 0.4
  float vmax;                    // 0.9
  float vol4;                    // 4 / ppcAxis^3
  uint32_t num_blocks;
  // fluid <-> rigid coupling (src/physics/coupling.js): body table and pass parameters
  const float4* bodies;          // nbodies x 12 float4, the reference's Body record
  int32_t* body_acc;             // nbodies x 8 i32: J x 16384 [0..2], L x 1024 [4..6]
  int32_t nbodies;
  uint32_t body_mask;            // group bits of the bodies that interact
  float origin[3];               // world origin of node 0
  float dx, inv_dx;
  float vel_to_lattice;          // substep dt / dx
  float friction, band;          // 0.2, 0.5 cells
};

struct TickScene {               // per tick and active scene, host built
  const SceneParams* prm;
  float4* P;                     // particle state read this substep (current buffer)
  float4* Palt;                  // destination of the sort's gather
  int4* grid;                    // grid of this substep
  int4* grid_next;               // grid of the next substep
  int32_t* box_cur;              // stencil-base box (min xyz, max xyz) of the P2G that filled `grid`
  int32_t* box_next;             // the same for `grid_next` (the fused P2G of this substep adds to it)
  uint32_t* keys;                // block keys this tick's sort reads (pre-sort order; k_keys fills them)
  uint32_t* keys_next;           // where the G2P writes the keys of the next sort (the other buffer
                                 // when this tick sorts, so the last sort's keys stay readable)
  uint32_t* starts;              // per-scene starts (num_blocks + 1)
  int64_t cap;                   // stream stride in float4
  int32_t n;                     // particles
  uint32_t flags;
  uint32_t seg_base;             // first slot of this scene in the concatenated sort arrays
  uint32_t bin_base;             // first global bin of this scene
  uint32_t pchunk_begin;         // first particle chunk of this scene (prefix over the tick)
  uint32_t nchunk_begin;         // first node chunk
  int32_t node_chunk;            // grid nodes per node chunk of this scene (256..kNodeChunk)
  uint32_t cchunk_begin;         // first 4^3 node tile of the coupling pass
  float lead;                    // coupling: bodies extrapolated by v * lead = (s + 0.5) * dt
};

struct TickInfo {                // one tick's totals (kernel arguments)
  const TickScene* ts;
  int32_t nscenes;
  uint32_t pchunks;              // particle chunks of all scenes
  uint32_t nchunks;              // node chunks
  int32_t chunk;                 // particles per chunk (= kCtaThreads * ppt)
  int32_t tile_nodes;            // shared tile capacity in nodes
  uint32_t cchunks;              // 4^3 node tiles of the coupled scenes
  float nz;                      // -0.0f: the addend of packed products (see mul2z in si_kernels.cu)
  uint32_t* grid_done;           // CTAs of k_grid that finished (the last one resets it to 0)
  const float4* gscratch;        // k_pregather's output: streams x, v, f0, f1, f2 of the sorting
                                 // particles in sorted order (segment seg_base of each scene)
  int64_t gstride;               // stream stride of gscratch in float4
  uint32_t* g2p_sched;           // k_g2p: [0] chunks handed out past the first wave, [1] CTAs
                                 // finished (the last one resets both to 0)
  int32_t reset_boxes;           // k_grid's last CTA empties every scene's box_next
};

struct SortInfo {                // one tick's sort
  uint32_t n;                    // elements = particles of the sorting scenes
  uint32_t bins;                 // total bins
  int32_t passes;
  uint32_t* keys_a; uint32_t* vals_a;
  uint32_t* keys_b; uint32_t* vals_b;
  uint32_t* hist;                // 256 x tiles
  uint32_t* digit_total;         // 256
  const uint32_t* keys_in;       // one sorting scene at offset 0: its keys, read by the first pass
                                 // with identity indices (no concatenation), else nullptr
  uint32_t* starts_out;          // that scene's starts (written by the one-CTA sort), else nullptr
  // Segmented sort (keys_in == nullptr): every sorting scene's keys are its own block keys, its
  // segment starts on a tile boundary and is padded to whole tiles with `sentinel` (above every key),
  // and each pass ranks digits within a scene's tiles only, so the passes cover the largest scene's
  // key range instead of the tick's total bins.
  uint32_t* tile_scene;          // tiles: the tick-table index of the scene a tile belongs to
  uint32_t* seg_total;           // scenes x 256: a scene's digit totals of the current pass
  uint32_t sentinel;
};

// One sorting scene small enough for the one-CTA sort (k_small_sort): its keys and per-warp bin
// counters fit in shared memory, and one pass over all bins replaces the radix passes and the
// starts kernel.
constexpr uint32_t kSmallSortMaxN = 32768;
constexpr uint32_t kSmallSortMaxBins = 512;
inline bool small_sort_ok(uint32_t n, uint32_t bins, bool single) {
  return single && n > 0 && n <= kSmallSortMaxN && bins > 0 && bins <= kSmallSortMaxBins;
}

// ---- launchers (si_kernels.cu / si_sort.cu); all enqueue on `st`.
void launch_p2g(const TickInfo& t, int grid_ctas, cudaStream_t st);
void launch_clear(const TickInfo& t, int grid_ctas, cudaStream_t st);
void launch_grid(const TickInfo& t, int grid_ctas, int grid_ctas_wide, cudaStream_t st);
void launch_box_reset(const TickInfo& t, cudaStream_t st);
void launch_couple(const TickInfo& t, int grid_ctas, cudaStream_t st);
void launch_g2p(const TickInfo& t, const uint32_t* perm, int grid_ctas, cudaStream_t st,
                bool pre,     // the tick holds a one-buffer scene that sorts
                bool fast);   // snow and sand decompose F to a tolerance
void launch_reorder(const TickInfo& t, const uint32_t* perm, int grid_ctas, cudaStream_t st);
void launch_pregather(const TickInfo& t, const uint32_t* perm, float4* scratch, int64_t stride, int grid_ctas,
                      cudaStream_t st);
constexpr int kPregatherStreams = 5;   // x, v (for J), f0, f1, f2: what the G2P reads of the old state
void launch_keys(const TickInfo& t, int grid_ctas, cudaStream_t st);
void launch_retime(float4* P, int64_t cap, int32_t n, float k, cudaStream_t st);
void launch_aos_to_soa(const float* aos, float4* P, int64_t cap, int64_t off, int64_t n, cudaStream_t st);
void launch_soa_to_aos(const float4* P, int64_t cap, int64_t off, int64_t n, float* aos, cudaStream_t st);
void launch_instances(const float4* P, int64_t cap, int64_t off, int64_t n, float scale, const float offset[3],
                      float radius, float vel_scale, uint32_t mat_mask, float* out, cudaStream_t st);
void launch_positions(const float4* P, int64_t cap, int64_t off, int64_t n, double dx,
                      const double origin[3], float* xyz, cudaStream_t st);
// Sort of one tick: builds the concatenated (key, index) arrays of the sorting scenes, radix
// sorts them and leaves perm (sorted source indices, per segment) in *perm_out and the sorted
// keys in *keys_out.
bool launch_sort(const TickInfo& t, const SortInfo& s, const uint32_t** perm_out,
                 const uint32_t** keys_out, int grid_ctas, cudaStream_t st);   // true: starts written
// Per-scene starts (reference blockCount after the scan) of every sorting scene.
void launch_scene_starts_all(const TickInfo& t, const uint32_t* sorted_keys, uint32_t max_blocks,
                             cudaStream_t st);
// Per-device kernel attributes (dynamic shared memory opt-ins), set with the device current.
cudaError_t configure_sort_kernels();
int p2g_smem_bytes(int tile_nodes, int ppt);
int max_tile_nodes();
int occupancy_ctas(int which, int tile_nodes, int ppt);
int couple_ctas_per_sm();                                 // resident k_couple CTAs per SM   // resident CTAs per SM of kernel `which`

}  // namespace si
