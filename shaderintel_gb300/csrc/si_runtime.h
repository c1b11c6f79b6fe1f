// si_runtime.h — host objects of libsi_cuda (internal): the world, the scene, cached graph plans.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "si_cuda.h"
#include "si_device.h"

struct GraphTick {
  int mode;
  uint32_t pchunks, nchunks, cchunks;
  bool any_p2g, any_clear, any_gather, any_keys_now;
  uint32_t sort_n;
  int passes;
};

// A plan of ticks captured once and replayed while the tables it was built from repeat.
struct GraphPlan {
  cudaGraphExec_t exec = nullptr;
  void* table = nullptr;            // device copy of the plan's tick tables
  std::vector<uint8_t> bytes;       // host copy, the replay key
  std::vector<GraphTick> ticks;
  int ppt = 0, tile_nodes = 0;
  uint64_t last_use = 0;
  int64_t kernels = 0;              // kernels in the graph
  ~GraphPlan();
};

struct si_world {
  int device = 0;
  cudaStream_t st = nullptr;
  int sms = 1;
  int max_smem_optin = 48 * 1024;
  std::vector<si_mpm*> scenes;
  bool destroyed = false;
  std::atomic<si_server*> server{nullptr};
  std::recursive_mutex api_mu;      // serialises API calls on this world with the server's rounds
  // tuning (autotuner: particles per CTA = 256 * ppt, shared tile capacity in nodes)
  int ppt = 1, tile_nodes = 2048;
  int flush = 0;                    // P2G flush: 0 shared tile + non-zero node flush, 1 global atomics
  int ctas_p2g = 0, ctas_g2p = 0, ctas_grid = 0, ctas_grid_wide = 0, ctas_misc = 0, ctas_couple = 0;
  // sort scratch (grown on demand)
  uint32_t *ka = nullptr, *va = nullptr, *kb = nullptr, *vb = nullptr;
  size_t sort_cap = 0;
  uint32_t* hist = nullptr;
  size_t hist_cap = 0;
  uint32_t* digit_total = nullptr;
  uint32_t* tile_scene = nullptr;   // segmented sort: scene of every tile
  size_t tile_scene_cap = 0;
  uint32_t* seg_total = nullptr;    // segmented sort: 256 digit totals per scene of a tick
  size_t seg_total_cap = 0;
  // One-buffer scenes (created while `compact` is set, as a server's are): their sort substeps
  // gather the G2P's inputs into this scratch (kPregatherStreams x 16 B per sorting particle), and a
  // tick whose sorting particles exceed group_particles runs as several groups of scenes, so the
  // scratch (with the sort's) stays below group_particles x 96 B.
  bool compact = false;
  int64_t group_particles = 0;      // 0: no limit
  float4* gscratch = nullptr;
  size_t gscratch_cap = 0;          // particles
  uint32_t* grid_done = nullptr;    // k_grid's finished-CTA counter, then k_g2p's chunk and finished-CTA
                                    // counters (all zero between launches)
  // tick tables of direct (non-graph) execution
  si::TickScene* tab = nullptr;
  size_t tab_cap = 0;
  // graphs
  bool use_graphs = true;
  bool svd_tolerance = false;       // snow/sand SVD to a tolerance (si_world_set_svd_tolerance)
  std::vector<std::unique_ptr<GraphPlan>> graphs;
  uint64_t graph_clock = 0;
  uint64_t seen[16] = {};           // hashes of recent plans: a plan is captured when it repeats
  int seen_next = 0;
  // profiling: per-phase time [sort, p2g, grid, g2p]
  bool profile = false;
  double prof_ms[4] = {0, 0, 0, 0};
  cudaEvent_t pev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t marks[8] = {};
  std::map<uint64_t, cudaEvent_t> reads;   // asynchronous readbacks in flight, by ticket
  cudaStream_t st_copy = nullptr;          // their device-to-host copies, beside the next steps
  uint64_t next_read = 1;
  int64_t launches = 0;             // kernels enqueued (graph replays add their kernel count)
  // Pinned staging of host-to-device uploads. From pageable memory cudaMemcpyAsync first waits for
  // the stream, so a per-frame parameter or table upload would hold the host until the GPU drained
  // and leave the GPU idle while the next frame is enqueued. A slot is reused once the copy out of
  // it has run (its event), which only waits when the host is a whole ring ahead of the stream.
  static constexpr int kPrmSlots = 1024;
  si::SceneParams* prm_ring = nullptr;      // kPrmSlots slots, allocated on first use
  cudaEvent_t prm_ev[kPrmSlots] = {};
  int prm_next = 0;
  static constexpr int kStageSlots = 8;
  void* stage[kStageSlots] = {};            // tick tables and body tables, grown on demand
  size_t stage_cap[kStageSlots] = {};
  cudaEvent_t stage_ev[kStageSlots] = {};
  int stage_next = 0;
};

struct si_mpm {
  si_world* w = nullptr;
  bool own_world = false;
  bool destroyed = false;
  // properties of the reference object (mpm.js:89-127)
  int64_t cap = 0;                  // maxParticles
  int32_t dims[3] = {0, 0, 0};
  double dx = 0, size[3] = {0, 0, 0}, origin[3] = {0, 0, 0}, gravity[3] = {0, 0, 0};
  int32_t substeps = 8, sort_every = 4, ppc_axis = 2, bound = 3;
  double time_scale = 1, dt = 0;
  int64_t count = 0, step_count = 0, nodes = 0;
  uint32_t num_blocks = 0;
  float mats[96] = {};
  int32_t nmats = 0;
  float cols[192] = {};
  int32_t ncol = 0;
  // device state
  float4* pbuf[2] = {nullptr, nullptr};   // pbuf[1] is null for a one-buffer (compact) scene
  bool compact = false;
  int pcur = 0;
  int4* grid[2] = {nullptr, nullptr};
  int gcur = 0;                     // grid of the last substep
  uint32_t* keys[2] = {nullptr, nullptr};   // block keys: [kpend] for the next sort, the other the last sort's
  int kpend = 0;
  uint32_t* starts = nullptr;
  int32_t* box = nullptr;           // [2][8]: stencil-base box of the P2G that filled grid[0] / grid[1]
  int box_ok = 0;                   // standard substeps in a row (>= 2: both boxes describe the arrays)
  // fluid <-> rigid coupling (src/physics/coupling.js): the body table and its impulse sums
  float4* bodies = nullptr;         // nbodies x 12 float4
  int32_t* body_acc = nullptr;      // nbodies x 8 i32
  int32_t nbodies = 0;
  uint32_t body_mask = 0xffffffffu;
  double friction = 0.2, band = 0.5, density_scale = 1.0;
  int32_t frame_sub = 0;            // substeps since the step call began (the coupling's lead)
  si::SceneParams* prm = nullptr;
  bool prm_dirty = true;
  bool pending = false;             // grid[1-gcur] holds the P2G of the current particle state
  bool next_clear = false;          // grid[1-gcur] is zero
  bool keys_valid = false;          // keys hold the block keys of the current positions
  int64_t device_bytes = 0;
  // serving: a scene admitted by a server is retired through it
  bool served = false;
};

int world_configure(si_world* w, int ppt, int tile_nodes);
int run_substeps(si_world* w, const std::vector<si_mpm*>& scenes, int K);
int scene_create(si_world* w, const si_mpm_desc* in, si_mpm** out, bool own_world);
int64_t scene_footprint_of(const si_mpm_desc* in, bool compact);
constexpr int64_t kGroupBytesPerParticle = 16 + 16 * si::kPregatherStreams;   // sort + pregather scratch

namespace si {
cudaError_t configure_kernels(int tile_nodes);   // per device, with it current
}
