// si_runtime.cpp — host runtime of libsi_cuda: worlds (a CUDA stream and its scenes), scenes (the
// reference's MPM object, mpm.js:82-680), the substep schedule (mpm.js:582-604) and its execution
// as ticks of persistent kernels, replayed from CUDA graphs when a plan repeats.
//
// Schedule of one substep of scene s (the reference runs sort?, clear+P2G, grid, G2P):
//   sort (every sort_every substeps): keys of the current positions, stable radix sort -> perm;
//   P2G: already done by the previous G2P ("pending") or a standalone P2G into the grid;
//   grid update: in place, and clears the other grid array;
//   G2P: reads P (through perm when sorting, writing the sorted buffer), then scatters the new
//        state into the other grid array (the next substep's P2G) and, when the next substep
//        sorts, writes the block keys of the new positions.
// Grid sums are integer and order-independent, so the fused P2G equals the reference's P2G bit
// for bit even though it runs over the pre-sort order.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "si_cuda.h"
#include "si_device.h"
#include "si_emit.h"
#include "si_internal.h"
#include "si_runtime.h"

using namespace si;

namespace {
thread_local std::string t_err;
}

int si_fail(int code, const std::string& msg) {
  t_err = msg;
  return code;
}

extern "C" int si_fail_c(int code, const char* msg) { return si_fail(code, msg ? msg : ""); }

#define CK(call)                                                                               \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return si_fail(SI_EDEVICE, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------------------ helpers
static double js_round(double x) {   // Math.round: halves toward +infinity
  double f = std::floor(x);
  return (x - f >= 0.5) ? f + 1.0 : f;
}

static uint32_t num_blocks_for(const int32_t d[3]) {
  int32_t bmax = 0;
  for (int a = 0; a < 3; a++) bmax = std::max(bmax, (int32_t)std::ceil(d[a] / 4.0));
  uint32_t bpow = 1u << (uint32_t)std::ceil(std::log2((double)bmax));
  return bpow * bpow * bpow;
}

// Device bytes of a scene: particle buffers (two, or one for a compact scene), two grids, two key
// buffers (none for a compact scene), the starts, the parameters and the boxes.
static int64_t scene_footprint(int64_t cap, int64_t nodes, uint32_t nb, bool compact) {
  return (compact ? 1 : 2) * (int64_t)kStreams * 16 * cap + 2 * 16 * nodes + (compact ? 0 : 2 * 4 * cap) +
         4 * ((int64_t)nb + 1) + (int64_t)sizeof(SceneParams) + 64;
}

int64_t scene_footprint_of(const si_mpm_desc* in, bool compact) {
  si_mpm_desc d;
  si_mpm_desc_default(&d);
  if (in) {
    if (in->max_particles > 0) d.max_particles = in->max_particles;
    if (in->grid > 0) d.grid = in->grid;
    if (in->size[0] > 0 || in->size[1] > 0 || in->size[2] > 0)
      for (int a = 0; a < 3; a++) d.size[a] = in->size[a];
  }
  double dx = std::max(d.size[0], std::max(d.size[1], d.size[2])) / d.grid;
  int32_t dims[3];
  for (int a = 0; a < 3; a++) dims[a] = (int32_t)std::max(8.0, js_round(d.size[a] / dx));
  return scene_footprint(d.max_particles, (int64_t)dims[0] * dims[1] * dims[2], num_blocks_for(dims), compact);
}

void si_scene_geometry(const si_mpm* h, si_scene_geom* g) {
  for (int a = 0; a < 3; a++) { g->dims[a] = h->dims[a]; g->origin[a] = h->origin[a]; }
  g->dx = h->dx;
  g->substep_dt = h->dt;
  g->bound = h->bound;
}

// ------------------------------------------------------------------ world
static int world_init(si_world* w) {
  CK(cudaGetDevice(&w->device));
  cudaDeviceProp p;
  CK(cudaGetDeviceProperties(&p, w->device));
  w->sms = p.multiProcessorCount;
  w->max_smem_optin = (int)p.sharedMemPerBlockOptin;
  CK(cudaStreamCreateWithFlags(&w->st, cudaStreamNonBlocking));
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, w->device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  for (auto& e : w->pev) CK(cudaEventCreate(&e));
  for (auto& e : w->marks) CK(cudaEventCreate(&e));
  CK(cudaMalloc((void**)&w->grid_done, 4 * sizeof(uint32_t)));   // k_grid's counter, k_g2p's two
  CK(cudaMemset(w->grid_done, 0, 4 * sizeof(uint32_t)));
  return world_configure(w, w->ppt, std::min(w->tile_nodes, max_tile_nodes()));
}

int world_configure(si_world* w, int ppt, int tile_nodes) {
  if (ppt != 1 && ppt != 2 && ppt != 4) return si_fail(SI_EINVAL, "particles per CTA must be 256, 512 or 1024");
  if (tile_nodes < 343 || tile_nodes > max_tile_nodes() || p2g_smem_bytes(tile_nodes, ppt) > w->max_smem_optin)
    return si_fail(SI_EINVAL, "tile capacity must hold at least 7^3 nodes and fit shared memory");
  {
    // kernel attributes are per device: set them on the world's, whichever device this thread has current
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) cur = -1;
    if (cur != w->device) CK(cudaSetDevice(w->device));
    const cudaError_t e = configure_kernels(tile_nodes);
    if (cur >= 0 && cur != w->device) cudaSetDevice(cur);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return si_fail(SI_EDEVICE, "setting the kernels' shared-memory attributes failed");
    }
  }
  w->ppt = ppt;
  w->tile_nodes = tile_nodes;
  const int which_g2p = ppt == 1 ? 3 : (ppt == 4 ? 4 : 1);
  w->ctas_p2g = w->sms * occupancy_ctas(0, tile_nodes, ppt);
  w->ctas_g2p = w->sms * occupancy_ctas(which_g2p, tile_nodes, ppt);
  w->ctas_grid = w->sms * occupancy_ctas(2, tile_nodes, ppt);
  w->ctas_grid_wide = w->sms * occupancy_ctas(5, tile_nodes, ppt);
  w->ctas_misc = w->sms * 4;
  w->ctas_couple = w->sms * couple_ctas_per_sm();
  cudaGetLastError();
  w->graphs.clear();
  return SI_OK;
}

static void world_free_graphs(si_world* w) {
  if (!w->graphs.empty()) cudaStreamSynchronize(w->st);
  w->graphs.clear();
}

GraphPlan::~GraphPlan() {
  if (exec) cudaGraphExecDestroy(exec);
  if (table) cudaFree(table);
}

static int ensure_dev(si_world* w, void** p, size_t* cap, size_t need) {
  if (need <= *cap) return SI_OK;
  size_t n = std::max(need, *cap + *cap / 2);
  if (*p) CK(cudaFreeAsync(*p, w->st));
  *p = nullptr;
  *cap = 0;
  CK(cudaMallocAsync(p, n, w->st));
  *cap = n;
  return SI_OK;
}

// ------------------------------------------------------------------ scene parameters
static void build_params(const si_mpm* h, SceneParams* p) {
  std::memset(p, 0, sizeof(*p));
  std::memcpy(p->mats, h->mats, sizeof(h->mats));
  std::memcpy(p->cols, h->cols, sizeof(h->cols));
  for (int a = 0; a < 3; a++) {
    p->dims[a] = h->dims[a];
    p->gravity[a] = (float)((h->gravity[a] * h->dt * h->dt) / h->dx);   // mpm.js:588
  }
  p->ncol = std::min(16, h->ncol);
  p->bound = (float)h->bound;
  p->floor_friction = 0.4f;   // mpm.js:594
  p->vmax = 0.9f;             // mpm.js:599
  p->vol4 = (float)(4 * (1.0 / std::pow((double)h->ppc_axis, 3.0)));   // mpm.js:589,610
  p->num_blocks = h->num_blocks;
  // coupling uniforms, coupling.js:212-214 (JavaScript numbers written as f32)
  p->bodies = h->bodies;
  p->body_acc = h->body_acc;
  p->nbodies = h->nbodies;
  p->body_mask = h->body_mask;
  for (int a = 0; a < 3; a++) p->origin[a] = (float)h->origin[a];
  p->dx = (float)h->dx;
  p->inv_dx = (float)(1.0 / h->dx);
  p->vel_to_lattice = (float)(h->dt / h->dx);
  p->friction = (float)h->friction;
  p->band = (float)h->band;
}

// The event guarding a staging slot: wait for the copy that last used it, or create it.
static int stage_slot_ready(cudaEvent_t& ev) {
  if (ev) CK(cudaEventSynchronize(ev));
  else CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  return SI_OK;
}

// Host-to-device copy through a pinned staging buffer of the world (see si_world::stage).
static int stage_upload(si_world* w, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return SI_OK;
  const int slot = w->stage_next;
  w->stage_next = (slot + 1) % si_world::kStageSlots;
  int r = stage_slot_ready(w->stage_ev[slot]);
  if (r) return r;
  if (w->stage_cap[slot] < bytes) {
    if (w->stage[slot]) CK(cudaFreeHost(w->stage[slot]));
    w->stage[slot] = nullptr;
    w->stage_cap[slot] = 0;
    const size_t cap = std::max<size_t>(std::max<size_t>(bytes, 4096), 2 * w->stage_cap[slot]);
    CK(cudaHostAlloc(&w->stage[slot], cap, cudaHostAllocDefault));
    w->stage_cap[slot] = cap;
  }
  std::memcpy(w->stage[slot], src, bytes);
  CK(cudaMemcpyAsync(dst, w->stage[slot], bytes, cudaMemcpyHostToDevice, w->st));
  CK(cudaEventRecord(w->stage_ev[slot], w->st));
  return SI_OK;
}

static int upload_params(si_mpm* h) {
  if (!h->prm_dirty) return SI_OK;
  si_world* w = h->w;
  if (!w->prm_ring) CK(cudaHostAlloc((void**)&w->prm_ring, sizeof(SceneParams) * si_world::kPrmSlots, cudaHostAllocDefault));
  const int slot = w->prm_next;
  w->prm_next = (slot + 1) % si_world::kPrmSlots;
  int r = stage_slot_ready(w->prm_ev[slot]);
  if (r) return r;
  SceneParams* p = w->prm_ring + slot;
  build_params(h, p);
  CK(cudaMemcpyAsync(h->prm, p, sizeof(*p), cudaMemcpyHostToDevice, w->st));
  CK(cudaEventRecord(w->prm_ev[slot], w->st));
  h->prm_dirty = false;
  return SI_OK;
}

static void invalidate(si_mpm* h) {
  if (h->pending) h->next_clear = false;
  h->pending = false;
  h->keys_valid = false;
  h->box_ok = 0;
}

// ------------------------------------------------------------------ ticks
enum TickMode { T_SUBSTEP = 0, T_P2G = 1, T_GRID = 2, T_G2P = 3, T_SORT = 4 };

struct HostTick {
  int mode = T_SUBSTEP;
  std::vector<TickScene> ts;
  std::vector<uint32_t> nb, nck, nct;   // per entry: num_blocks, node chunks, coupling tiles (host side)
  std::vector<int64_t> nodes;           // per entry: grid nodes
  uint32_t pchunks = 0, nchunks = 0, cchunks = 0;
  bool any_p2g = false, any_clear = false, any_gather = false, any_keys_now = false, any_pregather = false;
  uint32_t sort_n = 0, sort_bins = 0, max_blocks = 0;
  int passes = 0;
  uint32_t sentinel = 0;   // segmented sort: the key that pads each scene's segment to whole tiles
};

static TickScene base_entry(si_mpm* h) {
  TickScene t;
  std::memset(&t, 0, sizeof(t));
  t.prm = h->prm;
  t.P = h->pbuf[h->pcur];
  t.Palt = h->compact ? h->pbuf[0] : h->pbuf[1 - h->pcur];
  t.keys = h->keys[h->kpend];
  t.keys_next = h->keys[h->kpend];
  t.starts = h->starts;
  t.cap = h->cap;
  t.n = (int32_t)h->count;
  return t;
}

static void finish_tick(si_world* w, HostTick& k) {
  // Nodes per work item of the grid kernels: kNodeChunk, halved (down to one node per thread) while
  // the whole tick has fewer than 128 items, so that a small scene's grid is spread over many CTAs
  // instead of a few threads walking many nodes one after another (a tick of many scenes has items
  // enough at the full size).
  int64_t all_nodes = 0;
  for (int64_t n : k.nodes) all_nodes += n;
  int32_t node_chunk = kNodeChunk;
  while (node_chunk > kCtaThreads && all_nodes / node_chunk < 128) node_chunk /= 2;
  k.nck.clear();
  for (size_t e = 0; e < k.ts.size(); e++) {
    k.ts[e].node_chunk = node_chunk;
    k.nck.push_back((uint32_t)((k.nodes[e] + node_chunk - 1) / node_chunk));
  }
  uint32_t pc = 0, nc = 0, cc = 0, seg = 0, bin = 0;
  const uint32_t chunk = (uint32_t)(kCtaThreads * w->ppt);
  // One sorting scene with its own keys is sorted in place of the concatenation (its keys feed the
  // first pass directly); otherwise the sort is segmented: each sorting scene keeps its own block keys,
  // its segment starts on a tile boundary and is padded to whole tiles, and the passes cover the
  // largest scene's keys rather than the tick's total bins.
  int sorting = 0;
  bool any_from_x = false;
  for (const TickScene& t : k.ts)
    if (t.flags & F_GATHER) { sorting++; if (t.flags & F_KEYS_FROM_X) any_from_x = true; }
  const bool segmented = sorting > 1 || any_from_x;
  for (size_t e = 0; e < k.ts.size(); e++) {
    TickScene& t = k.ts[e];
    t.pchunk_begin = pc;
    t.nchunk_begin = nc;
    t.cchunk_begin = cc;
    cc += k.nct[e];
    pc += (uint32_t)((t.n + chunk - 1) / chunk);
    if (t.flags & F_P2G) k.any_p2g = true;
    if (t.flags & F_CLEAR) k.any_clear = true;
    if (t.flags & F_KEYS_NOW) k.any_keys_now = true;
    if (t.flags & F_PREGATHER) k.any_pregather = true;
    t.seg_base = seg;   // a scene that does not sort sits at the running end with no slots
    if (t.flags & F_GATHER) {
      k.any_gather = true;
      t.bin_base = segmented ? 0u : bin;
      seg += segmented ? (((uint32_t)t.n + kSortTile - 1) / kSortTile) * kSortTile : (uint32_t)t.n;
      bin += k.nb[e];
      k.max_blocks = std::max(k.max_blocks, k.nb[e]);
    }
    nc += k.nck[e];
  }
  k.pchunks = pc;
  k.nchunks = nc;
  k.cchunks = cc;
  k.sort_n = seg;
  k.sort_bins = bin;
  // key range: the tick's bins, or (segmented) the largest scene's bins plus the sentinel above them
  const uint64_t range = segmented ? (uint64_t)k.max_blocks + 1 : std::max<uint32_t>(bin, 2u);
  int bits = 1;
  while (bits < 32 && (1ull << bits) < range) bits++;
  k.passes = (bits + kRadixBits - 1) / kRadixBits;
  k.sentinel = segmented ? (k.passes * kRadixBits >= 32 ? 0xffffffffu : (1u << (k.passes * kRadixBits)) - 1u) : 0u;
}

static void push_entry(HostTick& k, const si_mpm* h, const TickScene& t) {
  k.ts.push_back(t);
  k.nb.push_back(h->num_blocks);
  k.nodes.push_back(h->nodes);
  k.nct.push_back((t.flags & F_COUPLE) ? (uint32_t)(((h->dims[0] + 3) / 4) * ((h->dims[1] + 3) / 4) * ((h->dims[2] + 3) / 4)) : 0u);
}

static TickScene substep_entry(si_mpm* h) {
  TickScene t = base_entry(h);
  t.grid = h->grid[1 - h->gcur];
  t.grid_next = h->grid[h->gcur];
  t.box_cur = h->box + 8 * (1 - h->gcur);
  t.box_next = h->box + 8 * h->gcur;
  const bool sort_now = h->sort_every > 0 && h->step_count % h->sort_every == 0;
  const bool next_sort = h->sort_every > 0 && (h->step_count + 1) % h->sort_every == 0;
  uint32_t f = F_FUSE;
  if (h->w->flush) f |= F_FORCE_GLOBAL;
  if (!h->pending) { f |= F_P2G; if (!h->next_clear) f |= F_CLEAR; }
  if (sort_now) {
    f |= F_GATHER;
    if (h->compact) f |= F_PREGATHER | F_KEYS_FROM_X;   // no key buffers: the sort keys the positions itself
    else if (!h->keys_valid) f |= F_KEYS_NOW;
  }
  if (next_sort && !h->compact) f |= F_KEYS;
  if (sort_now) t.keys_next = h->keys[1 - h->kpend];   // the sort consumes keys[kpend]
  // both boxes are exact once two standard substeps ran in a row: box_cur from the P2G that filled
  // `grid` (the previous G2P, or the standalone P2G of a substep that started after box_ok was
  // reset), box_next from the one before, whose grid update left values only inside it
  if (h->box_ok >= 2) f |= F_BOXED;
  if (h->nbodies > 0) {   // coupling.substep(s) after the grid update, mpm.js:596; lead = (s + 0.5) dt
    f |= F_COUPLE;
    t.lead = (float)((h->frame_sub + 0.5) * h->dt);
  }
  h->frame_sub++;
  t.flags = f;
  // state after the substep
  h->gcur = 1 - h->gcur;
  if (sort_now) { if (!h->compact) h->pcur = 1 - h->pcur; h->kpend = 1 - h->kpend; }
  h->pending = true;
  h->next_clear = false;
  h->keys_valid = next_sort;
  h->step_count++;
  h->box_ok = std::min(h->box_ok + 1, 2);
  return t;
}

static int ensure_sort_scratch(si_world* w, uint32_t n, uint32_t scenes) {
  const size_t need = (size_t)std::max<uint32_t>(n, 1u) * 4;
  if (need > w->sort_cap) {
    size_t cap = std::max(need, w->sort_cap + w->sort_cap / 2);
    for (uint32_t** p : {&w->ka, &w->va, &w->kb, &w->vb}) {
      if (*p) CK(cudaFreeAsync(*p, w->st));
      *p = nullptr;
      CK(cudaMallocAsync((void**)p, cap, w->st));
    }
    w->sort_cap = cap;
    world_free_graphs(w);
  }
  const size_t tiles = (std::max<uint32_t>(n, 1u) + kSortTile - 1) / kSortTile;
  size_t hcap = w->hist_cap;
  void* hp = w->hist;
  if (256 * tiles * 4 > hcap) {
    int r = ensure_dev(w, &hp, &hcap, 256 * tiles * 4);
    if (r) return r;
    w->hist = (uint32_t*)hp;
    w->hist_cap = hcap;
    world_free_graphs(w);
  }
  if (!w->digit_total) CK(cudaMallocAsync((void**)&w->digit_total, 256 * 4, w->st));
  // segmented sort: the scene of every tile, and every scene's digit totals of the current pass
  const size_t need_ts = tiles * 4, need_st = (size_t)std::max<uint32_t>(scenes, 1u) * 256 * 4;
  if (need_ts > w->tile_scene_cap) {
    void* q = w->tile_scene;
    int r = ensure_dev(w, &q, &w->tile_scene_cap, need_ts);
    if (r) return r;
    w->tile_scene = (uint32_t*)q;
    world_free_graphs(w);
  }
  if (need_st > w->seg_total_cap) {
    void* q = w->seg_total;
    int r = ensure_dev(w, &q, &w->seg_total_cap, need_st);
    if (r) return r;
    w->seg_total = (uint32_t*)q;
    world_free_graphs(w);
  }
  return SI_OK;
}

// The one scene a tick sorts, if it sorts exactly one and that one sits at segment and bin 0: its
// keys feed the first radix pass directly.
static const TickScene* single_sort_scene(const HostTick& k) {
  const TickScene* only = nullptr;
  int sorting = 0;
  for (const TickScene& e : k.ts)
    if (e.flags & F_GATHER) { sorting++; only = &e; }
  return (sorting == 1 && only->seg_base == 0 && only->bin_base == 0 && !(only->flags & F_KEYS_FROM_X)) ? only
                                                                                                   : nullptr;
}

static int64_t tick_kernels(const HostTick& k) {
  int64_t n = 0;
  if (k.any_keys_now) n++;
  if (k.any_gather && k.sort_n)
    n += small_sort_ok(k.sort_n, k.sort_bins, single_sort_scene(k) != nullptr)
             ? 1 + (k.mode == T_SORT ? 1 : 0)
             : (single_sort_scene(k) ? 1 : 2) + 3 * k.passes + (k.mode == T_SORT ? 1 : 0);
  if (k.any_pregather) n++;
  if (k.any_clear) n++;
  if (k.any_p2g) n++;
  if ((k.mode == T_SUBSTEP || k.mode == T_GRID) && k.nchunks) n++;
  if (k.mode == T_SUBSTEP && !k.nchunks) n++;   // box reset by its own kernel when k_grid does not run
  if (k.cchunks) n++;
  if (k.mode == T_SUBSTEP || k.mode == T_G2P) n++;
  return n;
}

static void enqueue_tick(si_world* w, const HostTick& k, const TickScene* dev_table, bool profile) {
  TickInfo t;
  t.ts = dev_table;
  t.nscenes = (int32_t)k.ts.size();
  t.pchunks = k.pchunks;
  t.nchunks = k.nchunks;
  t.cchunks = k.cchunks;
  t.chunk = kCtaThreads * w->ppt;
  t.tile_nodes = w->tile_nodes;
  t.nz = -0.0f;
  t.grid_done = w->grid_done;
  t.g2p_sched = w->grid_done + 1;
  t.gscratch = w->gscratch;
  t.gstride = (int64_t)w->gscratch_cap;
  t.reset_boxes = (k.mode == T_SUBSTEP && k.nchunks > 0) ? 1 : 0;   // else k_box_reset below
  cudaStream_t st = w->st;
  if (profile) cudaEventRecord(w->pev[0], st);
  const uint32_t* perm = nullptr;
  const uint32_t* skeys = nullptr;
  if (k.any_keys_now) launch_keys(t, w->ctas_misc, st);
  if (k.any_gather) {
    SortInfo s;
    s.n = k.sort_n; s.bins = k.sort_bins; s.passes = k.passes;
    s.keys_a = w->ka; s.vals_a = w->va; s.keys_b = w->kb; s.vals_b = w->vb;
    s.hist = w->hist; s.digit_total = w->digit_total;
    s.tile_scene = w->tile_scene; s.seg_total = w->seg_total; s.sentinel = k.sentinel;
    const TickScene* only = single_sort_scene(k);
    s.keys_in = only ? only->keys : nullptr;
    s.starts_out = only ? only->starts : nullptr;
    if (!launch_sort(t, s, &perm, &skeys, w->ctas_misc, st)) launch_scene_starts_all(t, skeys, k.max_blocks, st);
    if (k.mode == T_SORT) launch_reorder(t, perm, w->ctas_misc, st);
    if (k.any_pregather) launch_pregather(t, perm, w->gscratch, (int64_t)w->gscratch_cap, w->ctas_misc, st);
  }
  if (profile) cudaEventRecord(w->pev[1], st);
  if (k.any_clear) launch_clear(t, w->ctas_grid, st);
  if (k.any_p2g) launch_p2g(t, w->ctas_p2g, st);
  if (profile) cudaEventRecord(w->pev[2], st);
  if (k.mode == T_SUBSTEP || k.mode == T_GRID) launch_grid(t, w->ctas_grid, w->ctas_grid_wide, st);
  if (k.cchunks) launch_couple(t, w->ctas_couple, st);
  if (k.mode == T_SUBSTEP && !t.reset_boxes) launch_box_reset(t, st);   // box_next starts empty for the fused P2G
  if (profile) cudaEventRecord(w->pev[3], st);
  if (k.mode == T_SUBSTEP || k.mode == T_G2P) launch_g2p(t, perm, w->ctas_g2p, st, k.any_pregather, w->svd_tolerance);
  if (profile) {
    cudaEventRecord(w->pev[4], st);
    cudaEventSynchronize(w->pev[4]);
    for (int i = 0; i < 4; i++) {
      float ms = 0;
      cudaEventElapsedTime(&ms, w->pev[i], w->pev[i + 1]);
      w->prof_ms[i] += ms;
    }
  }
}

static size_t table_bytes(const std::vector<HostTick>& plan) {
  size_t n = 0;
  for (const HostTick& k : plan) n += k.ts.size();
  return n * sizeof(TickScene);
}

static bool same_plan(const GraphPlan& g, const std::vector<HostTick>& plan, const std::vector<uint8_t>& bytes,
                      const si_world* w) {
  if (g.bytes != bytes || g.ppt != w->ppt || g.tile_nodes != w->tile_nodes || g.ticks.size() != plan.size())
    return false;
  for (size_t i = 0; i < plan.size(); i++) {
    const HostTick& a = plan[i];
    const GraphTick& b = g.ticks[i];
    if (a.mode != b.mode || a.pchunks != b.pchunks || a.nchunks != b.nchunks || a.cchunks != b.cchunks || a.any_p2g != b.any_p2g ||
        a.any_clear != b.any_clear || a.any_gather != b.any_gather || a.any_keys_now != b.any_keys_now ||
        a.sort_n != b.sort_n || a.passes != b.passes)
      return false;
  }
  return true;
}

static int run_plan(si_world* w, std::vector<HostTick>& plan) {
  if (plan.empty()) return SI_OK;
  uint32_t max_sort = 0, max_pre = 0, max_scenes = 0;
  for (const HostTick& k : plan) {
    max_sort = std::max(max_sort, k.sort_n);
    max_scenes = std::max(max_scenes, (uint32_t)k.ts.size());
    if (k.any_pregather) max_pre = std::max(max_pre, k.sort_n);
  }
  int r = ensure_sort_scratch(w, max_sort, max_scenes);
  if (r) return r;
  if (max_pre > w->gscratch_cap) {   // the pregather scratch, grown like the sort's (graphs hold its address)
    if (w->gscratch) CK(cudaFreeAsync(w->gscratch, w->st));
    w->gscratch = nullptr;
    const size_t cap = std::max<size_t>(max_pre, w->gscratch_cap + w->gscratch_cap / 2);
    CK(cudaMallocAsync((void**)&w->gscratch, cap * 16 * kPregatherStreams, w->st));
    w->gscratch_cap = cap;
    world_free_graphs(w);
  }
  std::vector<uint8_t> bytes(table_bytes(plan));
  {
    size_t off = 0;
    for (const HostTick& k : plan) {
      std::memcpy(bytes.data() + off, k.ts.data(), k.ts.size() * sizeof(TickScene));
      off += k.ts.size() * sizeof(TickScene);
    }
  }
  bool graph_ok = w->use_graphs && !w->profile;
  if (graph_ok) {
    for (auto& g : w->graphs) {
      if (same_plan(*g, plan, bytes, w)) {
        g->last_use = ++w->graph_clock;
        CK(cudaGraphLaunch(g->exec, w->st));
        w->launches += g->kernels;
        return SI_OK;
      }
    }
    // A plan is captured the second time it is seen; one that does not repeat (a serving round
    // over a changing set of scenes) runs as direct launches and pays no capture.
    uint64_t hsh = 1469598103934665603ull;
    for (uint8_t b : bytes) hsh = (hsh ^ b) * 1099511628211ull;
    hsh ^= ((uint64_t)w->ppt << 48) ^ ((uint64_t)plan.size() << 32) ^ (uint64_t)w->tile_nodes;
    bool repeat = false;
    for (uint64_t s : w->seen) repeat |= (s == hsh);
    if (!repeat) {
      w->seen[w->seen_next] = hsh;
      w->seen_next = (w->seen_next + 1) % 16;
      graph_ok = false;
    }
  }
  if (graph_ok) {
    auto g = std::make_unique<GraphPlan>();
    CK(cudaMalloc((void**)&g->table, std::max<size_t>(bytes.size(), 16)));
    r = stage_upload(w, g->table, bytes.data(), bytes.size());
    if (r) return r;
    CK(cudaStreamBeginCapture(w->st, cudaStreamCaptureModeThreadLocal));
    size_t off = 0;
    for (const HostTick& k : plan) {
      enqueue_tick(w, k, reinterpret_cast<const TickScene*>(reinterpret_cast<uint8_t*>(g->table) + off), false);
      off += k.ts.size() * sizeof(TickScene);
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(w->st, &graph);
    if (e != cudaSuccess) return si_fail(SI_EDEVICE, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return si_fail(SI_EDEVICE, std::string("graph instantiate: ") + cudaGetErrorString(e));
    g->bytes = std::move(bytes);
    g->ppt = w->ppt;
    g->tile_nodes = w->tile_nodes;
    for (const HostTick& k : plan) {
      GraphTick t;
      t.mode = k.mode; t.pchunks = k.pchunks; t.nchunks = k.nchunks; t.cchunks = k.cchunks; t.any_p2g = k.any_p2g;
      t.any_clear = k.any_clear; t.any_gather = k.any_gather; t.any_keys_now = k.any_keys_now;
      t.sort_n = k.sort_n; t.passes = k.passes;
      g->ticks.push_back(t);
    }
    for (const HostTick& k : plan) g->kernels += tick_kernels(k);
    g->last_use = ++w->graph_clock;
    CK(cudaGraphLaunch(g->exec, w->st));
    w->launches += g->kernels;
    if (w->graphs.size() >= 8) {
      auto it = std::min_element(w->graphs.begin(), w->graphs.end(),
                                 [](const std::unique_ptr<GraphPlan>& a, const std::unique_ptr<GraphPlan>& b) {
                                   return a->last_use < b->last_use;
                                 });
      cudaStreamSynchronize(w->st);
      w->graphs.erase(it);
    }
    w->graphs.push_back(std::move(g));
    return SI_OK;
  }
  void* tab = w->tab;
  size_t cap = w->tab_cap;
  r = ensure_dev(w, &tab, &cap, std::max<size_t>(bytes.size(), 16));
  if (r) return r;
  w->tab = (TickScene*)tab;
  w->tab_cap = cap;
  r = stage_upload(w, w->tab, bytes.data(), bytes.size());
  if (r) return r;
  size_t off = 0;
  for (const HostTick& k : plan) {
    enqueue_tick(w, k, reinterpret_cast<const TickScene*>(reinterpret_cast<uint8_t*>(w->tab) + off), w->profile);
    w->launches += tick_kernels(k);
    off += k.ts.size() * sizeof(TickScene);
  }
  CK(cudaGetLastError());
  return SI_OK;
}

// K substeps of the given scenes in lockstep: one plan of K ticks.
int run_substeps(si_world* w, const std::vector<si_mpm*>& scenes, int K) {
  std::vector<si_mpm*> act;
  for (si_mpm* h : scenes)
    if (!h->destroyed && h->count > 0) act.push_back(h);
  if (act.empty() || K <= 0) return SI_OK;
  for (si_mpm* h : act) {
    int r = upload_params(h);
    if (r) return r;
  }
  std::vector<HostTick> plan;
  plan.reserve(K);
  for (int s = 0; s < K; s++) {
    // Scenes are independent, so a tick may run as several groups of scenes, one after another. A
    // compact world splits a tick whose sorting particles exceed group_particles, which bounds the
    // sort and pregather scratch; every scene's substep is the same in any group.
    HostTick k;
    k.mode = T_SUBSTEP;
    int64_t sorting = 0;
    for (si_mpm* h : act) {
      const bool sorts = h->sort_every > 0 && h->step_count % h->sort_every == 0;
      const int64_t slots = (h->count + kSortTile - 1) / kSortTile * kSortTile;   // its padded segment
      if (sorts && w->group_particles > 0 && sorting > 0 && sorting + slots > w->group_particles) {
        finish_tick(w, k);
        plan.push_back(std::move(k));
        k = HostTick();
        k.mode = T_SUBSTEP;
        sorting = 0;
      }
      if (sorts) sorting += slots;
      push_entry(k, h, substep_entry(h));
    }
    finish_tick(w, k);
    plan.push_back(std::move(k));
  }
  return run_plan(w, plan);
}

static int run_phase(si_mpm* h, int mode, uint32_t extra_flags) {
  si_world* w = h->w;
  int r = upload_params(h);
  if (r) return r;
  if (h->count == 0 && mode != T_P2G) return SI_OK;
  HostTick k;
  k.mode = mode;
  TickScene t = base_entry(h);
  t.grid = h->grid[h->gcur];
  t.grid_next = h->grid[1 - h->gcur];
  t.box_cur = h->box + 8 * h->gcur;
  t.box_next = h->box + 8 * (1 - h->gcur);
  h->box_ok = 0;   // a phase run by itself leaves the arrays as the reference does: the next substeps
                   // visit the whole grid until both boxes are known again
  switch (mode) {
    case T_P2G: t.flags = F_P2G | F_CLEAR | extra_flags; break;
    case T_GRID: t.flags = F_NO_CLEAR_NEXT; break;
    case T_G2P: t.flags = 0; break;
    case T_SORT: t.flags = F_GATHER | (h->compact ? F_KEYS_FROM_X : (h->keys_valid ? 0u : F_KEYS_NOW)); break;
  }
  float4* fresh = nullptr;   // a compact scene's explicit sort reorders into a new buffer, then frees the old
  if (mode == T_SORT && h->compact) {
    CK(cudaMallocAsync((void**)&fresh, std::max<size_t>((size_t)kStreams * 16 * (size_t)h->cap, 16), w->st));
    t.Palt = fresh;
  }
  push_entry(k, h, t);
  finish_tick(w, k);
  std::vector<HostTick> plan;
  plan.push_back(std::move(k));
  const bool g = w->use_graphs;
  w->use_graphs = false;   // one-off phases are not worth a graph
  r = run_plan(w, plan);
  w->use_graphs = g;
  if (r) {
    if (fresh) cudaFreeAsync(fresh, w->st);
    return r;
  }
  if (mode == T_G2P) invalidate(h);
  if (mode == T_SORT) {
    if (h->compact) {
      CK(cudaFreeAsync(h->pbuf[0], w->st));
      h->pbuf[0] = fresh;
    } else {
      h->pcur = 1 - h->pcur;
    }
    h->kpend = 1 - h->kpend;
    h->keys_valid = false;
  }
  return SI_OK;
}

// ------------------------------------------------------------------ C ABI
// Every entry point holds the world's lock for its whole body: calls on one world from several
// threads (and a server's rounds) are serialised.
#define GUARD_WORLD(w)                                                                    \
  if (!(w)) return si_fail(SI_EINVAL, "null world");                                     \
  std::lock_guard<std::recursive_mutex> guard_((w)->api_mu);                              \
  if ((w)->destroyed) return si_fail(SI_EDESTROYED, "the world was destroyed")
#define GUARD(h)                                                                          \
  if (!(h)) return si_fail(SI_EINVAL, "null MPM handle");                                \
  GUARD_WORLD((h)->w);                                                                    \
  if ((h)->destroyed) return si_fail(SI_EDESTROYED, "MPM: it was destroyed")

extern "C" {

const char* si_last_error(void) { return t_err.c_str(); }
const char* si_version(void) { return "si_cuda 0.1.0 (sm_103a)"; }

int si_world_create(si_world** out) {
  if (!out) return si_fail(SI_EINVAL, "null out");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return si_fail(SI_EDEVICE, "no CUDA device");
  }
  auto* w = new si_world();
  int r = world_init(w);
  if (r) { delete w; return r; }
  *out = w;
  return SI_OK;
}

static void scene_release(si_mpm* h) {
  if (h->destroyed) return;
  si_world* w = h->w;
  h->destroyed = true;
  for (void* p : {(void*)h->pbuf[0], (void*)h->pbuf[1], (void*)h->grid[0], (void*)h->grid[1], (void*)h->keys[0],
                  (void*)h->keys[1],
                  (void*)h->starts, (void*)h->prm, (void*)h->box, (void*)h->bodies, (void*)h->body_acc})
    if (p) cudaFreeAsync(p, w->st);
  h->bodies = nullptr;
  h->body_acc = nullptr;
  h->nbodies = 0;
  h->pbuf[0] = h->pbuf[1] = nullptr;
  h->grid[0] = h->grid[1] = nullptr;
  h->keys[0] = h->keys[1] = h->starts = nullptr;
  h->prm = nullptr;
  h->box = nullptr;
  w->scenes.erase(std::remove(w->scenes.begin(), w->scenes.end(), h), w->scenes.end());
  world_free_graphs(w);
}

int si_world_destroy(si_world* w) {
  if (!w) return si_fail(SI_EINVAL, "null world");
  std::lock_guard<std::recursive_mutex> g(w->api_mu);
  if (w->destroyed) return SI_OK;
  if (w->server) return si_fail(SI_EBUSY, "destroy the server first");
  std::vector<si_mpm*> sc = w->scenes;
  for (si_mpm* h : sc) scene_release(h);
  world_free_graphs(w);
  for (void* p : {(void*)w->ka, (void*)w->va, (void*)w->kb, (void*)w->vb, (void*)w->hist, (void*)w->digit_total,
                  (void*)w->tile_scene, (void*)w->seg_total, (void*)w->tab, (void*)w->grid_done, (void*)w->gscratch})
    if (p) cudaFreeAsync(p, w->st);
  cudaStreamSynchronize(w->st);
  for (auto& e : w->pev) if (e) cudaEventDestroy(e);
  for (auto& e : w->marks) if (e) cudaEventDestroy(e);
  if (w->st_copy) {
    cudaStreamSynchronize(w->st_copy);
    cudaStreamDestroy(w->st_copy);
    w->st_copy = nullptr;
  }
  for (auto& kv : w->reads) cudaEventDestroy(kv.second);
  w->reads.clear();
  for (auto& e : w->prm_ev) if (e) cudaEventDestroy(e);
  for (auto& e : w->stage_ev) if (e) cudaEventDestroy(e);
  if (w->prm_ring) cudaFreeHost(w->prm_ring);
  w->prm_ring = nullptr;
  for (int i = 0; i < si_world::kStageSlots; i++)
    if (w->stage[i]) { cudaFreeHost(w->stage[i]); w->stage[i] = nullptr; }
  cudaStreamDestroy(w->st);
  w->destroyed = true;
  return SI_OK;
}

int si_world_step(si_world* w, int32_t K) {
  GUARD_WORLD(w);
  if (K <= 0) return si_fail(SI_EINVAL, "si_world_step: K must be > 0");
  for (si_mpm* h : w->scenes) h->frame_sub = 0;
  return run_substeps(w, w->scenes, K);
}

int si_world_sync(si_world* w) {
  GUARD_WORLD(w);
  CK(cudaStreamSynchronize(w->st));
  CK(cudaGetLastError());
  return SI_OK;
}

int si_world_set_svd_tolerance(si_world* w, int32_t enable) {
  GUARD_WORLD(w);
  if (w->svd_tolerance != (enable != 0)) {
    world_free_graphs(w);   // captured plans hold the kernel variant
    w->svd_tolerance = enable != 0;
  }
  return SI_OK;
}

int si_world_set_graphs(si_world* w, int32_t enable) {
  GUARD_WORLD(w);
  w->use_graphs = enable != 0;
  if (!w->use_graphs) world_free_graphs(w);
  return SI_OK;
}

int si_world_profile(si_world* w, int32_t enable, double ms_out[4], int32_t reset) {
  GUARD_WORLD(w);
  if (ms_out) for (int i = 0; i < 4; i++) ms_out[i] = w->prof_ms[i];
  if (reset) for (double& x : w->prof_ms) x = 0;
  w->profile = enable != 0;
  return SI_OK;
}

int si_world_set_tuning(si_world* w, int32_t particles_per_cta, int32_t tile_nodes, int32_t flush) {
  GUARD_WORLD(w);
  if (particles_per_cta % kCtaThreads) return si_fail(SI_EINVAL, "particles per CTA must be a multiple of 256");
  if (flush != 0 && flush != 1) return si_fail(SI_EINVAL, "flush strategy must be 0 (shared tile) or 1 (global)");
  CK(cudaStreamSynchronize(w->st));
  int r = world_configure(w, particles_per_cta / kCtaThreads, tile_nodes);
  if (!r) w->flush = flush;
  return r;
}

int si_world_mark(si_world* w, int32_t slot) {
  GUARD_WORLD(w);
  if (slot < 0 || slot >= 8) return si_fail(SI_EINVAL, "mark slot must be 0..7");
  CK(cudaEventRecord(w->marks[slot], w->st));
  return SI_OK;
}

int si_world_elapsed(si_world* w, int32_t a, int32_t b, double* ms) {
  GUARD_WORLD(w);
  if (a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) return si_fail(SI_EINVAL, "bad mark slots");
  CK(cudaEventSynchronize(w->marks[b]));
  float f = 0;
  CK(cudaEventElapsedTime(&f, w->marks[a], w->marks[b]));
  *ms = f;
  return SI_OK;
}

int si_world_launches(si_world* w, int64_t* count) {
  GUARD_WORLD(w);
  if (!count) return si_fail(SI_EINVAL, "null count");
  *count = w->launches;
  return SI_OK;
}

void si_mpm_desc_default(si_mpm_desc* d) {
  if (!d) return;
  d->max_particles = 262144;
  d->grid = 64;
  d->sort_every = 4;
  d->substeps = 8;
  d->ppc_axis = 2;
  for (int a = 0; a < 3; a++) { d->size[a] = 1.0; d->origin[a] = 0.0; d->gravity[a] = 0.0; }
  d->gravity[1] = -9.81;
  d->time_scale = 1.0;
}

}  // extern "C"

int scene_create(si_world* w, const si_mpm_desc* in, si_mpm** out, bool own_world) {
  si_mpm_desc d;
  si_mpm_desc_default(&d);
  if (in) {
    if (in->max_particles > 0) d.max_particles = in->max_particles;
    if (in->grid > 0) d.grid = in->grid;
    if (in->sort_every > 0) d.sort_every = in->sort_every;
    if (in->substeps > 0) d.substeps = in->substeps;
    if (in->ppc_axis > 0) d.ppc_axis = in->ppc_axis;
    bool size_set = in->size[0] > 0 || in->size[1] > 0 || in->size[2] > 0;
    for (int a = 0; a < 3; a++) {
      if (size_set) d.size[a] = in->size[a];
      d.origin[a] = in->origin[a];
      d.gravity[a] = in->gravity[a];
    }
    if (!std::isnan(in->time_scale)) d.time_scale = in->time_scale;
  }
  if (d.max_particles > 0x7fffffff - 4096) return si_fail(SI_EINVAL, "max_particles must be < 2^31");
  for (int a = 0; a < 3; a++)
    if (!(d.size[a] > 0)) return si_fail(SI_EINVAL, "MPM: size must be positive");
  auto* h = new si_mpm();
  h->w = w;
  h->own_world = own_world;
  h->cap = d.max_particles;
  h->dx = std::max(d.size[0], std::max(d.size[1], d.size[2])) / d.grid;
  for (int a = 0; a < 3; a++) {
    h->dims[a] = (int32_t)std::max(8.0, js_round(d.size[a] / h->dx));
    h->size[a] = h->dims[a] * h->dx;
    h->origin[a] = d.origin[a];
    h->gravity[a] = d.gravity[a];
  }
  h->substeps = std::max(1, (int)js_round(d.substeps));
  h->time_scale = d.time_scale;
  h->sort_every = d.sort_every;
  h->ppc_axis = d.ppc_axis;
  h->dt = 1.0 / 60 * h->time_scale / h->substeps;   // mpm.js:109
  h->nodes = (int64_t)h->dims[0] * h->dims[1] * h->dims[2];
  if (h->nodes * 4 > 0x7fffffffLL) { delete h; return si_fail(SI_EINVAL, "grid too large"); }
  h->num_blocks = num_blocks_for(h->dims);
  h->compact = w->compact;
  h->device_bytes = scene_footprint(h->cap, h->nodes, h->num_blocks, h->compact);
  cudaStream_t st = w->st;
  const size_t pbytes = (size_t)kStreams * 16 * (size_t)h->cap;
  cudaError_t e = cudaSuccess;
  for (int b = 0; b < (h->compact ? 1 : 2) && e == cudaSuccess; b++)
    e = cudaMallocAsync((void**)&h->pbuf[b], std::max<size_t>(pbytes, 16), st);
  for (int b = 0; b < 2 && e == cudaSuccess; b++) e = cudaMallocAsync((void**)&h->grid[b], (size_t)h->nodes * 16, st);
  for (int b = 0; b < (h->compact ? 0 : 2) && e == cudaSuccess; b++)   // a compact scene keeps no keys
    e = cudaMallocAsync((void**)&h->keys[b], std::max<size_t>(4 * (size_t)h->cap, 16), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&h->starts, 4 * ((size_t)h->num_blocks + 1), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&h->prm, sizeof(SceneParams), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&h->box, 64, st);
  if (e == cudaSuccess) {
    static const int32_t empty[16] = {0x3fffffff, 0x3fffffff, 0x3fffffff, -0x3fffffff, -0x3fffffff, -0x3fffffff, 0, 0,
                                      0x3fffffff, 0x3fffffff, 0x3fffffff, -0x3fffffff, -0x3fffffff, -0x3fffffff, 0, 0};
    e = cudaMemcpyAsync(h->box, empty, sizeof(empty), cudaMemcpyHostToDevice, st);
  }
  for (int b = 0; b < 2 && e == cudaSuccess; b++) e = cudaMemsetAsync(h->grid[b], 0, (size_t)h->nodes * 16, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->starts, 0, 4 * ((size_t)h->num_blocks + 1), st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    w->scenes.push_back(h);
    scene_release(h);
    delete h;
    return si_fail(e == cudaErrorMemoryAllocation ? SI_ENOMEM : SI_EDEVICE,
                   std::string("MPM: device allocation failed: ") + cudaGetErrorString(e));
  }
  h->next_clear = true;
  h->prm_dirty = true;
  w->scenes.push_back(h);
  world_free_graphs(w);
  *out = h;
  return SI_OK;
}

extern "C" {

int si_mpm_create(si_world* world, const si_mpm_desc* desc, si_mpm** out) {
  if (!out) return si_fail(SI_EINVAL, "null out");
  *out = nullptr;
  bool own = false;
  if (!world) {
    int r = si_world_create(&world);
    if (r) return r;
    own = true;
  }
  std::unique_lock<std::recursive_mutex> g(world->api_mu);
  if (world->destroyed) return si_fail(SI_EDESTROYED, "the world was destroyed");
  int r = scene_create(world, desc, out, own);
  g.unlock();
  if (r && own) { si_world_destroy(world); delete world; }
  return r;
}

int si_mpm_destroy(si_mpm* h) {
  if (!h) return si_fail(SI_EINVAL, "null MPM handle");
  {
    std::lock_guard<std::recursive_mutex> g(h->w->api_mu);
    if (h->destroyed) return SI_OK;
    if (h->served && h->w->server) return si_fail(SI_EBUSY, "MPM: a served scene is retired by si_server_retire");
    scene_release(h);
  }
  if (h->own_world) si_world_destroy(h->w);
  return SI_OK;
}

void si_mpm_free(si_mpm* h) {
  if (!h) return;
  if (!h->destroyed) si_mpm_destroy(h);
  if (!h->destroyed) return;   // still resident in a running server
  if (h->own_world) delete h->w;
  delete h;
}

int si_mpm_get_info(const si_mpm* h, si_mpm_info* o) {
  if (!h || !o) return si_fail(SI_EINVAL, "null argument");
  std::lock_guard<std::recursive_mutex> g(h->w->api_mu);
  std::memset(o, 0, sizeof(*o));
  o->count = h->count;
  o->max_particles = h->cap;
  o->step_count = h->step_count;
  for (int a = 0; a < 3; a++) { o->dims[a] = h->dims[a]; o->origin[a] = h->origin[a]; o->gravity[a] = h->gravity[a]; }
  o->num_materials = h->nmats;
  o->num_colliders = h->ncol;
  o->sort_every = h->sort_every;
  o->substeps = h->substeps;
  o->ppc_axis = h->ppc_axis;
  o->bound = h->bound;
  o->num_nodes = h->nodes;
  o->num_blocks = h->num_blocks;
  o->dx = h->dx;
  o->substep_dt = h->dt;
  o->time_scale = h->time_scale;
  o->device_bytes = h->destroyed ? 0 : h->device_bytes;
  return SI_OK;
}

int si_mpm_set_materials(si_mpm* h, const float* rows, int32_t m) {
  GUARD(h);
  if (m < 0 || m > SI_MAX_MATERIALS || (m && !rows))
    return si_fail(SI_EINVAL, "MPM: at most 8 distinct materials at once (clear() frees them)");
  std::memset(h->mats, 0, sizeof(h->mats));
  if (m) std::memcpy(h->mats, rows, sizeof(float) * 12 * (size_t)m);
  h->nmats = m;
  h->prm_dirty = true;
  invalidate(h);
  return SI_OK;
}

static int put_records(si_mpm* h, const float* rec, int64_t off, int64_t n) {
  si_world* w = h->w;
  float* stage = nullptr;
  CK(cudaMallocAsync((void**)&stage, (size_t)n * 128, w->st));
  CK(cudaMemcpyAsync(stage, rec, (size_t)n * 128, cudaMemcpyHostToDevice, w->st));
  launch_aos_to_soa(stage, h->pbuf[h->pcur], h->cap, off, n, w->st);
  CK(cudaFreeAsync(stage, w->st));
  CK(cudaGetLastError());
  return SI_OK;
}

int si_mpm_add_particles(si_mpm* h, const float* rec, int64_t n, int64_t* added) {
  if (added) *added = 0;
  GUARD(h);
  if (n < 0 || (n && !rec)) return si_fail(SI_EINVAL, "MPM.add: bad particle array");
  n = std::min(n, h->cap - h->count);   // mpm.js:211
  if (n <= 0) return SI_OK;
  int r = put_records(h, rec, h->count, n);
  if (r) return r;
  h->count += n;
  invalidate(h);
  world_free_graphs(h->w);
  if (added) *added = n;
  return SI_OK;
}

// One xorshift32 step (sampleShape's rand(), mpm.js:685) and its GF(2) matrix powers.
static uint32_t xs_step_host(uint32_t s) {
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  return s;
}
static uint32_t gf2_apply_host(const uint32_t* cols, uint32_t v) {
  uint32_t r = 0;
  for (int j = 0; j < 32; j++)
    if ((v >> j) & 1u) r ^= cols[j];
  return r;
}

int si_mpm_emit(si_mpm* h, int32_t shape, const double a[3], const double b[3], double radius, double half_height,
                double jitter, uint32_t seed, int32_t material, const double velocity[3], int64_t* added) {
  if (added) *added = 0;
  GUARD(h);
  if (!a || (shape == 0 && !b)) return si_fail(SI_EINVAL, "MPM.add: shape needs box | sphere | cylinder");
  if (shape < 0 || shape > 2) return si_fail(SI_EINVAL, "MPM.add: shape needs box | sphere | cylinder | sdf | points");
  if (material < 0 || material >= std::max(1, h->nmats)) return si_fail(SI_EINVAL, "MPM.add: unknown material slot");
  EmitInfo e;
  std::memset(&e, 0, sizeof(e));
  const double spacing = h->dx / h->ppc_axis;
  double lo[3], hi[3];
  if (shape == 0) {
    for (int k = 0; k < 3; k++) { lo[k] = a[k]; hi[k] = b[k]; }
  } else if (shape == 1) {
    for (int k = 0; k < 3; k++) { lo[k] = a[k] - radius; hi[k] = a[k] + radius; }
  } else {
    lo[0] = a[0] - radius; lo[1] = a[1] - half_height; lo[2] = a[2] - radius;
    hi[0] = a[0] + radius; hi[1] = a[1] + half_height; hi[2] = a[2] + radius;
  }
  e.total = 1;
  for (int k = 0; k < 3; k++) {
    const double q = std::floor((hi[k] - lo[k]) / spacing);
    e.n[k] = (int64_t)std::max(1.0, q);
    e.total *= e.n[k];
    e.lo[k] = lo[k];
    e.a[k] = a[k];
    e.origin[k] = h->origin[k];
    e.hi[k] = (double)(h->dims[k] - h->bound);
  }
  if (e.total > (int64_t)1 << 31) return si_fail(SI_EINVAL, "MPM.add: more than 2^31 lattice points");
  const int64_t room = h->cap - h->count;   // mpm.js:211
  if (room <= 0) return SI_OK;
  e.shape = shape;
  e.r = radius;
  e.spacing = spacing;
  e.jitter = jitter;
  e.seed = seed ? seed : 1u;
  uint32_t m[32];
  for (int j = 0; j < 32; j++) m[j] = xs_step_host(1u << j);
  uint32_t m2[32];
  for (int j = 0; j < 32; j++) m2[j] = gf2_apply_host(m, m[j]);
  for (int j = 0; j < 32; j++) e.jump[0][j] = gf2_apply_host(m, m2[j]);          // M^3
  for (int i = 1; i < 32; i++)
    for (int j = 0; j < 32; j++) e.jump[i][j] = gf2_apply_host(e.jump[i - 1], e.jump[i - 1][j]);
  e.dx = h->dx;
  e.bound = (double)h->bound;
  const double s = h->dt / h->dx;
  for (int k = 0; k < 3; k++) e.vel[k] = (float)((velocity ? velocity[k] : 0.0) * s);
  e.material = (uint32_t)material;
  e.P = h->pbuf[h->pcur];
  e.cap = h->cap;
  e.offset = h->count;
  e.room = room;
  const int64_t ctas = (e.total + 255) / 256;
  uint32_t* scratch = nullptr;
  cudaStream_t st = h->w->st;
  CK(cudaMallocAsync((void**)&scratch, (size_t)(ctas + 1) * 4, st));
  if (launch_emit(e, scratch, st) != 0) {
    cudaFreeAsync(scratch, st);
    return si_fail(SI_EDEVICE, "MPM.add: emission launch failed");
  }
  int64_t inside = e.total;
  if (shape == 0) {
    // every lattice point of a box is kept (its inside test is always true, mpm.js:689), so the
    // count is known here and nothing waits for the stream, which may hold other scenes' substeps
    // (a server admitting a scene while its rounds run)
    CK(cudaFreeAsync(scratch, st));
  } else {
    uint32_t counted = 0;
    CK(cudaMemcpyAsync(&counted, scratch + ctas, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaFreeAsync(scratch, st));
    CK(cudaStreamSynchronize(st));
    inside = counted;
  }
  const int64_t n = std::min<int64_t>(inside, room);
  h->count += n;
  invalidate(h);
  world_free_graphs(h->w);
  if (added) *added = n;
  return SI_OK;
}

int si_mpm_clear(si_mpm* h) {
  GUARD(h);
  h->count = 0;
  invalidate(h);
  world_free_graphs(h->w);
  return SI_OK;
}

int si_mpm_write_particles(si_mpm* h, const float* rec, int64_t off, int64_t n) {
  GUARD(h);
  if (off < 0 || n < 0 || off + n > h->count || (n && !rec))
    return si_fail(SI_EINVAL, "MPM: write outside [0, count)");
  if (n == 0) return SI_OK;
  int r = put_records(h, rec, off, n);
  if (r) return r;
  invalidate(h);
  return SI_OK;
}

int si_mpm_read_particles(si_mpm* h, float* rec, int64_t off, int64_t n) {
  GUARD(h);
  if (off < 0 || n < 0 || off + n > h->count || (n && !rec))
    return si_fail(SI_EINVAL, "MPM: read outside [0, count)");
  if (n == 0) return SI_OK;
  si_world* w = h->w;
  float* stage = nullptr;
  CK(cudaMallocAsync((void**)&stage, (size_t)n * 128, w->st));
  launch_soa_to_aos(h->pbuf[h->pcur], h->cap, off, n, stage, w->st);
  CK(cudaMemcpyAsync(rec, stage, (size_t)n * 128, cudaMemcpyDeviceToHost, w->st));
  CK(cudaFreeAsync(stage, w->st));
  CK(cudaStreamSynchronize(w->st));
  CK(cudaGetLastError());
  return SI_OK;
}

int si_mpm_read_positions(si_mpm* h, float* xyz, int64_t off, int64_t n) {
  GUARD(h);
  if (off < 0 || n < 0 || off + n > h->count || (n && !xyz))
    return si_fail(SI_EINVAL, "MPM: read outside [0, count)");
  if (n == 0) return SI_OK;
  si_world* w = h->w;
  float* stage = nullptr;
  CK(cudaMallocAsync((void**)&stage, (size_t)n * 12, w->st));
  launch_positions(h->pbuf[h->pcur], h->cap, off, n, h->dx, h->origin, stage, w->st);
  CK(cudaMemcpyAsync(xyz, stage, (size_t)n * 12, cudaMemcpyDeviceToHost, w->st));
  CK(cudaFreeAsync(stage, w->st));
  CK(cudaStreamSynchronize(w->st));
  CK(cudaGetLastError());
  return SI_OK;
}

int si_mpm_read_instances(si_mpm* h, float* out, int64_t off, int64_t n, uint32_t mat_mask, double size) {
  GUARD(h);
  if (off < 0 || n < 0 || off + n > h->count || (n && !out))
    return si_fail(SI_EINVAL, "MPM: read outside [0, count)");
  if (n == 0) return SI_OK;
  si_world* w = h->w;
  // the layer's uniforms (mpm.js:662-664), JavaScript numbers written as f32
  const float scale = (float)h->dx;
  const float offset[3] = {(float)h->origin[0], (float)h->origin[1], (float)h->origin[2]};
  const float radius = (float)((h->dx / h->ppc_axis) * 0.6 * size);
  const float vel_scale = (float)(h->dx / h->dt);
  float* stage = nullptr;
  CK(cudaMallocAsync((void**)&stage, (size_t)n * 32, w->st));
  launch_instances(h->pbuf[h->pcur], h->cap, off, n, scale, offset, radius, vel_scale, mat_mask, stage, w->st);
  CK(cudaMemcpyAsync(out, stage, (size_t)n * 32, cudaMemcpyDeviceToHost, w->st));
  CK(cudaFreeAsync(stage, w->st));
  CK(cudaStreamSynchronize(w->st));
  CK(cudaGetLastError());
  return SI_OK;
}

int si_mpm_read_positions_async(si_mpm* h, float* xyz, int64_t off, int64_t n, uint64_t* ticket) {
  GUARD(h);
  if (!ticket || off < 0 || n < 0 || off + n > h->count || (n && !xyz))
    return si_fail(SI_EINVAL, "MPM: read outside [0, count)");
  si_world* w = h->w;
  if (!w->st_copy) CK(cudaStreamCreateWithFlags(&w->st_copy, cudaStreamNonBlocking));
  cudaEvent_t ev = nullptr;
  CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  if (n > 0) {
    // the positions are converted in stream order; the copy to the host runs on the copy stream
    // while the next steps run (they never touch the staging buffer)
    float* stage = nullptr;
    CK(cudaMallocAsync((void**)&stage, (size_t)n * 12, w->st));
    launch_positions(h->pbuf[h->pcur], h->cap, off, n, h->dx, h->origin, stage, w->st);
    CK(cudaEventRecord(ev, w->st));
    CK(cudaStreamWaitEvent(w->st_copy, ev, 0));
    CK(cudaMemcpyAsync(xyz, stage, (size_t)n * 12, cudaMemcpyDeviceToHost, w->st_copy));
    CK(cudaFreeAsync(stage, w->st_copy));
  }
  CK(cudaEventRecord(ev, n > 0 ? w->st_copy : w->st));
  *ticket = w->next_read++;
  w->reads[*ticket] = ev;
  return SI_OK;
}

int si_mpm_read_wait(si_mpm* h, uint64_t ticket) {
  if (!h) return si_fail(SI_EINVAL, "null MPM handle");
  cudaEvent_t ev = nullptr;
  {
    std::lock_guard<std::recursive_mutex> g(h->w->api_mu);
    auto it = h->w->reads.find(ticket);
    if (it == h->w->reads.end()) return si_fail(SI_EINVAL, "MPM: unknown read ticket");
    ev = it->second;
    h->w->reads.erase(it);
  }
  const cudaError_t e = cudaEventSynchronize(ev);   // outside the lock: other calls may proceed
  cudaEventDestroy(ev);
  return e == cudaSuccess ? SI_OK : si_fail(SI_EDEVICE, std::string("MPM: read failed: ") + cudaGetErrorString(e));
}

int si_mpm_device_ptr(si_mpm* h, int32_t what, const void** ptr, int64_t* count, int64_t* stride) {
  GUARD(h);
  if (!ptr || !count || !stride) return si_fail(SI_EINVAL, "null output");
  if (what >= 0 && what < (int32_t)kStreams) {
    *ptr = h->pbuf[h->pcur] + (size_t)what * (size_t)h->cap;
    *count = h->count;
    *stride = 16;
  } else if (what == 8) {
    *ptr = h->grid[h->gcur];
    *count = h->nodes;
    *stride = 16;
  } else if (what == 9) {
    if (h->compact) return si_fail(SI_EINVAL, "si_mpm_device_ptr: a scene admitted to a server keeps no keys");
    *ptr = h->keys[1 - h->kpend];
    *count = h->count;
    *stride = 4;
  } else if (what == 10) {
    *ptr = h->starts;
    *count = (int64_t)h->num_blocks + 1;
    *stride = 4;
  } else {
    return si_fail(SI_EINVAL, "si_mpm_device_ptr: what must be 0..10");
  }
  return SI_OK;
}

int si_mpm_set_colliders(si_mpm* h, const float* rows, int32_t k) {
  GUARD(h);
  if (k < 0 || (k && !rows)) return si_fail(SI_EINVAL, "MPM: bad collider table");
  k = std::min(k, SI_MAX_COLLIDERS);   // colliders.slice(0, 16), mpm.js:280
  std::memset(h->cols, 0, sizeof(h->cols));
  if (k) std::memcpy(h->cols, rows, sizeof(float) * 12 * (size_t)k);
  h->ncol = k;
  h->prm_dirty = true;
  return SI_OK;
}

int si_mpm_couple(si_mpm* h, const float* bodies, int32_t n, double friction, double band, uint32_t mask,
                  double density_scale) {
  GUARD(h);
  if (n < 0 || (n && !bodies)) return si_fail(SI_EINVAL, "MPM.couple: bad body table");
  cudaStream_t st = h->w->st;
  if (h->bodies) CK(cudaFreeAsync(h->bodies, st));
  if (h->body_acc) CK(cudaFreeAsync(h->body_acc, st));
  h->bodies = nullptr;
  h->body_acc = nullptr;
  h->nbodies = 0;
  h->prm_dirty = true;
  if (n == 0) return SI_OK;   // uncouple(), mpm.js:255-259
  CK(cudaMallocAsync((void**)&h->bodies, (size_t)n * 192, st));
  CK(cudaMallocAsync((void**)&h->body_acc, (size_t)n * 32, st));
  CK(cudaMemcpyAsync(h->bodies, bodies, (size_t)n * 192, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(h->body_acc, 0, (size_t)n * 32, st));
  CK(cudaStreamSynchronize(st));   // the host table may be reused by the caller
  h->nbodies = n;
  h->friction = friction;
  h->band = band;
  h->body_mask = mask;
  h->density_scale = density_scale;
  return SI_OK;
}

int si_mpm_set_bodies(si_mpm* h, const float* bodies, int32_t n) {
  GUARD(h);
  if (!bodies || n != h->nbodies) return si_fail(SI_EINVAL, "MPM: the body table must keep the coupled count");
  if (n == 0) return SI_OK;
  return stage_upload(h->w, h->bodies, bodies, (size_t)n * 192);   // the caller's table is free on return
}

int si_mpm_read_impulses(si_mpm* h, float* out, int32_t n) {
  GUARD(h);
  if (!out || n != h->nbodies) return si_fail(SI_EINVAL, "MPM: impulses are read for the coupled bodies");
  if (n == 0) return SI_OK;
  std::vector<int32_t> acc((size_t)n * 8);
  CK(cudaMemcpyAsync(acc.data(), h->body_acc, (size_t)n * 32, cudaMemcpyDeviceToHost, h->w->st));
  CK(cudaMemsetAsync(h->body_acc, 0, (size_t)n * 32, h->w->st));
  CK(cudaStreamSynchronize(h->w->st));
  // mpm-rigid-apply, coupling.js:188-196, on the host: momToWorld = densityScale dx^4 / dt (f32)
  const float m2w = (float)(h->density_scale * std::pow(h->dx, 4.0) / h->dt);
  const float dx = (float)h->dx;
  for (int32_t i = 0; i < n; i++) {
    const int32_t* a = acc.data() + 8 * (size_t)i;
    float* o = out + 8 * (size_t)i;
    std::memset(o, 0, 8 * sizeof(float));
    if (a[0] == 0 && a[1] == 0 && a[2] == 0 && a[4] == 0 && a[5] == 0 && a[6] == 0) continue;
    for (int k = 0; k < 3; k++) {
      o[k] = 0.0f + ((float)a[k] / 16384.0f) * m2w;
      o[4 + k] = 0.0f + (((float)a[4 + k] / 1024.0f) * m2w) * dx;
    }
  }
  return SI_OK;
}

int si_mpm_set_gravity(si_mpm* h, const double g[3]) {
  GUARD(h);
  if (!g) return si_fail(SI_EINVAL, "null gravity");
  for (int a = 0; a < 3; a++) h->gravity[a] = g[a];
  h->prm_dirty = true;
  return SI_OK;
}

int si_mpm_set_sort_every(si_mpm* h, int32_t n) {
  GUARD(h);
  h->sort_every = n > 0 ? n : 4;   // `o.sortEvery || 4`
  return SI_OK;
}

int si_mpm_set_substep_dt(si_mpm* h, double dt) {
  GUARD(h);
  if (!(dt > 0) || !std::isfinite(dt)) return si_fail(SI_EINVAL, "MPM: substep dt must be positive");
  const double k = dt / h->dt;   // mpm.js:143
  h->dt = dt;
  h->prm_dirty = true;
  if (h->count && std::fabs(k - 1) > 1e-12) {
    launch_retime(h->pbuf[h->pcur], h->cap, (int32_t)h->count, (float)k, h->w->st);
    CK(cudaGetLastError());
    invalidate(h);
  }
  return SI_OK;
}

int si_mpm_set_frame(si_mpm* h, int32_t substeps, double time_scale) {
  GUARD(h);
  if (substeps > 0) h->substeps = substeps;
  if (!std::isnan(time_scale)) h->time_scale = std::max(1e-6, time_scale);   // mpm.js:139
  return si_mpm_set_substep_dt(h, (1.0 / 60) * h->time_scale / h->substeps);
}

int si_mpm_step(si_mpm* h, double dt, int32_t K) {
  GUARD(h);
  if (dt > 0 && dt != h->dt) {
    int r = si_mpm_set_substep_dt(h, dt);
    if (r) return r;
  }
  if (K <= 0) K = h->substeps;
  if (h->count == 0) return SI_OK;   // mpm.js:584
  h->frame_sub = 0;
  std::vector<si_mpm*> one{h};
  return run_substeps(h->w, one, K);
}

int si_mpm_sort(si_mpm* h) { GUARD(h); return run_phase(h, T_SORT, 0); }
int si_mpm_p2g(si_mpm* h, int32_t force_global) {
  GUARD(h);
  return run_phase(h, T_P2G, force_global ? F_FORCE_GLOBAL : 0u);
}
int si_mpm_grid_update(si_mpm* h) { GUARD(h); return run_phase(h, T_GRID, 0); }
int si_mpm_g2p(si_mpm* h) { GUARD(h); return run_phase(h, T_G2P, 0); }

int si_mpm_read_grid(si_mpm* h, int32_t* nodes4) {
  GUARD(h);
  if (!nodes4) return si_fail(SI_EINVAL, "null output");
  CK(cudaMemcpyAsync(nodes4, h->grid[h->gcur], (size_t)h->nodes * 16, cudaMemcpyDeviceToHost, h->w->st));
  CK(cudaStreamSynchronize(h->w->st));
  return SI_OK;
}

int si_mpm_read_bins(si_mpm* h, uint32_t* keys, uint32_t* starts) {
  GUARD(h);
  if (keys && h->compact) return si_fail(SI_EINVAL, "si_mpm_read_bins: a scene admitted to a server keeps no keys");
  if (keys && h->count)
    CK(cudaMemcpyAsync(keys, h->keys[1 - h->kpend], (size_t)h->count * 4, cudaMemcpyDeviceToHost, h->w->st));
  if (starts)
    CK(cudaMemcpyAsync(starts, h->starts, ((size_t)h->num_blocks + 1) * 4, cudaMemcpyDeviceToHost, h->w->st));
  CK(cudaStreamSynchronize(h->w->st));
  return SI_OK;
}

int si_mpm_sync(si_mpm* h) {
  GUARD(h);
  CK(cudaStreamSynchronize(h->w->st));
  CK(cudaGetLastError());
  return SI_OK;
}

}  // extern "C"
