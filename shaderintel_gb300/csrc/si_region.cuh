// si_region.cuh — the grid nodes a scene's substep can touch (device code, included by the kernels).
#pragma once
#include "si_device.h"

namespace si {

// The nodes a scene's grid update visits: the whole grid, or with F_BOXED the nodes under the
// stencils of box_cur + box_next (bases lo..hi reach nodes lo..hi+2), clipped to the grid. Outside it
// both arrays are zero (never scattered to, or cleared since), so the update writes nothing there.
struct NodeRegion {
  int32_t x0, y0, z0, nx, ny, nz;
};
__device__ __forceinline__ NodeRegion grid_region(const TickScene& ts, const int32_t* d) {
  NodeRegion r{0, 0, 0, d[0], d[1], d[2]};
  if (ts.flags & F_BOXED) {
    int32_t lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      lo[a] = max(0, min(ts.box_cur[a], ts.box_next[a]));
      hi[a] = min(d[a], max(ts.box_cur[3 + a], ts.box_next[3 + a]) + 3);
      if (hi[a] < lo[a]) hi[a] = lo[a];
    }
    r = NodeRegion{lo[0], lo[1], lo[2], hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  }
  return r;
}

// A per-scene prefix of the tick table (FIELD: kSceneP the first particle chunk, kSceneN the first
// node chunk, kSceneSeg the first slot of the scene's sort segment), copied into shared memory by each
// CTA once per launch when the tick has at most kSceneTable scenes: the scene of a chunk or slot is
// then found by a binary search in shared memory instead of one through the tick table in global
// memory (eight dependent loads for 256 scenes, on lines the particle streams evict from L1).
constexpr int kSceneTable = 1024;
enum { kSceneP = 0, kSceneN = 1, kSceneSeg = 2 };
template <int FIELD>
__device__ __forceinline__ uint32_t scene_field(const TickScene& e) {
  return FIELD == kSceneP ? e.pchunk_begin : (FIELD == kSceneN ? e.nchunk_begin : e.seg_base);
}
template <int FIELD>
__device__ __forceinline__ void scene_table_load(const TickInfo& t, uint32_t* tab) {
  if (t.nscenes <= kSceneTable)
    for (int i = threadIdx.x; i < t.nscenes; i += blockDim.x) tab[i] = scene_field<FIELD>(t.ts[i]);
}
// the last scene whose prefix is <= x
template <int FIELD>
__device__ __forceinline__ int scene_of(const TickInfo& t, const uint32_t* tab, uint32_t x) {
  const bool shared_tab = t.nscenes <= kSceneTable;
  int lo = 0, hi = t.nscenes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const uint32_t b = shared_tab ? tab[mid] : scene_field<FIELD>(t.ts[mid]);
    if (b <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace si
