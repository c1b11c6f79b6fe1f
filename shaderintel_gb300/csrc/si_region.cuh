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

}  // namespace si
