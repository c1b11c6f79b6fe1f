// si_couple.cu — the fluid <-> rigid coupling pass (src/physics/coupling.js:83-186) for sm_103a.
//
// After the grid update of a substep, every node with mass within `band` cells of a body has its
// velocity relative to the body projected (no penetration, Coulomb friction on the tangent), and the
// momentum that adds is the body's reaction impulse. The reference's unit of work is kept: a 4^3
// tile of nodes culls the bodies whose bounding spheres reach it into a candidate list in index
// order (at most 128), and runs its nodes against the candidates in that order. Here one warp owns
// a tile (two nodes per lane, no CTA barrier), and the warps of the launch take only the tiles of the
// region the grid update visited; a tile without mass leaves at once; the cull is one ballot per 32
// bodies; a node computes a candidate's normal only when its distance lies inside the band; and the
// tile's fixed-point impulse sums per candidate (J x 16384, L x 1024) are warp integer reductions
// added to the per-body accumulators with i32 atomics, the same integers the reference's shared
// atomics sum, so the result does not depend on execution order.
// Built with -fmad=false; the f32 order follows the reference's WGSL as written (see si_math.cuh).
#include "si_device.h"
#include "si_math.cuh"
#include "si_region.cuh"

namespace si {

constexpr int kMaxCand = 128;          // MAX_CAND, coupling.js:25
constexpr float kFPJ = 16384.0f;       // coupling.js:26
constexpr float kFPL = 1024.0f;        // coupling.js:27
constexpr uint32_t kSensor = 2u, kDisabled = 4u;   // rigid-wgsl.js:35-36

// qmat of src/shaders/math.js:56-62 (columns)
__device__ __forceinline__ m3 qmat(float4 q) {
  const float x = q.x, y = q.y, z = q.z, w = q.w;
  m3 r;
  r.c[0] = V(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + w * z), 2.0f * (x * z - w * y));
  r.c[1] = V(2.0f * (x * y - w * z), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + w * x));
  r.c[2] = V(2.0f * (x * z + w * y), 2.0f * (y * z - w * x), 1.0f - 2.0f * (x * x + y * y));
  return r;
}

// i32(e) of WGSL: truncation, saturating at the ends of the range, NaN -> 0 (cvt.rzi.s32.f32)
__device__ __forceinline__ int32_t wgsl_i32(float x) { return __float2int_rz(x); }

// bodySDF, coupling.js:31-58, split in two: the distance from p to a body (centre c, rotation
// R = qmat(q), size and shape code s), which every node within a candidate's reach needs, and the
// outward normal, which only nodes inside the band need. Both halves evaluate the reference's
// expressions in its order, so distance and normal equal those of the one-piece function bit for bit.
__device__ __forceinline__ float body_dist(const m3& R, float4 size, uint32_t s, v3 c, v3 p, v3& lp) {
  lp = mv(mT(R), vsub(p, c));
  if (s == 0u) return vlen(lp) - size.x;
  if (s == 2u) {
    const float h = size.y;
    return vlen(V(lp.x, lp.y - clampf(lp.y, -h, h), lp.z)) - size.x;
  }
  const v3 q = V(fabsf(lp.x) - size.x, fabsf(lp.y) - size.y, fabsf(lp.z) - size.z);
  if (q.x > 0.0f || q.y > 0.0f || q.z > 0.0f)
    return vlen(V(lp.x - clampf(lp.x, -size.x, size.x), lp.y - clampf(lp.y, -size.y, size.y),
                  lp.z - clampf(lp.z, -size.z, size.z)));
  int ax = 0;
  if (q.y > get(q, ax)) ax = 1;
  if (q.z > get(q, ax)) ax = 2;
  return get(q, ax);
}
__device__ __forceinline__ v3 body_normal(const m3& R, float4 size, uint32_t s, v3 lp) {
  if (s == 0u) {
    const float d = vlen(lp);
    const float m = fmaxf(d, 1e-6f);
    return mv(R, V(lp.x / m, lp.y / m, lp.z / m));
  }
  if (s == 2u) {
    const float h = size.y;
    const v3 q = V(lp.x, lp.y - clampf(lp.y, -h, h), lp.z);
    const float d = vlen(q);
    const float m = fmaxf(d, 1e-6f);
    const v3 t = V(q.x / m, q.y / m, q.z / m);
    const float sg = lp.y > 0.0f ? 1.0f : (lp.y < 0.0f ? -1.0f : 0.0f);
    return mv(R, d > 1e-6f ? t : V(0.0f, sg, 0.0f));
  }
  const v3 q = V(fabsf(lp.x) - size.x, fabsf(lp.y) - size.y, fabsf(lp.z) - size.z);
  if (q.x > 0.0f || q.y > 0.0f || q.z > 0.0f) {
    const v3 dv = V(lp.x - clampf(lp.x, -size.x, size.x), lp.y - clampf(lp.y, -size.y, size.y),
                    lp.z - clampf(lp.z, -size.z, size.z));
    const float d = vlen(dv);
    const float m = fmaxf(d, 1e-9f);
    return mv(R, V(dv.x / m, dv.y / m, dv.z / m));
  }
  int ax = 0;
  if (q.y > get(q, ax)) ax = 1;
  if (q.z > get(q, ax)) ax = 2;
  const float sg = get(lp, ax) >= 0.0f ? 1.0f : -1.0f;
  return mv(R, V(ax == 0 ? sg : 0.0f, ax == 1 ? sg : 0.0f, ax == 2 ? sg : 0.0f));
}

constexpr int kCoupleWarps = 8;   // tiles (warps) per CTA

// The tiles of a coupled scene that can hold mass are those of the region its grid update visited
// (4^3 tiles aligned to multiples of 4, as the reference's workgroups): every warp of the launch
// takes that scene's region tiles in a grid-stride loop, with the scene's parameters read once.
__global__ void __launch_bounds__(kCoupleWarps * 32) k_couple(TickInfo t) {
  const int lane = threadIdx.x & 31;
  const uint32_t gwarp = blockIdx.x * kCoupleWarps + (threadIdx.x >> 5), nwarps = gridDim.x * kCoupleWarps;
  for (int si = 0; si < t.nscenes; si++) {
    const TickScene& ts = t.ts[si];
    if (!(ts.flags & F_COUPLE)) continue;
    const SceneParams* prm = ts.prm;
    const int32_t X = prm->dims[0], Y = prm->dims[1], Z = prm->dims[2];
    const NodeRegion rg = grid_region(ts, prm->dims);
    if (rg.nx <= 0 || rg.ny <= 0 || rg.nz <= 0) continue;
    const int bx0 = rg.x0 / 4, by0 = rg.y0 / 4, bz0 = rg.z0 / 4;
    const int nbx = (rg.x0 + rg.nx + 3) / 4 - bx0, nby = (rg.y0 + rg.ny + 3) / 4 - by0;
    const int nbz = (rg.z0 + rg.nz + 3) / 4 - bz0;
    const uint32_t ntiles = (uint32_t)nbx * (uint32_t)nby * (uint32_t)nbz;
    const float inv_dx = prm->inv_dx, band = prm->band, lead = ts.lead;
    const v3 origin = V(prm->origin[0], prm->origin[1], prm->origin[2]);
    const int nbodies = prm->nbodies;
    // the cull's inputs of the first 32 bodies stay in registers across the scene's tiles (body `lane`)
    float4 c_bx = make_float4(0.0f, 0.0f, 0.0f, 0.0f), c_bv = c_bx;
    bool c_on = false;
    if (lane < nbodies) {
      const float4* b = prm->bodies + 12 * (size_t)lane;
      const float4 info = b[11];
      c_on = (__float_as_uint(info.z) & (kDisabled | kSensor)) == 0u && (__float_as_uint(info.x) & prm->body_mask) != 0u;
      c_bx = b[0];
      c_bv = b[2];
    }
    // the lane's two nodes of tile i: (lane & 3, (lane >> 2) & 3, lane >> 4) and two z layers higher;
    // a warp loads the nodes of its next tile before it works on the current one
    auto tile_nodes = [&](uint32_t i, int g[2][3], float4* node[2], float4 cell[2]) {
      const int tx = bx0 + (int)(i % (uint32_t)nbx), ty = by0 + (int)((i / (uint32_t)nbx) % (uint32_t)nby);
      const int tz = bz0 + (int)(i / ((uint32_t)nbx * (uint32_t)nby));
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int q = lane + 32 * h;
        g[h][0] = tx * 4 + (q & 3); g[h][1] = ty * 4 + ((q >> 2) & 3); g[h][2] = tz * 4 + (q >> 4);
        node[h] = nullptr;
        cell[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (i < ntiles && g[h][0] < X && g[h][1] < Y && g[h][2] < Z) {
          node[h] = reinterpret_cast<float4*>(ts.grid) +
                    ((size_t)g[h][0] + (size_t)X * ((size_t)g[h][1] + (size_t)Y * (size_t)g[h][2]));
          cell[h] = *node[h];
        }
      }
    };
    int ngx[2][3];
    float4* nnode[2];
    float4 ncell[2];
    tile_nodes(gwarp, ngx, nnode, ncell);
    for (uint32_t i = gwarp; i < ntiles; i += nwarps) {
      int gxyz[2][3];
      float4* node[2];
      float4 cell[2];
      bool live[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        gxyz[h][0] = ngx[h][0]; gxyz[h][1] = ngx[h][1]; gxyz[h][2] = ngx[h][2];
        node[h] = nnode[h];
        cell[h] = ncell[h];
        live[h] = node[h] != nullptr && cell[h].w > 0.0f;
      }
      tile_nodes(i + nwarps, ngx, nnode, ncell);
      const int tx = gxyz[0][0] >> 2, ty = gxyz[0][1] >> 2, tz = gxyz[0][2] >> 2;
      if (!__any_sync(0xffffffffu, live[0] || live[1])) continue;   // no mass in the tile: nothing to do
      // 1. candidates: bodies whose bounding sphere (extrapolated to the lead) reaches the tile, in
      // index order, at most kMaxCand (coupling.js:96-124); kept as one ballot mask per 32 bodies
      const float lo_off = band + 1.0f, hi_off = (3.0f + band) + 1.0f;
      const v3 tl = V((float)(tx * 4) - lo_off, (float)(ty * 4) - lo_off, (float)(tz * 4) - lo_off);
      const v3 th = V((float)(tx * 4) + hi_off, (float)(ty * 4) + hi_off, (float)(tz * 4) + hi_off);
      v3 v[2] = {V(cell[0].x, cell[0].y, cell[0].z), V(cell[1].x, cell[1].y, cell[1].z)};
      bool moved[2] = {false, false};
      int ncand = 0;
      for (int r = 0; r < nbodies && ncand < kMaxCand; r += 32) {
        const int bi = r + lane;
        bool on = c_on;
        float4 bx = c_bx, bv = c_bv;
        if (r > 0) {
          on = false;
          if (bi < nbodies) {
            const float4* b = prm->bodies + 12 * (size_t)bi;
            const float4 info = b[11];
            on = (__float_as_uint(info.z) & (kDisabled | kSensor)) == 0u &&
                 (__float_as_uint(info.x) & prm->body_mask) != 0u;
            bx = b[0];
            bv = b[2];
          }
        }
        bool hit = false;
        if (on) {
          const v3 cc = vscale(inv_dx, vsub(vadd(V(bx.x, bx.y, bx.z), vscale(lead, V(bv.x, bv.y, bv.z))), origin));
          const v3 q = V(clampf(cc.x, tl.x, th.x), clampf(cc.y, tl.y, th.y), clampf(cc.z, tl.z, th.z));
          hit = vlen(vsub(cc, q)) <= bx.w * inv_dx;
        }
        unsigned mask = __ballot_sync(0xffffffffu, hit);
        const int room = kMaxCand - ncand;   // the first kMaxCand candidates only
        if (__popc(mask) > room) {
          unsigned keep = 0u;
          for (int k = 0; k < room; k++) { const unsigned low = mask & (0u - mask); keep |= low; mask ^= low; }
          mask = keep;
        }
        ncand += __popc(mask);
        // 2. the tile's nodes against this round's candidates, in index order (coupling.js:127-160)
        while (mask) {
          const int k = __ffs(mask) - 1;
          mask &= mask - 1u;
          const float4* b = prm->bodies + 12 * (size_t)(r + k);
          const float4 cx = b[0], cv = b[2], cw = b[3], size = b[8];
          const bool dyn = b[9].x > 0.0f;
          const uint32_t shape = (uint32_t)(size.w + 0.5f);   // shapeOf, rigid-wgsl.js:75
          const m3 R = qmat(b[1]);
          const v3 bc = vadd(V(cx.x, cx.y, cx.z), vscale(lead, V(cv.x, cv.y, cv.z)));
          uint32_t jx = 0, jy = 0, jz = 0, lx = 0, ly = 0, lz = 0;   // i32 sums, wrapping as the atomics do
          bool any = false;
#pragma unroll
          for (int h = 0; h < 2; h++) {
            if (!live[h]) continue;
            const v3 pw = vadd(origin, vscale(prm->dx, V((float)gxyz[h][0], (float)gxyz[h][1], (float)gxyz[h][2])));
            v3 lp;
            const float dist = body_dist(R, size, shape, bc, pw, lp);
            if (!(dist * inv_dx < band)) continue;
            const v3 nr = body_normal(R, size, shape, lp);
            const v3 rr = vsub(pw, bc);
            const v3 vb = vscale(prm->vel_to_lattice, vadd(V(cv.x, cv.y, cv.z), vcross(V(cw.x, cw.y, cw.z), rr)));
            v3 vr = vsub(v[h], vb);
            const float vn = vdot(vr, nr);
            if (vn < 0.0f) {
              vr = vsub(vr, vscale(vn, nr));
              const float vt = vlen(vr);
              if (vt > 1e-9f) vr = vscale(fmaxf(0.0f, 1.0f - (prm->friction * -vn) / vt), vr);
              const v3 vnew = vadd(vr, vb);
              if (dyn) {
                const float m = cell[h].w;
                const v3 J = vscale(-m, vsub(vnew, v[h]));
                const v3 L = vcross(vscale(inv_dx, rr), J);
                jx += (uint32_t)wgsl_i32(rintf(J.x * kFPJ)); jy += (uint32_t)wgsl_i32(rintf(J.y * kFPJ));
                jz += (uint32_t)wgsl_i32(rintf(J.z * kFPJ)); lx += (uint32_t)wgsl_i32(rintf(L.x * kFPL));
                ly += (uint32_t)wgsl_i32(rintf(L.y * kFPL)); lz += (uint32_t)wgsl_i32(rintf(L.z * kFPL));
                any = true;
              }
              v[h] = vnew;
              moved[h] = true;
            }
          }
          // 3. the tile's sums for this body (coupling.js:176-181): warp integer sums, one atomic each
          if (__any_sync(0xffffffffu, any)) {
            jx = __reduce_add_sync(0xffffffffu, jx); jy = __reduce_add_sync(0xffffffffu, jy);
            jz = __reduce_add_sync(0xffffffffu, jz); lx = __reduce_add_sync(0xffffffffu, lx);
            ly = __reduce_add_sync(0xffffffffu, ly); lz = __reduce_add_sync(0xffffffffu, lz);
            if (lane == 0) {
              uint32_t* u = reinterpret_cast<uint32_t*>(prm->body_acc + (size_t)(r + k) * 8);
              if (jx) atomicAdd(&u[0], jx);
              if (jy) atomicAdd(&u[1], jy);
              if (jz) atomicAdd(&u[2], jz);
              if (lx) atomicAdd(&u[4], lx);
              if (ly) atomicAdd(&u[5], ly);
              if (lz) atomicAdd(&u[6], lz);
            }
          }
        }
      }
#pragma unroll
      for (int h = 0; h < 2; h++)
        if (moved[h]) *node[h] = make_float4(v[h].x, v[h].y, v[h].z, cell[h].w);
    }
  }
}

// grid_ctas: the CTAs that are resident at once (the warps then loop over the region's tiles)
void launch_couple(const TickInfo& t, int grid_ctas, cudaStream_t st) {
  if (t.cchunks == 0) return;
  const int ctas = (int)min((t.cchunks + kCoupleWarps - 1) / kCoupleWarps, (uint32_t)grid_ctas);
  k_couple<<<ctas, kCoupleWarps * 32, 0, st>>>(t);
}
int couple_ctas_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_couple, kCoupleWarps * 32, 0);
  return n > 0 ? n : 1;
}

}  // namespace si
