// si_couple.cu — the fluid <-> rigid coupling pass (src/physics/coupling.js:83-186) for sm_103a.
//
// After the grid update of a substep, every node with mass within `band` cells of a body has its
// velocity relative to the body projected (no penetration, Coulomb friction on the tangent), and the
// momentum that adds is the body's reaction impulse. One CTA of 64 threads handles a 4^3 tile of
// nodes: it culls the bodies whose bounding spheres reach the tile into a candidate list in index
// order (at most 128, as the reference), runs its nodes against the candidates in that order, sums
// the impulses in fixed point (J x 16384, L x 1024) in shared memory and adds the sums to the
// per-body accumulators with i32 atomics, so the result is the same in any execution order.
// Built with -fmad=false; the f32 order follows the reference's WGSL as written (see si_math.cuh).
#include "si_device.h"
#include "si_math.cuh"

namespace si {

constexpr int kMaxCand = 128;          // MAX_CAND, coupling.js:25
constexpr float kFPJ = 16384.0f;       // coupling.js:26
constexpr float kFPL = 1024.0f;        // coupling.js:27
constexpr uint32_t kSensor = 2u, kDisabled = 4u;   // rigid-wgsl.js:35-36

__device__ __forceinline__ int find_scene_c(const TickScene* ts, int n, uint32_t chunk) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (ts[mid].cchunk_begin <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

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

// bodySDF, coupling.js:31-58: distance from p to body b (centre c) and the outward normal
__device__ __forceinline__ float body_sdf(const float4* b, v3 c, v3 p, v3& n) {
  const float4 size = b[8];
  const uint32_t s = (uint32_t)(size.w + 0.5f);           // shapeOf, rigid-wgsl.js:75
  const m3 R = qmat(b[1]);
  const v3 lp = mv(mT(R), vsub(p, c));
  if (s == 0u) {
    const float d = vlen(lp);
    const float m = fmaxf(d, 1e-6f);
    n = mv(R, V(lp.x / m, lp.y / m, lp.z / m));
    return d - size.x;
  }
  if (s == 2u) {
    const float h = size.y;
    const v3 q = V(lp.x, lp.y - clampf(lp.y, -h, h), lp.z);
    const float d = vlen(q);
    const float m = fmaxf(d, 1e-6f);
    const v3 t = V(q.x / m, q.y / m, q.z / m);
    const float sg = lp.y > 0.0f ? 1.0f : (lp.y < 0.0f ? -1.0f : 0.0f);
    n = mv(R, d > 1e-6f ? t : V(0.0f, sg, 0.0f));
    return d - size.x;
  }
  const v3 q = V(fabsf(lp.x) - size.x, fabsf(lp.y) - size.y, fabsf(lp.z) - size.z);
  if (q.x > 0.0f || q.y > 0.0f || q.z > 0.0f) {
    const v3 dv = V(lp.x - clampf(lp.x, -size.x, size.x), lp.y - clampf(lp.y, -size.y, size.y),
                    lp.z - clampf(lp.z, -size.z, size.z));
    const float d = vlen(dv);
    const float m = fmaxf(d, 1e-9f);
    n = mv(R, V(dv.x / m, dv.y / m, dv.z / m));
    return d;
  }
  int ax = 0;
  if (q.y > get(q, ax)) ax = 1;
  if (q.z > get(q, ax)) ax = 2;
  const float sg = get(lp, ax) >= 0.0f ? 1.0f : -1.0f;
  n = mv(R, V(ax == 0 ? sg : 0.0f, ax == 1 ? sg : 0.0f, ax == 2 ? sg : 0.0f));
  return get(q, ax);
}

__global__ void __launch_bounds__(64) k_couple(TickInfo t) {
  __shared__ int cand[kMaxCand];
  __shared__ int accj[kMaxCand * 3], accl[kMaxCand * 3];
  __shared__ int wcnt[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (uint32_t c = blockIdx.x; c < t.cchunks; c += gridDim.x) {
    const TickScene& ts = t.ts[find_scene_c(t.ts, t.nscenes, c)];
    const SceneParams* prm = ts.prm;
    const int32_t X = prm->dims[0], Y = prm->dims[1], Z = prm->dims[2];
    const uint32_t tnx = (X + 3) / 4, tny = (Y + 3) / 4;
    const uint32_t tile = c - ts.cchunk_begin;
    const int tx = (int)(tile % tnx), ty = (int)((tile / tnx) % tny), tz = (int)(tile / (tnx * tny));
    const float inv_dx = prm->inv_dx, band = prm->band, lead = ts.lead;
    const v3 origin = V(prm->origin[0], prm->origin[1], prm->origin[2]);
    // 1. candidates: bodies whose bounding sphere (extrapolated to the lead) reaches the tile, in
    // index order (coupling.js:96-124)
    const float lo_off = band + 1.0f, hi_off = (3.0f + band) + 1.0f;
    const v3 tl = V((float)(tx * 4) - lo_off, (float)(ty * 4) - lo_off, (float)(tz * 4) - lo_off);
    const v3 th = V((float)(tx * 4) + hi_off, (float)(ty * 4) + hi_off, (float)(tz * 4) + hi_off);
    int base = 0;
    for (int r = 0; r < prm->nbodies && base < kMaxCand; r += 64) {
      const int bi = r + tid;
      bool hit = false;
      if (bi < prm->nbodies) {
        const float4* b = prm->bodies + 12 * (size_t)bi;
        const float4 info = b[11];
        if ((__float_as_uint(info.z) & (kDisabled | kSensor)) == 0u && (__float_as_uint(info.x) & prm->body_mask) != 0u) {
          const float4 bx = b[0], bv = b[2];
          const v3 cc = vscale(inv_dx, vsub(vadd(V(bx.x, bx.y, bx.z), vscale(lead, V(bv.x, bv.y, bv.z))), origin));
          const v3 q = V(clampf(cc.x, tl.x, th.x), clampf(cc.y, tl.y, th.y), clampf(cc.z, tl.z, th.z));
          hit = vlen(vsub(cc, q)) <= bx.w * inv_dx;
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, hit);
      if (lane == 0) wcnt[warp] = __popc(bal);
      __syncthreads();
      const int before = (warp == 1 ? wcnt[0] : 0) + __popc(bal & ((1u << lane) - 1u));
      if (hit && base + before < kMaxCand) cand[base + before] = bi;
      base += wcnt[0] + wcnt[1];
      __syncthreads();
    }
    const int nc = min(base, kMaxCand);
    if (nc == 0) continue;   // the same on every thread of the CTA
    for (int k = tid; k < nc * 3; k += 64) { accj[k] = 0; accl[k] = 0; }
    __syncthreads();
    // 2. this thread's node against the candidates, in order (coupling.js:127-160)
    const int gx = tx * 4 + (tid & 3), gy = ty * 4 + ((tid >> 2) & 3), gz = tz * 4 + (tid >> 4);
    if (gx < X && gy < Y && gz < Z) {
      float4* node = reinterpret_cast<float4*>(ts.grid) + ((size_t)gx + (size_t)X * ((size_t)gy + (size_t)Y * (size_t)gz));
      const float4 cell = *node;
      const float m = cell.w;
      if (m > 0.0f) {
        v3 v = V(cell.x, cell.y, cell.z);
        const v3 pw = vadd(origin, vscale(prm->dx, V((float)gx, (float)gy, (float)gz)));
        for (int k = 0; k < nc; k++) {
          const float4* b = prm->bodies + 12 * (size_t)cand[k];
          const float4 bx = b[0], bv = b[2], bw = b[3];
          const v3 bc = vadd(V(bx.x, bx.y, bx.z), vscale(lead, V(bv.x, bv.y, bv.z)));
          v3 nr;
          const float dist = body_sdf(b, bc, pw, nr);
          if (!(dist * inv_dx < band)) continue;
          const v3 r = vsub(pw, bc);
          const v3 vb = vscale(prm->vel_to_lattice, vadd(V(bv.x, bv.y, bv.z), vcross(V(bw.x, bw.y, bw.z), r)));
          v3 vr = vsub(v, vb);
          const float vn = vdot(vr, nr);
          if (vn < 0.0f) {
            vr = vsub(vr, vscale(vn, nr));
            const float vt = vlen(vr);
            if (vt > 1e-9f) vr = vscale(fmaxf(0.0f, 1.0f - (prm->friction * -vn) / vt), vr);
            const v3 vnew = vadd(vr, vb);
            if (b[9].x > 0.0f) {
              const v3 J = vscale(-m, vsub(vnew, v));
              const v3 L = vcross(vscale(inv_dx, r), J);
              atomicAdd(&accj[k * 3], wgsl_i32(rintf(J.x * kFPJ)));
              atomicAdd(&accj[k * 3 + 1], wgsl_i32(rintf(J.y * kFPJ)));
              atomicAdd(&accj[k * 3 + 2], wgsl_i32(rintf(J.z * kFPJ)));
              atomicAdd(&accl[k * 3], wgsl_i32(rintf(L.x * kFPL)));
              atomicAdd(&accl[k * 3 + 1], wgsl_i32(rintf(L.y * kFPL)));
              atomicAdd(&accl[k * 3 + 2], wgsl_i32(rintf(L.z * kFPL)));
            }
            v = vnew;
          }
        }
        *node = make_float4(v.x, v.y, v.z, m);
      }
    }
    __syncthreads();
    // 3. the tile's sums to the bodies (coupling.js:176-181)
    for (int k = tid; k < nc * 3; k += 64) {
      const int bi = cand[k / 3], a = k % 3;
      if (accj[k] != 0) atomicAdd(&prm->body_acc[bi * 8 + a], accj[k]);
      if (accl[k] != 0) atomicAdd(&prm->body_acc[bi * 8 + 4 + a], accl[k]);
    }
    __syncthreads();
  }
}

void launch_couple(const TickInfo& t, int grid_ctas, cudaStream_t st) {
  if (t.cchunks == 0) return;
  const int ctas = (int)min(t.cchunks, (uint32_t)grid_ctas);
  k_couple<<<ctas, 64, 0, st>>>(t);
}

}  // namespace si
