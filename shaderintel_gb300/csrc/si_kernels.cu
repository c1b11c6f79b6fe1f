// si_kernels.cu — the substep kernels for sm_103a: P2G (tile / global, optional sort gather),
// grid update, G2P (with the next substep's P2G and block keys fused in), retime, record I/O.
//
// Built with -fmad=false: the f32 order of si_math.cuh is the contract with the CPU oracle.
// Work mapping: persistent CTAs walk flat chunk indices of one tick; a chunk belongs to one scene
// (binary search over the prefixes the host wrote), so one launch per phase serves every scene.
#include <algorithm>

#include "si_device.h"
#include "si_math.cuh"
#include "si_region.cuh"
#include "si_runtime.h"

// Resident CTAs per SM the G2P/P2G kernels are compiled for (register budget 65536 / (256 * n)):
// three (80 registers, a few spilled) beat two (128) by 9 % on the mixed scene and four (64) by 3 %.
#ifndef SI_G2P_MIN_CTAS
#define SI_G2P_MIN_CTAS 3
#endif

namespace si {

// Shared tile: kTileNodes nodes, used first as the gather tile of the G2P (vec4f per node) and then
// as the P2G scatter tile (four planes of i32, stride kTileNodes, so the four channel atomics of a
// node share one address computation). TickInfo::tile_nodes (<= kTileNodes) is the usable capacity.
#ifndef SI_TILE_NODES
#define SI_TILE_NODES 2048
#endif
constexpr int kTileNodes = SI_TILE_NODES;

// CTA barrier that lanes of one warp may reach along different paths (after an `if` on the lane's
// own particle or a tail loop). __syncthreads() is the warp-aligned barrier (barrier.sync.aligned),
// undefined when a warp's lanes arrive at different instructions; the non-aligned form counts each
// arriving thread, so every thread of the CTA has passed the preceding phase when it completes.
__device__ __forceinline__ void cta_sync() { asm volatile("barrier.sync 0;" ::: "memory"); }

__device__ __forceinline__ int find_scene_p(const TickScene* ts, int n, uint32_t chunk) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (ts[mid].pchunk_begin <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ int find_scene_n(const TickScene* ts, int n, uint32_t chunk) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (ts[mid].nchunk_begin <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ------------------------------------------------------------------ P2G inputs of one particle
struct Scat {
  int32_t b[3];      // base node
  float f[3];        // fx = x - base
  float aff[9];      // affine = -vol4 tau + m C, column-major
  float mv[3];       // m v
  float mass;
};

__device__ __forceinline__ void prep_scatter(Scat& s, float4 x, float4 v, float4 c0, float4 c1, float4 c2,
                                             float t01, float t02, float t12, const SceneParams* prm) {
  s.b[0] = base_of(x.x, prm->dims[0]);
  s.b[1] = base_of(x.y, prm->dims[1]);
  s.b[2] = base_of(x.z, prm->dims[2]);
  s.f[0] = x.x - (float)s.b[0];
  s.f[1] = x.y - (float)s.b[1];
  s.f[2] = x.z - (float)s.b[2];
  uint32_t mid = __float_as_uint(x.w) & 7u;
  float mass = __ldg(&prm->mats[mid * 3].y);
  s.mass = mass;
  float nv = -prm->vol4;
  // tau columns (tau00 tau01 tau02), (tau01 tau11 tau12), (tau02 tau12 tau22): mpm.js:324
  s.aff[0] = nv * c0.w + mass * c0.x;
  s.aff[1] = nv * t01 + mass * c0.y;
  s.aff[2] = nv * t02 + mass * c0.z;
  s.aff[3] = nv * t01 + mass * c1.x;
  s.aff[4] = nv * c1.w + mass * c1.y;
  s.aff[5] = nv * t12 + mass * c1.z;
  s.aff[6] = nv * t02 + mass * c2.x;
  s.aff[7] = nv * t12 + mass * c2.y;
  s.aff[8] = nv * c2.w + mass * c2.z;
  s.mv[0] = mass * v.x;
  s.mv[1] = mass * v.y;
  s.mv[2] = mass * v.z;
}

__device__ __forceinline__ bool in_grid(int gx, int gy, int gz, const int32_t* d) {
  return (unsigned)gx < (unsigned)d[0] && (unsigned)gy < (unsigned)d[1] && (unsigned)gz < (unsigned)d[2];
}

// i32(round(x * 2^22)) for |x| < 1, a pair at a time: x * 2^22 is exact, so one fused add of
// 1.5 * 2^23 rounds it to nearest-even exactly like rint, and the low bits of the sum are the
// integer. Equal to to_fixed(x) wherever it is used (the caller proves |x| < 0.9 first).
__device__ __forceinline__ int2 to_fixed_small2(float2 x) {
  const float2 f = fma2(x, make_float2(4194304.0f, 4194304.0f), make_float2(12582912.0f, 12582912.0f));
  return make_int2(__float_as_int(f.x) - 0x4B400000, __float_as_int(f.y) - 0x4B400000);
}

// True when every value the particle scatters has |x| < 0.9: |wt| <= 1, |dpos| <= 1.5 and
// |m v_i + affine_i . dpos| <= |m v_i| + 1.5 sum_k |affine_ki| (bounded with margin here). NaN or
// infinity fails the test.
__device__ __forceinline__ bool scatter_small(const Scat& s) {
  if (s.b[0] < -1000 || s.b[1] < -1000 || s.b[2] < -1000) return false;
  bool ok = fabsf(s.mass) < 0.9f;   // each comparison is false for NaN
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float r = fabsf(s.mv[i]) + 2.0f * ((fabsf(s.aff[i]) + fabsf(s.aff[3 + i])) + fabsf(s.aff[6 + i]));
    ok = ok && r < 0.9f;
  }
  return ok;
}

// 27-node scatter of mpm.js:328-349 into the shared tile (planar channels) or the global grid.
// Lanes whose particles share a base node would hit the same 27 addresses step for step and their
// atomics would serialise (sorted neighbours fill a warp: about 2.7 lanes per base node on the
// mixed 128^3 scene). So each lane takes its rank r among the warp's lanes with the same base node
// and visits the x offsets rotated by (r mod 3) and the y offsets by (r / 3 mod 3): groups of up to
// nine lanes never meet on a node. Every node's contribution is computed by the same expression as
// in the unrotated order, so the i32 sums are unchanged.
template <bool SMALL>
__device__ __forceinline__ void scatter_impl(const Scat& s, const int32_t* dims, int* __restrict__ grid,
                                             int* tile, int o0, int o1, int o2, int sy, int sz, bool use_tile,
                                             float nz) {
  constexpr int tile_cap = kTileNodes;
  float wx[3], wy[3], wz[3];
  bspline(s.f[0], wx); bspline(s.f[1], wy); bspline(s.f[2], wz);
  const int lane = threadIdx.x & 31;
  const unsigned key = (unsigned)s.b[0] + ((unsigned)s.b[1] << 10) + ((unsigned)s.b[2] << 20);
  const int rank = __popc(__match_any_sync(0xffffffffu, key) & ((1u << lane) - 1u));
  const int ra = rank % 3, rb = (rank / 3) % 3;
  int ia[3], ib[3];
  float wa[3], wb[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int a = k + ra >= 3 ? k + ra - 3 : k + ra;
    const int b = k + rb >= 3 ? k + rb - 3 : k + rb;
    ia[k] = a; ib[k] = b;
    wa[k] = a == 0 ? wx[0] : (a == 1 ? wx[1] : wx[2]);
    wb[k] = b == 0 ? wy[0] : (b == 1 ? wy[1] : wy[2]);
  }
  // tile node (x, y, z) sits at x + sy y + sz z (row and layer strides of the tile's layout)
  const int t0 = (s.b[2] - o2) * sz + (s.b[1] - o1) * sy + (s.b[0] - o0);
  // The x/y components of every product and sum go through one packed instruction, z and the mass
  // scalar or paired with each other: the canonical expressions of mpm.js:333-347, per component
  //   r = ((a0 dx + a3 dy) + a6 dz, ...),  m = wt (mv + r),  q = toFixed(m), toFixed(wt mass)
  // with every product and sum rounded on its own.
  const float2 aff01 = make_float2(s.aff[0], s.aff[1]), aff34 = make_float2(s.aff[3], s.aff[4]);
  const float2 mv01 = make_float2(s.mv[0], s.mv[1]);
  float2 p67[3];
  float p8[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float dz = (float)c - s.f[2];
    p67[c] = mul2z(make_float2(s.aff[6], s.aff[7]), make_float2(dz, dz), nz);
    p8[c] = s.aff[8] * dz;
  }
#pragma unroll
  for (int ka = 0; ka < 3; ka++) {
    const int a = ia[ka];
    float dx = (float)a - s.f[0];
    const float2 ax01 = mul2z(aff01, make_float2(dx, dx), nz);
    const float ax2 = s.aff[2] * dx;
#pragma unroll
    for (int kb = 0; kb < 3; kb++) {
      const int b = ib[kb];
      float dy = (float)b - s.f[1];
      float wab = wa[ka] * wb[kb];
      const float2 s01 = add2(ax01, mul2z(aff34, make_float2(dy, dy), nz));
      const float s2 = ax2 + s.aff[5] * dy;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        float wt = wab * wz[c];
        int32_t q0, q1, q2, q3;
        const float2 r01 = add2(s01, p67[c]);
        const float r2 = s2 + p8[c];
        const float2 ww = make_float2(wt, wt);   // products that feed no add: plain mul2
        const float2 m01 = mul2(ww, add2(mv01, r01));
        const float2 m23 = mul2(ww, make_float2(s.mv[2] + r2, s.mass));
        if (SMALL) {
          const int2 q01 = to_fixed_small2(m01), q23 = to_fixed_small2(m23);
          q0 = q01.x; q1 = q01.y; q2 = q23.x; q3 = q23.y;
        } else {
          q0 = to_fixed(m01.x); q1 = to_fixed(m01.y); q2 = to_fixed(m23.x); q3 = to_fixed(m23.y);
        }
        if (use_tile) {
          const int ti = t0 + a + sy * b + sz * c;
          atomicAdd(&tile[ti], q0);
          atomicAdd(&tile[tile_cap + ti], q1);
          atomicAdd(&tile[2 * tile_cap + ti], q2);
          atomicAdd(&tile[3 * tile_cap + ti], q3);
        } else {
          const int gx = s.b[0] + a, gy = s.b[1] + b, gz = s.b[2] + c;
          if (in_grid(gx, gy, gz, dims)) {
            size_t gi = 4 * ((size_t)gx + (size_t)dims[0] * ((size_t)gy + (size_t)dims[1] * (size_t)gz));
            atomicAdd(&grid[gi], q0);
            atomicAdd(&grid[gi + 1], q1);
            atomicAdd(&grid[gi + 2], q2);
            atomicAdd(&grid[gi + 3], q3);
          }
        }
      }
    }
  }
}

// Every lane of the warp calls this (idle lanes with a silenced copy); the fast conversion is chosen
// per warp so the lanes stay on one path.
__device__ __forceinline__ void scatter_one(const Scat& s, const int32_t* dims, int* __restrict__ grid,
                                            int* tile, int o0, int o1, int o2, int sy, int sz, bool use_tile,
                                            float nz) {
  if (__all_sync(0xffffffffu, scatter_small(s))) scatter_impl<true>(s, dims, grid, tile, o0, o1, o2, sy, sz, use_tile, nz);
  else scatter_impl<false>(s, dims, grid, tile, o0, o1, o2, sy, sz, use_tile, nz);
}

// P2G inputs of the CTA's particles, staged in shared memory (SoA, kScatWords words per particle)
// when a thread handles more than one particle of a chunk.
constexpr int kScatWords = 19;

// A copy of a particle that contributes nothing (mass, momentum and affine zero; the base, which lies
// inside the chunk's box, stays): lets idle lanes run the scatter on the same path as the others.
__device__ __forceinline__ void scat_silence(Scat& s) {
  s.mass = 0.0f;
  s.mv[0] = s.mv[1] = s.mv[2] = 0.0f;
#pragma unroll
  for (int q = 0; q < 9; q++) s.aff[q] = 0.0f;
}

__device__ __forceinline__ void scat_store(float* sc, int chunk, int slot, const Scat& s) {
  sc[0 * chunk + slot] = __int_as_float(s.b[0]);
  sc[1 * chunk + slot] = __int_as_float(s.b[1]);
  sc[2 * chunk + slot] = __int_as_float(s.b[2]);
  sc[3 * chunk + slot] = s.f[0];
  sc[4 * chunk + slot] = s.f[1];
  sc[5 * chunk + slot] = s.f[2];
#pragma unroll
  for (int q = 0; q < 9; q++) sc[(6 + q) * chunk + slot] = s.aff[q];
  sc[15 * chunk + slot] = s.mv[0];
  sc[16 * chunk + slot] = s.mv[1];
  sc[17 * chunk + slot] = s.mv[2];
  sc[18 * chunk + slot] = s.mass;
}
__device__ __forceinline__ void scat_load(const float* sc, int chunk, int slot, Scat& s) {
  s.b[0] = __float_as_int(sc[0 * chunk + slot]);
  s.b[1] = __float_as_int(sc[1 * chunk + slot]);
  s.b[2] = __float_as_int(sc[2 * chunk + slot]);
  s.f[0] = sc[3 * chunk + slot];
  s.f[1] = sc[4 * chunk + slot];
  s.f[2] = sc[5 * chunk + slot];
#pragma unroll
  for (int q = 0; q < 9; q++) s.aff[q] = sc[(6 + q) * chunk + slot];
  s.mv[0] = sc[15 * chunk + slot];
  s.mv[1] = sc[16 * chunk + slot];
  s.mv[2] = sc[17 * chunk + slot];
  s.mass = sc[18 * chunk + slot];
}

// Visits every node of an ex x ey x ez tile once across the CTA and calls f(t, lx, ly, lz) with
// t = lx + ex (ly + ey lz). The nodes are taken as columns along z: a thread splits its column
// index into (lx, ly) once and then steps lz, instead of splitting every flat index with three
// integer divisions by the runtime extents. When a layer holds fewer nodes than the CTA has
// threads, floor(256 / layer) threads share each column at z offsets 0, 1, ...
template <typename Fn>
__device__ __forceinline__ void tile_walk(int ex, int ey, int ez, Fn&& f) {
  const int tid = threadIdx.x;
  const int exy = ex * ey;
  const bool narrow = exy < kCtaThreads;
  const int zs = narrow ? kCtaThreads / exy : 1;
  const int z0 = narrow ? tid / exy : 0;
  if (z0 >= zs) return;
  for (int col = narrow ? tid - z0 * exy : tid; col < exy; col += narrow ? exy : kCtaThreads) {
    const int ly = col / ex, lx = col - ly * ex;
    for (int lz = z0; lz < ez; lz += zs) f(col + exy * lz, lx, ly, lz);
  }
}

// Layout of the scatter tile: when the padded box fits the tile, rows of tx nodes padded by one and
// layers padded to a stride of 12 mod 32 words, so that lanes scattering into neighbouring rows and
// layers meet fewer shared-memory bank conflicts (a CPU model of the sorted mixed scene: 3.9 -> 3.4
// wavefronts per atomic); otherwise the dense layout, so that padding never makes a chunk overflow the
// tile. The layout moves only the tile's addresses, never what is summed.
#ifndef SI_TILE_PAD
#define SI_TILE_PAD 1
#endif
#ifndef SI_TILE_PADX
#define SI_TILE_PADX 1    // nodes added to a row
#endif
#ifndef SI_TILE_LMOD
#define SI_TILE_LMOD 12   // layer stride mod 32
#endif
__device__ __forceinline__ int tile_layer_stride_padded(int sy, int ty) {
  const int a = sy * ty;
  return a + ((SI_TILE_LMOD - (a & 31)) & 31);
}
__device__ __forceinline__ long long tile_padded_nodes(int tx, int ty, int tz) {
  return (long long)tile_layer_stride_padded(tx + SI_TILE_PADX, ty) * tz;
}

// Side of the largest cube of nodes the tile holds (dense layout; tile_nodes >= 343).
__device__ __forceinline__ int tile_cube_side(int tile_nodes) {
  int e = 7;
  while ((e + 1) * (e + 1) * (e + 1) <= tile_nodes) e++;
  return e;
}

// A box in shared memory: lo[3], hi[3] of node coordinates, grown with atomicMin/atomicMax. It is
// emptied by three threads; a CTA barrier must separate that from the atomics that grow it again.
__device__ __forceinline__ void box_empty(int* b) {
  if (threadIdx.x < 3) { b[threadIdx.x] = 0x3fffffff; b[3 + threadIdx.x] = -0x3fffffff; }
}

// CTA-wide P2G: AABB of the bases (mpm.js:353-377), tile if it fits (mpm.js:379-380), scatter,
// flush of the non-zero tile nodes with global i32 atomics (mpm.js:385-399). The particles come from
// `reg` (one per thread, valid if has_reg) when sc == nullptr, else from the `count` staged copies.
// `sbox` arrives empty (and ordered by an earlier barrier); before the final barrier this function
// empties it again for the next chunk, together with `gbox` (the caller's gather box, or nullptr),
// once every thread has read them: no barrier is spent on re-initialising either box.
__device__ __forceinline__ void cta_scatter(const Scat& reg, bool has_reg, const float* sc, int chunk, int count,
                                            const int32_t* dims, int* __restrict__ grid, bool force_global,
                                            int tile_nodes, int* tile, int* sbox, int* gbox, int32_t* scene_box,
                                            float nz) {
  constexpr int tile_cap = kTileNodes;
  const int tid = threadIdx.x;
  int lo0 = 0x3fffffff, lo1 = 0x3fffffff, lo2 = 0x3fffffff;
  int hi0 = -0x3fffffff, hi1 = -0x3fffffff, hi2 = -0x3fffffff;
  if (sc == nullptr) {
    if (has_reg) {
      lo0 = hi0 = reg.b[0]; lo1 = hi1 = reg.b[1]; lo2 = hi2 = reg.b[2];
    }
  } else {
    for (int slot = tid; slot < count; slot += blockDim.x) {   // count is a multiple of the CTA size here
      const int b0 = __float_as_int(sc[slot]), b1 = __float_as_int(sc[chunk + slot]), b2 = __float_as_int(sc[2 * chunk + slot]);
      lo0 = min(lo0, b0); lo1 = min(lo1, b1); lo2 = min(lo2, b2);
      hi0 = max(hi0, b0); hi1 = max(hi1, b1); hi2 = max(hi2, b2);
    }
  }
  lo0 = __reduce_min_sync(0xffffffffu, lo0); lo1 = __reduce_min_sync(0xffffffffu, lo1);
  lo2 = __reduce_min_sync(0xffffffffu, lo2);
  hi0 = __reduce_max_sync(0xffffffffu, hi0); hi1 = __reduce_max_sync(0xffffffffu, hi1);
  hi2 = __reduce_max_sync(0xffffffffu, hi2);
  if ((tid & 31) == 0) {
    atomicMin(&sbox[0], lo0); atomicMin(&sbox[1], lo1); atomicMin(&sbox[2], lo2);
    atomicMax(&sbox[3], hi0); atomicMax(&sbox[4], hi1); atomicMax(&sbox[5], hi2);
  }
  if (sc == nullptr && tid == kCtaThreads / 2) { sbox[8] = reg.b[0]; sbox[9] = reg.b[1]; sbox[10] = reg.b[2]; }
  cta_sync();
  const int o0 = sbox[0], o1 = sbox[1], o2 = sbox[2];
  const int ex = sbox[3] - o0 + 3, ey = sbox[4] - o1 + 3, ez = sbox[5] - o2 + 3;
  if (tid == 0 && scene_box != nullptr && ex > 0) {   // the scene's box of P2G bases (grid update bounds)
    atomicMin(&scene_box[0], o0); atomicMin(&scene_box[1], o1); atomicMin(&scene_box[2], o2);
    atomicMax(&scene_box[3], sbox[3]); atomicMax(&scene_box[4], sbox[4]); atomicMax(&scene_box[5], sbox[5]);
  }
  if (ex <= 0 || ey <= 0 || ez <= 0) {   // no valid particle in the chunk (the same for every thread)
    cta_sync();
    box_empty(sbox);
    if (gbox) box_empty(gbox);
    cta_sync();
    return;
  }
  const long long tn = (long long)ex * ey * ez;
  bool pad = SI_TILE_PAD && tile_padded_nodes(ex, ey, ez) <= tile_nodes;
  bool use_tile = tn <= tile_nodes && !force_global;
  // the tile's box: the chunk's, or (the chunk overflows the tile) the part of it inside a cube of
  // side e (e^3 <= tile_nodes) around the middle particle's base; particles whose base lies outside
  // that part scatter with global atomics
  int t0 = o0, t1 = o1, t2 = o2, tx = ex, ty = ey, tz = ez;
  bool clipped = false;
  if (!use_tile && !force_global) {
    const int e = tile_cube_side(tile_nodes);
    const int m = (sc == nullptr) ? 0 : count / 2;
    const int c0 = sc == nullptr ? sbox[8] : __float_as_int(sc[m]);
    const int c1 = sc == nullptr ? sbox[9] : __float_as_int(sc[chunk + m]);
    const int c2 = sc == nullptr ? sbox[10] : __float_as_int(sc[2 * chunk + m]);
    const int half = (e - 3) / 2;
    const int l0 = max(o0, c0 - half), l1 = max(o1, c1 - half), l2 = max(o2, c2 - half);
    const int h0 = min(sbox[3], c0 - half + (e - 3)), h1 = min(sbox[4], c1 - half + (e - 3)),
              h2 = min(sbox[5], c2 - half + (e - 3));
    if (h0 >= l0 && h1 >= l1 && h2 >= l2) {
      t0 = l0; t1 = l1; t2 = l2;
      tx = h0 - l0 + 3; ty = h1 - l1 + 3; tz = h2 - l2 + 3;
      use_tile = clipped = true;
      pad = false;
    }
  }
  const int sy = pad ? tx + SI_TILE_PADX : tx, sz = pad ? tile_layer_stride_padded(sy, ty) : sy * ty;
  const int tnodes = use_tile ? sz * tz : 0;   // extent of the layout, padding included
  if (use_tile) {
    for (int t = tid; t < tnodes; t += blockDim.x) {
      tile[t] = 0; tile[tile_cap + t] = 0; tile[2 * tile_cap + t] = 0; tile[3 * tile_cap + t] = 0;
    }
    cta_sync();
  }
  auto inside = [&](const Scat& q) {   // the particle's 27 nodes lie in the tile
    return !clipped || ((unsigned)(q.b[0] - t0) <= (unsigned)(tx - 3) && (unsigned)(q.b[1] - t1) <= (unsigned)(ty - 3) &&
                        (unsigned)(q.b[2] - t2) <= (unsigned)(tz - 3));
  };
  if (sc == nullptr) {
    scatter_one(reg, dims, grid, tile, t0, t1, t2, sy, sz, use_tile && inside(reg), nz);   // every lane
  } else {
#pragma unroll 1
    for (int slot = tid; slot < count; slot += blockDim.x) {
      Scat s;
      scat_load(sc, chunk, slot, s);
      scatter_one(s, dims, grid, tile, t0, t1, t2, sy, sz, use_tile && inside(s), nz);
    }
  }
  cta_sync();   // every thread has scattered, and has read the boxes long ago
  box_empty(sbox);
  if (gbox) box_empty(gbox);
  if (use_tile) {
    tile_walk(tx, ty, tz, [&](int, int lx, int ly, int lz) {
      const int t = lx + sy * ly + sz * lz;
      const int m = tile[3 * tile_cap + t], mx = tile[t], my = tile[tile_cap + t], mz = tile[2 * tile_cap + t];
      if ((m | mx | my | mz) != 0) {
        const int gx = t0 + lx, gy = t1 + ly, gz = t2 + lz;
        if (in_grid(gx, gy, gz, dims)) {
          size_t gi = 4 * ((size_t)gx + (size_t)dims[0] * ((size_t)gy + (size_t)dims[1] * (size_t)gz));
          atomicAdd(&grid[gi], mx);
          atomicAdd(&grid[gi + 1], my);
          atomicAdd(&grid[gi + 2], mz);
          atomicAdd(&grid[gi + 3], m);
        }
      }
    });
  }
  cta_sync();   // the tile and the staged inputs are reused by the next chunk
}

// ------------------------------------------------------------------ P2G kernel (mpm.js:306-401)
template <int PPT>
__global__ void __launch_bounds__(kCtaThreads, SI_G2P_MIN_CTAS) k_p2g(TickInfo t) {
  extern __shared__ __align__(16) int smem[];
  int* tile = smem;
  int* sbox = smem + 4 * kTileNodes;
  float* sc = reinterpret_cast<float*>(sbox + 24);
  constexpr int chunk = kCtaThreads * PPT;
  box_empty(sbox);
  cta_sync();
  for (uint32_t c = blockIdx.x; c < t.pchunks; c += gridDim.x) {
    const TickScene& ts = t.ts[find_scene_p(t.ts, t.nscenes, c)];
    const uint32_t flags = ts.flags;
    if (!(flags & F_P2G)) continue;
    const SceneParams* prm = ts.prm;
    const int first = (int)(c - ts.pchunk_begin) * chunk;
    const int count = min(chunk, ts.n - first);
    const int32_t dims[3] = {prm->dims[0], prm->dims[1], prm->dims[2]};
    const float4* src = ts.P;
    const int64_t cap = ts.cap;
    Scat reg;
#pragma unroll
    for (int k = 0; k < PPT; k++) {
      const bool valid = k * kCtaThreads + (int)threadIdx.x < count;
      const int64_t i = first + min(k * kCtaThreads + (int)threadIdx.x, count - 1);
      float4 x = __ldg(&src[i]), v = __ldg(&src[cap + i]);
      float4 c0 = __ldg(&src[2 * cap + i]), c1 = __ldg(&src[3 * cap + i]), c2 = __ldg(&src[4 * cap + i]);
      float t01 = __ldg(&src[5 * cap + i].w), t02 = __ldg(&src[6 * cap + i].w), t12 = __ldg(&src[7 * cap + i].w);
      prep_scatter(reg, x, v, c0, c1, c2, t01, t02, t12, prm);
      if (!valid) scat_silence(reg);
      if (PPT > 1) scat_store(sc, chunk, k * kCtaThreads + threadIdx.x, reg);
    }
    cta_scatter(reg, true, PPT > 1 ? sc : nullptr, chunk, PPT > 1 ? chunk : count, dims,
                reinterpret_cast<int*>(ts.grid), (flags & F_FORCE_GLOBAL) != 0, t.tile_nodes, tile, sbox, nullptr,
                ts.box_cur, t.nz);
  }
}

// zero the grid of scenes whose P2G target is not known to be clear (p2g() clears first, mpm.js:609)
__global__ void __launch_bounds__(kCtaThreads) k_clear(TickInfo t) {
  for (uint32_t chunk = blockIdx.x; chunk < t.nchunks; chunk += gridDim.x) {
    const TickScene& ts = t.ts[find_scene_n(t.ts, t.nscenes, chunk)];
    if (!(ts.flags & F_CLEAR)) continue;
    const SceneParams* prm = ts.prm;
    const int64_t nodes = (int64_t)prm->dims[0] * prm->dims[1] * prm->dims[2];
    const int64_t first = (int64_t)(chunk - ts.nchunk_begin) * ts.node_chunk;
    const int64_t last = min(first + (int64_t)ts.node_chunk, nodes);
    for (int64_t i = first + threadIdx.x; i < last; i += blockDim.x) ts.grid[i] = make_int4(0, 0, 0, 0);
  }
}

// the reorder of _sort() on its own (mpm.js:572-577): Palt[i] = P[perm[i]]
__global__ void __launch_bounds__(kCtaThreads) k_reorder(TickInfo t, const uint32_t* __restrict__ perm) {
  for (uint32_t chunk = blockIdx.x; chunk < t.pchunks; chunk += gridDim.x) {
    const TickScene& ts = t.ts[find_scene_p(t.ts, t.nscenes, chunk)];
    if (!(ts.flags & F_GATHER)) continue;
    const int first = (int)(chunk - ts.pchunk_begin) * t.chunk;
    const int last = min(first + t.chunk, ts.n);
    const int64_t cap = ts.cap;
    for (int i = first + threadIdx.x; i < last; i += blockDim.x) {
      const int64_t j = __ldg(&perm[ts.seg_base + i]);
#pragma unroll
      for (int k = 0; k < kStreams; k++) ts.Palt[k * cap + i] = __ldg(&ts.P[k * cap + j]);
    }
  }
}

// The sort substep of a scene with one particle buffer: the streams its G2P reads of the old state
// (x, v for J, and F unless the material is a fluid, whose G2P never reads F) are gathered through
// perm into the world's scratch, segment seg_base, in sorted order. The G2P then reads them there
// and writes the new state into P in place.
__global__ void __launch_bounds__(kCtaThreads) k_pregather(TickInfo t, const uint32_t* __restrict__ perm,
                                                          float4* __restrict__ scratch, int64_t stride) {
  for (uint32_t chunk = blockIdx.x; chunk < t.pchunks; chunk += gridDim.x) {
    const TickScene& ts = t.ts[find_scene_p(t.ts, t.nscenes, chunk)];
    if (!(ts.flags & F_PREGATHER)) continue;
    const int first = (int)(chunk - ts.pchunk_begin) * t.chunk;
    const int last = min(first + t.chunk, ts.n);
    const int64_t cap = ts.cap;
    const SceneParams* prm = ts.prm;
    float4* out = scratch + ts.seg_base;
    for (int i = first + threadIdx.x; i < last; i += blockDim.x) {
      const int64_t j = __ldg(&perm[ts.seg_base + i]);
      const float4 x = __ldcs(&ts.P[j]);
      out[i] = x;
      out[stride + i] = __ldcs(&ts.P[cap + j]);
      if (__float_as_uint(__ldg(&prm->mats[(__float_as_uint(x.w) & 7u) * 3].x)) != 0u) {
        out[2 * stride + i] = __ldcs(&ts.P[5 * cap + j]);
        out[3 * stride + i] = __ldcs(&ts.P[6 * cap + j]);
        out[4 * stride + i] = __ldcs(&ts.P[7 * cap + j]);
      }
    }
  }
}

// ------------------------------------------------------------------ grid update (mpm.js:414-471)
__device__ __forceinline__ float collider_sdf(uint32_t kind, v3 d, float4 s) {
  if (kind == 0u) return vlen(d) - s.x;
  if (kind == 1u) {
    v3 q = V(fabsf(d.x) - s.x, fabsf(d.y) - s.y, fabsf(d.z) - s.z);
    v3 qm = V(fmaxf(q.x, 0.0f), fmaxf(q.y, 0.0f), fmaxf(q.z, 0.0f));
    return vlen(qm) + fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f);
  }
  return vdot(d, V(s.x, s.y, s.z));
}

// The nodes [first, last) of a scene's region (flat region order), thread tid from first + tid at
// the CTA's stride.
__device__ __forceinline__ void grid_nodes(const TickScene& ts, const NodeRegion& reg, int64_t first, int64_t last) {
  const SceneParams* prm = ts.prm;
  const int64_t X = prm->dims[0], Y = prm->dims[1];
  const float bound = prm->bound, ff = prm->floor_friction;
  const float g0 = prm->gravity[0], g1 = prm->gravity[1], g2 = prm->gravity[2];
  const v3 hi = V((float)prm->dims[0] - bound, (float)prm->dims[1] - bound, (float)prm->dims[2] - bound);
  const int ncol = prm->ncol;
  const bool clear_next = !(ts.flags & F_NO_CLEAR_NEXT);
  // the thread's node (lx, ly, lz) of the region is split once and then advanced by the CTA's
  // stride without further divisions by the region's extents
  const uint32_t nxr = (uint32_t)reg.nx, nyr = (uint32_t)reg.ny, rxy = nxr * nyr;
  const uint32_t qy = blockDim.x / nxr, rx = blockDim.x - qy * nxr;
  uint32_t lz, ly, lx;
  {
    const uint32_t r0 = (uint32_t)(first + threadIdx.x);
    lz = r0 / rxy;
    const uint32_t rem = r0 - lz * rxy;
    ly = rem / nxr;
    lx = rem - ly * nxr;
  }
  for (int64_t r = first + threadIdx.x; r < last; r += blockDim.x) {
    if (r != first + threadIdx.x) {
      lx += rx;
      ly += qy;
      if (lx >= nxr) { lx -= nxr; ly++; }
      if (ly >= nyr) {
        if (ly < 2 * nyr) { ly -= nyr; lz++; }
        else { lz += ly / nyr; ly -= (ly / nyr) * nyr; }
      }
    }
    const int64_t nxi = reg.x0 + lx, nyi = reg.y0 + ly, nzi = reg.z0 + lz;
    const int64_t i = nxi + X * (nyi + Y * nzi);
    int4 g = ts.grid[i];
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (g.w > 0) {
      const float inv = 1.0f / 4194304.0f;
      float m = (float)g.w * inv;
      v3 v = V(((float)g.x * inv) / m + g0, ((float)g.y * inv) / m + g1, ((float)g.z * inv) / m + g2);
      v3 c = V((float)nxi, (float)nyi, (float)nzi);
      if (c.y < bound && v.y < 0.0f) {
        float vn = -v.y;
        v.y = 0.0f;
        float vt = sqrtf(v.x * v.x + v.z * v.z);
        if (vt > 1e-9f) {
          float f = fmaxf(0.0f, 1.0f - (ff * vn) / vt);
          v = V(v.x * f, 0.0f, v.z * f);
        }
      }
      if (c.x < bound && v.x < 0.0f) v.x = 0.0f;
      if (c.z < bound && v.z < 0.0f) v.z = 0.0f;
      if (c.x > hi.x && v.x > 0.0f) v.x = 0.0f;
      if (c.y > hi.y && v.y > 0.0f) v.y = 0.0f;
      if (c.z > hi.z && v.z > 0.0f) v.z = 0.0f;
      for (int k = 0; k < ncol; k++) {
        const float4 h = prm->cols[3 * k], s = prm->cols[3 * k + 1], cvv = prm->cols[3 * k + 2];
        const v3 cv = V(cvv.x, cvv.y, cvv.z);
        const uint32_t kind = __float_as_uint(h.x);
        const v3 d = V(c.x - h.y, c.y - h.z, c.z - h.w);
        float dist = collider_sdf(kind, d, s);
        if (dist < 1.0f) {
          const float e = 0.5f;
          v3 nr = V(collider_sdf(kind, V(d.x + e, d.y, d.z), s) - collider_sdf(kind, V(d.x - e, d.y, d.z), s),
                    collider_sdf(kind, V(d.x, d.y + e, d.z), s) - collider_sdf(kind, V(d.x, d.y - e, d.z), s),
                    collider_sdf(kind, V(d.x, d.y, d.z + e), s) - collider_sdf(kind, V(d.x, d.y, d.z - e), s));
          nr = V(nr.x + 0.0f, nr.y + 1e-7f, nr.z + 0.0f);
          float ln = vlen(nr);
          nr = V(nr.x / ln, nr.y / ln, nr.z / ln);
          v3 vr = vsub(v, cv);
          float vn = vdot(vr, nr);
          if (vn < 0.0f) {
            vr = vsub(vr, vscale(vn, nr));
            float vt = vlen(vr);
            if (vt > 1e-9f) vr = vscale(fmaxf(0.0f, 1.0f - (s.w * -vn) / vt), vr);
            v = vadd(vr, cv);
          }
        }
      }
      out = make_float4(v.x, v.y, v.z, m);
    }
    if ((g.x | g.y | g.z | g.w) != 0) reinterpret_cast<float4*>(ts.grid)[i] = out;   // zero stays zero
    if (clear_next) ts.grid_next[i] = make_int4(0, 0, 0, 0);
  }
}

// Every scene's region in node chunks of the host's table (ticks of several scenes).
__device__ __forceinline__ void grid_chunks(const TickInfo& t) {
  __shared__ uint32_t scene_tab[kSceneTable];
  scene_table_load<kSceneN>(t, scene_tab);
  __syncthreads();
  for (uint32_t chunk = blockIdx.x; chunk < t.nchunks; chunk += gridDim.x) {
    const TickScene& ts = t.ts[scene_of<kSceneN>(t, scene_tab, chunk)];
    const NodeRegion reg = grid_region(ts, ts.prm->dims);
    const int64_t nodes = (int64_t)reg.nx * reg.ny * reg.nz;
    const int64_t first = (int64_t)(chunk - ts.nchunk_begin) * ts.node_chunk;
    if (first >= nodes) continue;
    grid_nodes(ts, reg, first, min(first + (int64_t)ts.node_chunk, nodes));
  }
}

// Ticks of at most kSceneTable scenes: the concatenation of their boxed regions split evenly over
// the launch's CTAs, one contiguous piece each (multiples of 32 nodes), instead of the host's chunk
// table, which counts whole grids and leaves most chunks empty. Each CTA sums the scenes' region sizes
// itself (four scenes a thread, then a block scan) into an exclusive prefix in shared memory.
__device__ __forceinline__ void grid_even(const TickInfo& t) {
  static_assert(4 * kCtaThreads >= kSceneTable, "four scenes a thread cover the table");
  __shared__ long long pre[kSceneTable + 1];
  __shared__ long long wsum[kCtaThreads / 32];
  const int nsc = t.nscenes;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long v[4], sum = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int e = threadIdx.x * 4 + q;
    v[q] = 0;
    if (e < nsc) {
      const TickScene& ts = t.ts[e];
      const NodeRegion reg = grid_region(ts, ts.prm->dims);
      v[q] = (long long)reg.nx * reg.ny * reg.nz;
    }
    sum += v[q];
  }
  long long incl = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const long long o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += o;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  long long excl = incl - sum, total = 0;
  for (int w = 0; w < kCtaThreads / 32; w++) {
    if (w < warp) excl += wsum[w];
    total += wsum[w];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int e = threadIdx.x * 4 + q;
    if (e < nsc) pre[e] = excl;
    excl += v[q];
  }
  if (threadIdx.x == 0) pre[nsc] = total;
  __syncthreads();
  const long long per = ((total + gridDim.x - 1) / gridDim.x + 31) & ~31ll;
  const long long lo = (long long)blockIdx.x * per, hi = min(lo + per, total);
  if (lo >= hi) return;
  int a = 0, b = nsc - 1;                            // the scene holding node lo: the last e with pre[e] <= lo
  while (a < b) {
    const int mid = (a + b + 1) >> 1;
    if (pre[mid] <= lo) a = mid; else b = mid - 1;
  }
  for (int e = a; e < nsc && pre[e] < hi; e++) {
    const long long nodes = pre[e + 1] - pre[e];
    if (nodes == 0) continue;
    const long long first = max(lo - pre[e], 0ll), last = min(hi - pre[e], nodes);
    if (first >= last) continue;
    const TickScene& ts = t.ts[e];
    const NodeRegion reg = grid_region(ts, ts.prm->dims);
    grid_nodes(ts, reg, first, last);
  }
}

// The CTA that finishes last empties box_next of every scene for the fused P2G of the G2P that
// follows: every CTA has read the boxes (grid_region) before it counted itself done.
__device__ __forceinline__ void grid_boxes_reset(const TickInfo& t) {
  if (t.reset_boxes) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      last = atomicAdd(t.grid_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
      for (int s = threadIdx.x; s < t.nscenes; s += blockDim.x) {
        int32_t* b = t.ts[s].box_next;
        if (b) {
          b[0] = b[1] = b[2] = 0x3fffffff;
          b[3] = b[4] = b[5] = -0x3fffffff;
        }
      }
      if (threadIdx.x == 0) *t.grid_done = 0;
    }
  }
}

// The grid update of a tick of one scene (three CTAs per SM).
__global__ void __launch_bounds__(kCtaThreads) k_grid(TickInfo t) {
  if (t.nscenes == 1) {
    // One scene: its boxed region split evenly over the launch's CTAs, one piece each (multiples of
    // 32 nodes). The host's node chunks cover the whole grid, so taking the region's first chunks
    // left whatever exceeded one wave of CTAs to a second wave of a few (grid phase of the mixed
    // scene -9 %, plasticity -16 %).
    const TickScene& ts = t.ts[0];
    const NodeRegion reg = grid_region(ts, ts.prm->dims);
    const int64_t nodes = (int64_t)reg.nx * reg.ny * reg.nz;
    const int64_t per = ((nodes + gridDim.x - 1) / gridDim.x + 31) & ~(int64_t)31;
    const int64_t first = (int64_t)blockIdx.x * per;
    if (first < nodes) grid_nodes(ts, reg, first, min(first + per, nodes));
  } else {
    grid_chunks(t);
  }
  grid_boxes_reset(t);
}
// The grid update of a tick of several scenes, at four CTAs per SM (64 registers): their many small
// boxed regions gain from the extra warps (batched substep -0.7 %, single scenes +5 % in the grid
// phase). Up to kSceneTable scenes the regions are split evenly over the CTAs (batched substep -2.1 %
// against the chunk table).
__global__ void __launch_bounds__(kCtaThreads, 4) k_grid_wide(TickInfo t) {
  if (t.nscenes <= kSceneTable) grid_even(t);
  else grid_chunks(t);
  grid_boxes_reset(t);
}

// Empties box_next of every scene of the tick: the fused P2G of the G2P that follows rebuilds it.
__global__ void k_box_reset(TickInfo t) {
  for (int s = threadIdx.x; s < t.nscenes; s += blockDim.x) {
    int32_t* b = t.ts[s].box_next;
    if (b) {
      b[0] = b[1] = b[2] = 0x3fffffff;
      b[3] = b[4] = b[5] = -0x3fffffff;
    }
  }
}

// ------------------------------------------------------------------ G2P (mpm.js:474-560)
// The 27-node gather reads the CTA's shared tile (TILE: node (a,b,c) of the stencil at
// t0 + a + sx*b + sxy*c, always inside) or, when the CTA's stencils did not fit the tile, the
// global grid with bounds checks (nodes outside the grid read as zero).
// The gathered sums of one particle: v += t and B += outer3(t, dpos) with t = wt gv
// (mpm.js:500-509), product and sum rounded separately, in packed accumulators: (v.x, v.y),
// (B0.x, B0.y), (B1.x, B1.y), (B2.x, B2.y), (B0.z, B1.z), (v.z, B2.z), where column k of B gains
// t dpos_k.
struct Gathered {
  float2 vxy, bxy0, bxy1, bxy2, z01, z2v;
};

// The gather over the 27 nodes around a particle, from the shared tile (TILE) or from the grid.
// Only this part depends on where the nodes come from, so the kernel holds two copies of it and
// one of the constitutive update below.
template <bool TILE>
__device__ __forceinline__ Gathered g2p_gather(const float4& X, const SceneParams* prm,
                                               const float4* __restrict__ grid, const float4* tilef, int o0,
                                               int o1, int o2, int sx, int sxy, float negz) {
  const int32_t dx0 = prm->dims[0], dx1 = prm->dims[1], dx2 = prm->dims[2];
  const int b0 = base_of(X.x, dx0), b1 = base_of(X.y, dx1), b2 = base_of(X.z, dx2);
  const float f0 = X.x - (float)b0, f1 = X.y - (float)b1, f2 = X.z - (float)b2;
  float wx[3], wy[3], wz[3];
  bspline(f0, wx); bspline(f1, wy); bspline(f2, wz);
  float2 vxy = make_float2(0.0f, 0.0f), bxy0 = vxy, bxy1 = vxy, bxy2 = vxy, z01 = vxy, z2v = vxy;
  const int t0 = TILE ? ((b2 - o2) * (sxy / sx) + (b1 - o1)) * sx + (b0 - o0) : 0;
#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    const float dpx = (float)a - f0;
    const float wxa = a == 0 ? wx[0] : (a == 1 ? wx[1] : wx[2]);   // select, not a local-memory index
#pragma unroll
    for (int b = 0; b < 3; b++) {
      const float dpy = (float)b - f1;
      const float wab = wxa * wy[b];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float dpz = (float)c - f2;
        const float wt = wab * wz[c];
        v3 gv;
        if (TILE) {
          const float4 n = tilef[t0 + a + sx * b + sxy * c];
          gv = V(n.x, n.y, n.z);
        } else {
          const int gx = b0 + a, gy = b1 + b, gz = b2 + c;
          gv = V(0.0f, 0.0f, 0.0f);
          if ((unsigned)gx < (unsigned)dx0 && (unsigned)gy < (unsigned)dx1 && (unsigned)gz < (unsigned)dx2) {
            const float4 n = __ldg(&grid[(size_t)gx + (size_t)dx0 * ((size_t)gy + (size_t)dx1 * (size_t)gz)]);
            gv = V(n.x, n.y, n.z);
          }
        }
        const float2 txy = mul2z(make_float2(wt, wt), make_float2(gv.x, gv.y), negz);
        const float tz = wt * gv.z;
        const float2 tzz = make_float2(tz, tz);
        vxy = add2(vxy, txy);
        bxy0 = add2(bxy0, mul2z(txy, make_float2(dpx, dpx), negz));
        bxy1 = add2(bxy1, mul2z(txy, make_float2(dpy, dpy), negz));
        bxy2 = add2(bxy2, mul2z(txy, make_float2(dpz, dpz), negz));
        z01 = add2(z01, mul2z(tzz, make_float2(dpx, dpy), negz));
        z2v = add2(z2v, mul2z(tzz, make_float2(1.0f, dpz), negz));   // (t.z, t.z dpz): t.z * 1 is exact
      }
    }
  }
  return Gathered{vxy, bxy0, bxy1, bxy2, z01, z2v};
}

// C, velocity clamp, advection and the constitutive update of one particle from its gathered sums
// (mpm.js:510-558). FAST: snow and sand decompose F with svd3_fast (to a tolerance) instead of svd3.
template <bool FAST>
__device__ __forceinline__ void g2p_update(const Gathered& g, float4& X, float4& Vv, float4& C0, float4& C1,
                                           float4& C2, float4& F0, float4& F1, float4& F2,
                                           const SceneParams* prm) {
  const int32_t dx0 = prm->dims[0], dx1 = prm->dims[1], dx2 = prm->dims[2];
  const float2 vxy = g.vxy, bxy0 = g.bxy0, bxy1 = g.bxy1, bxy2 = g.bxy2, z01 = g.z01, z2v = g.z2v;
  v3 v;
  m3 B;
  v = V(vxy.x, vxy.y, z2v.x);
  B.c[0] = V(bxy0.x, bxy0.y, z01.x);
  B.c[1] = V(bxy1.x, bxy1.y, z01.y);
  B.c[2] = V(bxy2.x, bxy2.y, z2v.y);
  m3 C;
  C.c[0] = vscale(4.0f, B.c[0]); C.c[1] = vscale(4.0f, B.c[1]); C.c[2] = vscale(4.0f, B.c[2]);
  const float sp = vlen(v);
  if (sp > prm->vmax) v = vscale(prm->vmax / sp, v);
  const float bound = prm->bound;
  const float lo = bound - 1.0f;
  const float nx = clampf(X.x + v.x, lo, ((float)dx0 - bound) + 1.0f);
  const float ny = clampf(X.y + v.y, lo, ((float)dx1 - bound) + 1.0f);
  const float nz = clampf(X.z + v.z, lo, ((float)dx2 - bound) + 1.0f);
  const uint32_t mid = __float_as_uint(X.w) & 7u;
  const float4 m0 = prm->mats[mid * 3], m1 = prm->mats[mid * 3 + 1], m2 = prm->mats[mid * 3 + 2];
  const uint32_t kind = __float_as_uint(m0.x);
  m3 F;
  F.c[0] = V(F0.x, F0.y, F0.z); F.c[1] = V(F1.x, F1.y, F1.z); F.c[2] = V(F2.x, F2.y, F2.z);
  float t00, t11, t22, t01, t02, t12;   // tau[0].x tau[1].y tau[2].z tau[1].x tau[2].x tau[2].y
  float vw = Vv.w;
  if (kind == 0u) {
    const float J = clampf(vw * (1.0f + ((C.c[0].x + C.c[1].y) + C.c[2].z)), 0.6f, 1.4f);
    vw = J;
    const float a = m0.z * fminf(J - 1.0f, 0.02f);
    const float b = m1.x * J;
    t00 = a * 1.0f + b * (C.c[0].x + C.c[0].x);
    t11 = a * 1.0f + b * (C.c[1].y + C.c[1].y);
    t22 = a * 1.0f + b * (C.c[2].z + C.c[2].z);
    t01 = a * 0.0f + b * (C.c[1].x + C.c[0].y);
    t02 = a * 0.0f + b * (C.c[2].x + C.c[0].z);
    t12 = a * 0.0f + b * (C.c[2].y + C.c[1].z);
    F.c[0] = V(1.0f, 0.0f, 0.0f); F.c[1] = V(0.0f, 1.0f, 0.0f); F.c[2] = V(0.0f, 0.0f, 1.0f);
  } else {
    m3 IC;
    IC.c[0] = V(1.0f + C.c[0].x, 0.0f + C.c[0].y, 0.0f + C.c[0].z);
    IC.c[1] = V(0.0f + C.c[1].x, 1.0f + C.c[1].y, 0.0f + C.c[1].z);
    IC.c[2] = V(0.0f + C.c[2].x, 0.0f + C.c[2].y, 1.0f + C.c[2].z);
    F = mm(IC, F);
    const float mu0 = m0.z, la0 = m0.w;
    if (kind == 1u) {
      const float J = fmaxf(det3(F), 0.05f);
      const m3 FFt = mm(F, mT(F));
      const float l = la0 * si_logf(J);
      t00 = mu0 * (FFt.c[0].x - 1.0f) + l * 1.0f;
      t11 = mu0 * (FFt.c[1].y - 1.0f) + l * 1.0f;
      t22 = mu0 * (FFt.c[2].z - 1.0f) + l * 1.0f;
      t01 = mu0 * (FFt.c[1].x - 0.0f) + l * 0.0f;
      t02 = mu0 * (FFt.c[2].x - 0.0f) + l * 0.0f;
      t12 = mu0 * (FFt.c[2].y - 0.0f) + l * 0.0f;
    } else {
      // snow and sand share one inlined copy of the SVD
      m3 U, Vm; v3 sv;
      if (FAST) svd3_fast(F, U, sv, Vm);
      else svd3(F, U, sv, Vm);
      if (kind == 2u) {
        const float lo_s = 1.0f - m1.z, hi_s = 1.0f + m1.w;
        const v3 s = V(clampf(sv.x, lo_s, hi_s), clampf(sv.y, lo_s, hi_s), clampf(sv.z, lo_s, hi_s));
        const float Jold = (sv.x * sv.y) * sv.z;
        const float Jnew = (s.x * s.y) * s.z;
        vw = clampf(divx<FAST>(vw * Jold, Jnew), 0.6f, 20.0f);
        F = mmx<FAST>(mdiag_right(U, s), mT(Vm));
        const float h = expx<FAST>(m1.y * (1.0f - vw));
        const float mu = mu0 * h, la = la0 * h;
        const float J = Jnew;
        const float tm = 2.0f * mu;
        m3 P1;
        if (FAST) {
          // 2 mu (F - R) F^T with F = U S V^T and R = U V^T is U diag(2 mu (s - 1) s) U^T
          const v3 dd = V(tm * ((s.x - 1.0f) * s.x), tm * ((s.y - 1.0f) * s.y), tm * ((s.z - 1.0f) * s.z));
          P1 = mm_fma(mdiag_right(U, dd), mT(U));
        } else {
          const m3 R = mm(U, mT(Vm));
          m3 FR;
          FR.c[0] = vscale(tm, vsub(F.c[0], R.c[0]));
          FR.c[1] = vscale(tm, vsub(F.c[1], R.c[1]));
          FR.c[2] = vscale(tm, vsub(F.c[2], R.c[2]));
          P1 = mm(FR, mT(F));
        }
        const float l = (la * J) * (J - 1.0f);
        t00 = P1.c[0].x + l * 1.0f;
        t11 = P1.c[1].y + l * 1.0f;
        t22 = P1.c[2].z + l * 1.0f;
        t01 = P1.c[1].x + l * 0.0f;
        t02 = P1.c[2].x + l * 0.0f;
        t12 = P1.c[2].y + l * 0.0f;
      } else {
        v3 e = V(logx<FAST>(fmaxf(fabsf(sv.x), 1e-4f)), logx<FAST>(fmaxf(fabsf(sv.y), 1e-4f)),
                 logx<FAST>(fmaxf(fabsf(sv.z), 1e-4f)));
        const float tr = (e.x + e.y) + e.z;
        const float tr3 = tr / 3.0f;
        const v3 dev = V(e.x - tr3, e.y - tr3, e.z - tr3);
        const float devn = sqrtx<FAST>(vdot(dev, dev));
        if (tr >= 0.0f) {
          e = V(0.0f, 0.0f, 0.0f);
        } else {
          const float dg = devn + (((3.0f * la0 + 2.0f * mu0) / (2.0f * mu0)) * tr) * m2.x;
          if (dg > 0.0f && devn > 1e-12f) {
            if (FAST) {
              const float r = __fdividef(dg, devn);
              e = V(__fmaf_rn(-r, dev.x, e.x), __fmaf_rn(-r, dev.y, e.y), __fmaf_rn(-r, dev.z, e.z));
            } else {
              e = V(e.x - (dg * dev.x) / devn, e.y - (dg * dev.y) / devn, e.z - (dg * dev.z) / devn);
            }
          }
        }
        const v3 s = V(expx<FAST>(e.x), expx<FAST>(e.y), expx<FAST>(e.z));
        F = mmx<FAST>(mdiag_right(U, s), mT(Vm));
        const float te = (e.x + e.y) + e.z;
        const float tm = 2.0f * mu0;
        const float lt = la0 * te;
        const v3 dd = V(tm * e.x + lt, tm * e.y + lt, tm * e.z + lt);
        const m3 T = mmx<FAST>(mdiag_right(U, dd), mT(U));
        t00 = T.c[0].x; t11 = T.c[1].y; t22 = T.c[2].z;
        t01 = T.c[1].x; t02 = T.c[2].x; t12 = T.c[2].y;
      }
    }
  }
  X = make_float4(nx, ny, nz, X.w);
  Vv = make_float4(v.x, v.y, v.z, vw);
  C0 = make_float4(C.c[0].x, C.c[0].y, C.c[0].z, t00);
  C1 = make_float4(C.c[1].x, C.c[1].y, C.c[1].z, t11);
  C2 = make_float4(C.c[2].x, C.c[2].y, C.c[2].z, t22);
  F0 = make_float4(F.c[0].x, F.c[0].y, F.c[0].z, t01);
  F1 = make_float4(F.c[1].x, F.c[1].y, F.c[1].z, t02);
  F2 = make_float4(F.c[2].x, F.c[2].y, F.c[2].z, t12);
}

// AABB of the bases of the chunk's particles (x of each slot given by xs), into sbox[0..5], which
// arrives empty (see box_empty) and is complete for every thread on return.
template <int PPT>
__device__ __forceinline__ void cta_base_box(const float4 (&xs)[PPT], int count, const int32_t* dims, int* sbox) {
  const int tid = threadIdx.x;
  int lo0 = 0x3fffffff, lo1 = 0x3fffffff, lo2 = 0x3fffffff;
  int hi0 = -0x3fffffff, hi1 = -0x3fffffff, hi2 = -0x3fffffff;
  (void)count;   // lanes past the end hold a copy of the last particle: inside the box already
#pragma unroll
  for (int k = 0; k < PPT; k++) {
    const int b0 = base_of(xs[k].x, dims[0]), b1 = base_of(xs[k].y, dims[1]), b2 = base_of(xs[k].z, dims[2]);
    lo0 = min(lo0, b0); lo1 = min(lo1, b1); lo2 = min(lo2, b2);
    hi0 = max(hi0, b0); hi1 = max(hi1, b1); hi2 = max(hi2, b2);
  }
  lo0 = __reduce_min_sync(0xffffffffu, lo0); lo1 = __reduce_min_sync(0xffffffffu, lo1);
  lo2 = __reduce_min_sync(0xffffffffu, lo2);
  hi0 = __reduce_max_sync(0xffffffffu, hi0); hi1 = __reduce_max_sync(0xffffffffu, hi1);
  hi2 = __reduce_max_sync(0xffffffffu, hi2);
  if ((tid & 31) == 0) {
    atomicMin(&sbox[0], lo0); atomicMin(&sbox[1], lo1); atomicMin(&sbox[2], lo2);
    atomicMax(&sbox[3], hi0); atomicMax(&sbox[4], hi1); atomicMax(&sbox[5], hi2);
  }
  cta_sync();
}

// G2P of a chunk: gather tile (the grid nodes under the chunk's stencils, staged once in shared
// memory), per-particle G2P, store, then the fused P2G of the next substep through the same tile.
// PRE: the launch may hold one-buffer scenes that sort this substep (their old state comes from the
// pregathered scratch); ticks without one run the variant without that path.
// FAST: the world decomposes snow and sand to a tolerance (si_world_set_svd_tolerance).
template <int PPT, bool PRE, bool FAST>
__global__ void __launch_bounds__(kCtaThreads, SI_G2P_MIN_CTAS) k_g2p(TickInfo t, const uint32_t* __restrict__ perm) {
  extern __shared__ __align__(16) int smem[];
  int* tile = smem;
  float4* tilef = reinterpret_cast<float4*>(smem);
  int* gbox = smem + 4 * kTileNodes;   // box of the old stencils (gather tile)
  int* sbox = gbox + 8;                // box of the new bases (scatter tile) and its middle base
  float* sc = reinterpret_cast<float*>(gbox + 24);
  constexpr int chunk = kCtaThreads * PPT;
  const int tid = threadIdx.x;
  // Chunks are handed out in order as CTAs become free: the first wave by CTA index, the rest from a
  // counter that thread 0 bumps at the start of a chunk for the CTA's next one (chunk costs differ by
  // up to 2x with the material and the box, so a fixed stride leaves SMs idle at the end). The slot
  // alternates so that a chunk's write cannot meet a slow warp's read of the previous one.
  __shared__ uint32_t next_chunk[2];
  __shared__ uint32_t scene_tab[kSceneTable];
  scene_table_load<kSceneP>(t, scene_tab);
  box_empty(gbox);
  box_empty(sbox);
  cta_sync();
  uint32_t parity = 0;
  for (uint32_t c = blockIdx.x; c < t.pchunks; c = next_chunk[parity], parity ^= 1u) {
    if (tid == 0) next_chunk[parity] = gridDim.x + atomicAdd(&t.g2p_sched[0], 1u);
    const TickScene& ts = t.ts[scene_of<kSceneP>(t, scene_tab, c)];
    const uint32_t flags = ts.flags;
    const SceneParams* prm = ts.prm;
    const int first = (int)(c - ts.pchunk_begin) * chunk;
    const int count = min(chunk, ts.n - first);
    const bool fuse = (flags & F_FUSE) != 0;
    // a sort substep reads the old state through perm and writes the other buffer, or (one-buffer
    // scene) reads the pregathered copy in sorted order and writes its own buffer in place
    const bool pre = PRE && (flags & F_PREGATHER) != 0;
    const bool gather = (flags & F_GATHER) != 0 && !pre;
    const float4* Pin = pre ? t.gscratch + ts.seg_base : ts.P;
    float4* P = gather ? ts.Palt : ts.P;
    const int64_t cap = ts.cap;
    const int64_t cin = pre ? t.gstride : cap;             // stream stride of Pin
    const int64_t fin = pre ? 2 * t.gstride : 5 * cap;     // offset of Pin's f0 stream
    const float4* grid = reinterpret_cast<const float4*>(ts.grid);
    const int32_t dims[3] = {prm->dims[0], prm->dims[1], prm->dims[2]};
    // 1. positions and the box of the old stencils. Lanes past the end of a partial chunk work on a
    // copy of the chunk's last particle and store nothing: every lane of a warp takes the same path
    // up to each CTA barrier (a barrier completes for a warp once some of its lanes arrive, so lanes
    // must not reach it ahead of their warp-mates).
    float4 xs[PPT];
    int64_t js[PPT];
#pragma unroll
    for (int k = 0; k < PPT; k++) {
      const int slot = min(k * kCtaThreads + tid, count - 1);
      js[k] = gather ? (int64_t)__ldg(&perm[ts.seg_base + first + slot]) : (int64_t)(first + slot);
      xs[k] = __ldcs(&Pin[js[k]]);
    }
    // The loads of J (v.w) and, for the other models, F come after the staging barrier; start them
    // into L1 now, while the box and the gather tile are built (prefetches hold no registers).
#pragma unroll
    for (int k = 0; k < PPT; k++) {
      const int64_t j = js[k];
      asm volatile("prefetch.global.L1 [%0];" ::"l"(reinterpret_cast<const float*>(&Pin[cin + j]) + 3));
      if (__float_as_uint(__ldg(&prm->mats[(__float_as_uint(xs[k].w) & 7u) * 3].x)) != 0u) {
        asm volatile("prefetch.global.L1 [%0];" ::"l"(&Pin[fin + j]));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(&Pin[fin + cin + j]));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(&Pin[fin + 2 * cin + j]));
      }
    }
    cta_base_box<PPT>(xs, count, dims, gbox);
    const int o0 = gbox[0], o1 = gbox[1], o2 = gbox[2];
    const int ex = gbox[3] - o0 + 3, ey = gbox[4] - o1 + 3, ez = gbox[5] - o2 + 3;
    const long long gtn = (long long)ex * ey * ez;
    const bool gtile = ex > 0 && gtn <= t.tile_nodes;
    // 2. stage the gather tile: vec4f(v, m) of every node under the stencils (zero outside the grid)
    if (gtile) {
      tile_walk(ex, ey, ez, [&](int q, int lx, int ly, int lz) {
        const int gx = o0 + lx, gy = o1 + ly, gz = o2 + lz;
        float4 n = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if ((unsigned)gx < (unsigned)dims[0] && (unsigned)gy < (unsigned)dims[1] && (unsigned)gz < (unsigned)dims[2])
          n = __ldg(&grid[(size_t)gx + (size_t)dims[0] * ((size_t)gy + (size_t)dims[1] * (size_t)gz)]);
        tilef[q] = n;
      });
    }
    cta_sync();
    // 3. per-particle G2P
    Scat reg;
#pragma unroll
    for (int k = 0; k < PPT; k++) {
      const bool valid = k * kCtaThreads + tid < count;
      const int slot = min(k * kCtaThreads + tid, count - 1);
      const int64_t i = first + slot, j = js[k];
      // G2P reads x, J (v.w) and F; v.xyz, C and the stress are recomputed (mpm.js:479-559), so their
      // 52 bytes per particle are not loaded. A fluid's F is reset to I (mpm.js:520-525) and its input
      // F is never read, so its 48 bytes are loaded only for the other models.
      float4 x = xs[k];
      float4 v = make_float4(0.0f, 0.0f, 0.0f, __ldcs(reinterpret_cast<const float*>(&Pin[cin + j]) + 3));
      float4 c0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), c1 = c0, c2 = c0;
      float4 f0 = c0, f1 = c0, f2 = c0;
      if (__float_as_uint(__ldg(&prm->mats[(__float_as_uint(x.w) & 7u) * 3].x)) != 0u) {
        f0 = __ldcs(&Pin[fin + j]); f1 = __ldcs(&Pin[fin + cin + j]); f2 = __ldcs(&Pin[fin + 2 * cin + j]);
      }
      Gathered gs;
      if (gtile) gs = g2p_gather<true>(x, prm, grid, tilef, o0, o1, o2, ex, ex * ey, t.nz);
      else gs = g2p_gather<false>(x, prm, grid, tilef, 0, 0, 0, 1, 1, t.nz);
      g2p_update<FAST>(gs, x, v, c0, c1, c2, f0, f1, f2, prm);
      if (valid) {
        __stcs(&P[i], x); __stcs(&P[cap + i], v); __stcs(&P[2 * cap + i], c0); __stcs(&P[3 * cap + i], c1);
        __stcs(&P[4 * cap + i], c2); __stcs(&P[5 * cap + i], f0); __stcs(&P[6 * cap + i], f1);
        __stcs(&P[7 * cap + i], f2);
        if (flags & F_KEYS) ts.keys_next[i] = block_key(x.x, x.y, x.z, prm->num_blocks);
      }
      if (fuse) {
        prep_scatter(reg, x, v, c0, c1, c2, f0.w, f1.w, f2.w, prm);
        if (!valid) scat_silence(reg);
        if (PPT > 1) scat_store(sc, chunk, k * kCtaThreads + tid, reg);
      }
    }
    // 4. P2G of the next substep through the same shared memory; it empties both boxes for the next
    // chunk (every thread read gbox before the staging barrier)
    if (fuse) {
      cta_scatter(reg, true, PPT > 1 ? sc : nullptr, chunk, PPT > 1 ? chunk : count, dims,
                  reinterpret_cast<int*>(ts.grid_next), (flags & F_FORCE_GLOBAL) != 0, t.tile_nodes, tile, sbox, gbox,
                  ts.box_next, t.nz);
    } else {
      box_empty(gbox);
      cta_sync();
    }
  }
  // every CTA has taken its last (failed) chunk number before it counts itself done, so the last
  // one out can reset the counters for the next launch
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&t.g2p_sched[1], 1u) == gridDim.x - 1) {
      t.g2p_sched[0] = 0;
      t.g2p_sched[1] = 0;
      __threadfence();
    }
  }
}

// ------------------------------------------------------------------ keys of the current positions
__global__ void __launch_bounds__(kCtaThreads) k_keys(TickInfo t) {
  const int per = kCtaThreads * (t.chunk / kCtaThreads);
  for (uint32_t chunk = blockIdx.x; chunk < t.pchunks; chunk += gridDim.x) {
    const TickScene& ts = t.ts[find_scene_p(t.ts, t.nscenes, chunk)];
    if (!(ts.flags & F_KEYS_NOW)) continue;
    const int first = (int)(chunk - ts.pchunk_begin) * per;
    const int last = min(first + per, ts.n);
    const uint32_t nb = ts.prm->num_blocks;
    for (int i = first + threadIdx.x; i < last; i += blockDim.x) {
      float4 x = ts.P[i];
      ts.keys[i] = block_key(x.x, x.y, x.z, nb);
    }
  }
}

// ------------------------------------------------------------------ retime (mpm.js:405-413)
__global__ void k_retime(float4* P, int64_t cap, int32_t n, float k) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int r = 1; r <= 4; r++) {
      float4 a = P[r * cap + i];
      P[r * cap + i] = make_float4(a.x * k, a.y * k, a.z * k, a.w);
    }
  }
}

// ------------------------------------------------------------------ record I/O
__global__ void k_aos_to_soa(const float4* __restrict__ aos, float4* P, int64_t cap, int64_t off, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * kStreams; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = t / kStreams; int k = (int)(t % kStreams);
    P[k * cap + off + i] = aos[t];
  }
}
__global__ void k_soa_to_aos(const float4* __restrict__ P, int64_t cap, int64_t off, int64_t n, float4* aos) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * kStreams; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = t / kStreams; int k = (int)(t % kStreams);
    aos[t] = P[k * cap + off + i];
  }
}
// readPositions, mpm.js:627-628: f32(x * dx + origin) evaluated in f64 like JavaScript
__global__ void k_positions(const float4* __restrict__ P, int64_t off, int64_t n, double dx, double o0,
                            double o1, double o2, float* xyz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float4 x = P[off + i];
    xyz[3 * i] = (float)(__dadd_rn(__dmul_rn((double)x.x, dx), o0));
    xyz[3 * i + 1] = (float)(__dadd_rn(__dmul_rn((double)x.y, dx), o1));
    xyz[3 * i + 2] = (float)(__dadd_rn(__dmul_rn((double)x.z, dx), o2));
  }
}

// Instances of the sphere layer (spheres(), mpm.js:658-679; its vertex stage src/render/spheres.js:50-60)
// as a headless buffer: world = x * scale + offset and v * velScale in f32 as the shader computes them,
// the layer's radius, and a radius of 0 for a material the mask culls.
__global__ void k_instances(const float4* __restrict__ P, int64_t cap, int64_t off, int64_t n, float scale, float o0,
                            float o1, float o2, float radius, float vel_scale, uint32_t mat_mask, float4* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 x = P[off + i], v = P[cap + off + i];
    const uint32_t mat = __float_as_uint(x.w);
    const bool keep = ((mat_mask >> (mat & 31u)) & 1u) == 1u;
    out[2 * i] = make_float4(x.x * scale + o0, x.y * scale + o1, x.z * scale + o2, keep ? radius : 0.0f);
    out[2 * i + 1] = make_float4(v.x * vel_scale, v.y * vel_scale, v.z * vel_scale, x.w);
  }
}

// ------------------------------------------------------------------ launchers
int p2g_smem_bytes(int tile_nodes, int ppt) {
  (void)tile_nodes;
  return kTileNodes * 16 + 96 + (ppt > 1 ? kScatWords * 4 * kCtaThreads * ppt : 0);
}
int max_tile_nodes() { return kTileNodes; }

template <int PPT>
static cudaError_t set_smem_attr(int tile_nodes) {
  int bytes = p2g_smem_bytes(tile_nodes, PPT);
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_p2g<PPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    for (const void* k : {(const void*)k_g2p<PPT, false, false>, (const void*)k_g2p<PPT, true, false>,
                          (const void*)k_g2p<PPT, false, true>, (const void*)k_g2p<PPT, true, true>}) {
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

void launch_p2g(const TickInfo& t, int grid_ctas, cudaStream_t st) {
  if (t.pchunks == 0) return;
  int ctas = (int)std::min<uint32_t>(t.pchunks, (uint32_t)grid_ctas);
  int smem = p2g_smem_bytes(t.tile_nodes, t.chunk / kCtaThreads);
  switch (t.chunk / kCtaThreads) {
    case 1: k_p2g<1><<<ctas, kCtaThreads, smem, st>>>(t); break;
    case 4: k_p2g<4><<<ctas, kCtaThreads, smem, st>>>(t); break;
    default: k_p2g<2><<<ctas, kCtaThreads, smem, st>>>(t); break;
  }
}
template <int PPT>
static void launch_g2p_ppt(const TickInfo& t, const uint32_t* perm, int ctas, int smem, cudaStream_t st, bool pre,
                           bool fast) {
  if (pre) {
    if (fast) k_g2p<PPT, true, true><<<ctas, kCtaThreads, smem, st>>>(t, perm);
    else k_g2p<PPT, true, false><<<ctas, kCtaThreads, smem, st>>>(t, perm);
  } else {
    if (fast) k_g2p<PPT, false, true><<<ctas, kCtaThreads, smem, st>>>(t, perm);
    else k_g2p<PPT, false, false><<<ctas, kCtaThreads, smem, st>>>(t, perm);
  }
}
void launch_g2p(const TickInfo& t, const uint32_t* perm, int grid_ctas, cudaStream_t st, bool pre, bool fast) {
  if (t.pchunks == 0) return;
  int ctas = (int)std::min<uint32_t>(t.pchunks, (uint32_t)grid_ctas);
  int smem = p2g_smem_bytes(t.tile_nodes, t.chunk / kCtaThreads);
  switch (t.chunk / kCtaThreads) {
    case 1: launch_g2p_ppt<1>(t, perm, ctas, smem, st, pre, fast); break;
    case 4: launch_g2p_ppt<4>(t, perm, ctas, smem, st, pre, fast); break;
    default: launch_g2p_ppt<2>(t, perm, ctas, smem, st, pre, fast); break;
  }
}
void launch_clear(const TickInfo& t, int grid_ctas, cudaStream_t st) {
  if (t.nchunks == 0) return;
  int ctas = (int)std::min<uint32_t>(t.nchunks, (uint32_t)grid_ctas);
  k_clear<<<ctas, kCtaThreads, 0, st>>>(t);
}
void launch_reorder(const TickInfo& t, const uint32_t* perm, int grid_ctas, cudaStream_t st) {
  if (t.pchunks == 0) return;
  int ctas = (int)std::min<uint32_t>(t.pchunks, (uint32_t)grid_ctas);
  k_reorder<<<ctas, kCtaThreads, 0, st>>>(t, perm);
}
void launch_pregather(const TickInfo& t, const uint32_t* perm, float4* scratch, int64_t stride, int grid_ctas,
                      cudaStream_t st) {
  if (t.pchunks == 0) return;
  int ctas = (int)std::min<uint32_t>(t.pchunks, (uint32_t)grid_ctas);
  k_pregather<<<ctas, kCtaThreads, 0, st>>>(t, perm, scratch, stride);
}
void launch_grid(const TickInfo& t, int grid_ctas, int grid_ctas_wide, cudaStream_t st) {
  if (t.nchunks == 0) return;
  if (t.nscenes > 1) {
    k_grid_wide<<<(int)std::min<uint32_t>(t.nchunks, (uint32_t)grid_ctas_wide), kCtaThreads, 0, st>>>(t);
  } else {
    k_grid<<<(int)std::min<uint32_t>(t.nchunks, (uint32_t)grid_ctas), kCtaThreads, 0, st>>>(t);
  }
}
void launch_box_reset(const TickInfo& t, cudaStream_t st) {
  if (t.nscenes > 0) k_box_reset<<<1, kCtaThreads, 0, st>>>(t);
}
void launch_keys(const TickInfo& t, int grid_ctas, cudaStream_t st) {
  if (t.pchunks == 0) return;
  int ctas = (int)std::min<uint32_t>(t.pchunks, (uint32_t)grid_ctas);
  k_keys<<<ctas, kCtaThreads, 0, st>>>(t);
}
void launch_retime(float4* P, int64_t cap, int32_t n, float k, cudaStream_t st) {
  if (n <= 0) return;
  int ctas = (int)std::min<int64_t>((n + 255) / 256, 4096);
  k_retime<<<ctas, 256, 0, st>>>(P, cap, n, k);
}
void launch_aos_to_soa(const float* aos, float4* P, int64_t cap, int64_t off, int64_t n, cudaStream_t st) {
  if (n <= 0) return;
  int ctas = (int)std::min<int64_t>((n * kStreams + 255) / 256, 8192);
  k_aos_to_soa<<<ctas, 256, 0, st>>>(reinterpret_cast<const float4*>(aos), P, cap, off, n);
}
void launch_soa_to_aos(const float4* P, int64_t cap, int64_t off, int64_t n, float* aos, cudaStream_t st) {
  if (n <= 0) return;
  int ctas = (int)std::min<int64_t>((n * kStreams + 255) / 256, 8192);
  k_soa_to_aos<<<ctas, 256, 0, st>>>(P, cap, off, n, reinterpret_cast<float4*>(aos));
}
void launch_instances(const float4* P, int64_t cap, int64_t off, int64_t n, float scale, const float offset[3],
                      float radius, float vel_scale, uint32_t mat_mask, float* out, cudaStream_t st) {
  if (n <= 0) return;
  int ctas = (int)std::min<int64_t>((n + 255) / 256, 8192);
  k_instances<<<ctas, 256, 0, st>>>(P, cap, off, n, scale, offset[0], offset[1], offset[2], radius, vel_scale, mat_mask,
                                    reinterpret_cast<float4*>(out));
}
void launch_positions(const float4* P, int64_t cap, int64_t off, int64_t n, double dx, const double origin[3],
                      float* xyz, cudaStream_t st) {
  (void)cap;
  if (n <= 0) return;
  int ctas = (int)std::min<int64_t>((n + 255) / 256, 8192);
  k_positions<<<ctas, 256, 0, st>>>(P, off, n, dx, origin[0], origin[1], origin[2], xyz);
}

// Shared-memory opt-ins of the substep kernels and of the one-CTA sort, on the current device (the
// world's): an attribute set on one device does not carry over to another.
cudaError_t configure_kernels(int tile_nodes) {
  cudaError_t e = set_smem_attr<1>(tile_nodes);
  if (e == cudaSuccess) e = set_smem_attr<2>(tile_nodes);
  if (e == cudaSuccess) e = set_smem_attr<4>(tile_nodes);
  if (e == cudaSuccess) e = configure_sort_kernels();
  return e;
}

int occupancy_ctas(int which, int tile_nodes, int ppt) {
  int n = 0;
  int smem = p2g_smem_bytes(tile_nodes, ppt);
  switch (which) {
    case 0:
      if (ppt == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_p2g<1>, kCtaThreads, smem);
      else if (ppt == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_p2g<4>, kCtaThreads, smem);
      else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_p2g<2>, kCtaThreads, smem);
      break;
    case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_g2p<2, false, false>, kCtaThreads, smem); break;
    case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_grid, kCtaThreads, 0); break;
    case 3: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_g2p<1, false, false>, kCtaThreads, smem); break;
    case 4: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_g2p<4, false, false>, kCtaThreads, smem); break;
    case 5: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_grid_wide, kCtaThreads, 0); break;
    default: break;
  }
  return n > 0 ? n : 1;
}

}  // namespace si
