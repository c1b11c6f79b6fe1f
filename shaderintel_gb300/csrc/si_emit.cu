// si_emit.cu — MPM.add({box | sphere | cylinder}) on the device (mpm.js:207-232 with sampleShape,
// mpm.js:683-714): the same particles, bit for bit, as the host sampler and record conversion.
//
// sampleShape walks a jittered lattice (x fastest) drawing three xorshift32 numbers per point and
// keeps the points inside the shape, in lattice order. xorshift32 is linear over GF(2), so the
// generator state before point L is M^(3L) applied to the seed, M the 32x32 bit matrix of one step:
// the host passes M^(3 * 2^i) for every bit i, and each thread builds its point's state from the bits
// of L. Positions and the inside test are evaluated in f64 like JavaScript (-fmad=false: no
// contraction), rounded to f32 (the Float32Array), then converted to records as add() does. An
// ordered compaction (per-CTA counts, one scan, per-CTA prefix) places the kept points at the
// scene's end in lattice order.
#include <algorithm>

#include "si_device.h"
#include "si_emit.h"

namespace si {

__device__ __forceinline__ uint32_t gf2_apply(const uint32_t* cols, uint32_t v) {
  uint32_t r = 0;
#pragma unroll 8
  for (int j = 0; j < 32; j++) r ^= (0u - ((v >> j) & 1u)) & cols[j];
  return r;
}

__device__ __forceinline__ uint32_t xs_step(uint32_t s) {
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  return s;
}

// Position of lattice point L (world units, f64) and whether it lies inside the shape.
__device__ __forceinline__ bool emit_point(const EmitInfo& e, int64_t L, double p[3]) {
  uint32_t s = e.seed;
  for (int i = 0; i < 32 && (L >> i) != 0; i++)
    if ((L >> i) & 1) s = gf2_apply(e.jump[i], s);
  const int64_t x = L % e.n[0], y = (L / e.n[0]) % e.n[1], z = L / (e.n[0] * e.n[1]);
  const int64_t q[3] = {x, y, z};
  for (int a = 0; a < 3; a++) {
    s = xs_step(s);
    const double r = (double)s / 4294967296.0;
    p[a] = e.lo[a] + (((double)q[a] + 0.5) + (r - 0.5) * e.jitter) * e.spacing;
  }
  if (e.shape == 1) {
    const double d0 = p[0] - e.a[0], d1 = p[1] - e.a[1], d2 = p[2] - e.a[2];
    return (d0 * d0 + d1 * d1) + d2 * d2 <= e.r * e.r;
  }
  if (e.shape == 2) {
    const double d0 = p[0] - e.a[0], d2 = p[2] - e.a[2];
    return d0 * d0 + d2 * d2 <= e.r * e.r;
  }
  return true;
}

__global__ void __launch_bounds__(256) k_emit_count(EmitInfo e, uint32_t* cta_counts) {
  const int64_t L = (int64_t)blockIdx.x * 256 + threadIdx.x;
  double p[3];
  const bool in = L < e.total && emit_point(e, L, p);
  const int c = __syncthreads_count(in);
  if (threadIdx.x == 0) cta_counts[blockIdx.x] = (uint32_t)c;
}

// Exclusive scan of the per-CTA counts in place; counts[n] = total.
__global__ void __launch_bounds__(1024) k_emit_scan(uint32_t* counts, uint32_t n) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (n + 1023) / 1024;
  const uint32_t b = threadIdx.x * per, e = min(b + per, n);
  uint32_t sum = 0;
  for (uint32_t i = b; i < e; i++) sum += counts[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {   // inclusive Hillis-Steele scan of the parts
    const uint32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - sum;
  for (uint32_t i = b; i < e; i++) {
    const uint32_t c = counts[i];
    counts[i] = run;
    run += c;
  }
  if (threadIdx.x == 1023) counts[n] = part[1023];
}

__global__ void __launch_bounds__(256) k_emit_write(EmitInfo e, const uint32_t* offsets) {
  __shared__ uint32_t wsum[8];
  const int64_t L = (int64_t)blockIdx.x * 256 + threadIdx.x;
  double p[3];
  const bool in = L < e.total && emit_point(e, L, p);
  const unsigned bal = __ballot_sync(0xffffffffu, in);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wsum[warp] = __popc(bal);
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; w++) before += wsum[w];
  before += __popc(bal & ((1u << lane) - 1u));
  const int64_t k = (int64_t)offsets[blockIdx.x] + before;
  if (!in || k >= e.room) return;
  // add(), mpm.js:216-226: x = (f32(p) - origin) / dx clamped into [bound + 1e-3, dims - bound - 1e-3]
  float4 x;
  float c[3];
  for (int a = 0; a < 3; a++) {
    const double xf = (double)(float)p[a];
    const double v = (xf - e.origin[a]) / e.dx;
    const double lo = e.bound + 1e-3, hi = e.hi[a] - 1e-3;
    const double m = v > lo ? v : lo;   // Math.max(lo + 1e-3, x); x is never NaN here
    c[a] = (float)(m < hi ? m : hi);
  }
  x = make_float4(c[0], c[1], c[2], __uint_as_float(e.material));
  const int64_t i = e.offset + k;
  float4* P = e.P;
  const int64_t cap = e.cap;
  P[i] = x;
  P[cap + i] = make_float4(e.vel[0], e.vel[1], e.vel[2], 1.0f);
  const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  P[2 * cap + i] = z;
  P[3 * cap + i] = z;
  P[4 * cap + i] = z;
  P[5 * cap + i] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
  P[6 * cap + i] = make_float4(0.0f, 1.0f, 0.0f, 0.0f);
  P[7 * cap + i] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
}

int launch_emit(const EmitInfo& e, uint32_t* scratch, cudaStream_t st) {
  const uint32_t ctas = (uint32_t)((e.total + 255) / 256);
  k_emit_count<<<ctas, 256, 0, st>>>(e, scratch);
  k_emit_scan<<<1, 1024, 0, st>>>(scratch, ctas);
  k_emit_write<<<ctas, 256, 0, st>>>(e, scratch);
  return (int)cudaGetLastError();
}

}  // namespace si
