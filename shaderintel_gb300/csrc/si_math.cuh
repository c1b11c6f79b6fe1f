// si_math.cuh — the per-particle arithmetic of the substep, in the fixed f32 evaluation order
// that the CPU oracle also follows (every operation separately rounded: this header is only
// compiled with -fmad=false; IEEE division and square root; no fast-math).
//
// Sources in ShaderIntel v0.3.0: fixed point / B-spline / Morton mpm.js:64-78; linalg
// src/shaders/linalg.js:8-69; constitutive models mpm.js:511-556.
#pragma once
#include <stdint.h>

namespace si {

struct v3 { float x, y, z; };
struct m3 { v3 c[3]; };   // columns

// Packed FP32 pairs (FADD2 / FMUL2 / FFMA2 of sm_100+): each half rounds exactly like the scalar
// add.rn / mul.rn / fma.rn. The scalar path relies on mul.rn and add.rn never being contracted; for
// the packed forms ptxas does contract a mul.rn.f32x2 whose result feeds an add.rn.f32x2 into one
// fma (measured: such a chain equals the fused chain bit for bit, in spite of .rn, a literal -0
// addend or an empty asm barrier). So a product that feeds an add is formed by mul2z as
// fma(x, y, nz) with nz = -0.0f read from the kernel arguments: the compiler cannot drop the
// addend, an add of an fma result is not contracted, and x * y + (-0) rounds exactly like x * y
// (including the sign of a zero product).
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  float2 d;
  asm("{\n .reg .b64 x, y, r;\n mov.b64 x, {%2, %3};\n mov.b64 y, {%4, %5};\n mul.rn.f32x2 r, x, y;\n"
      " mov.b64 {%0, %1}, r;\n}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  float2 d;
  asm("{\n .reg .b64 x, y, r;\n mov.b64 x, {%2, %3};\n mov.b64 y, {%4, %5};\n add.rn.f32x2 r, x, y;\n"
      " mov.b64 {%0, %1}, r;\n}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n .reg .b64 x, y, z, r;\n mov.b64 x, {%2, %3};\n mov.b64 y, {%4, %5};\n mov.b64 z, {%6, %7};\n"
      " fma.rn.f32x2 r, x, y, z;\n mov.b64 {%0, %1}, r;\n}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
__device__ __forceinline__ float2 mul2z(float2 a, float2 b, float nz) { return fma2(a, b, make_float2(nz, nz)); }

__device__ __forceinline__ v3 V(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 vscale(float s, v3 a) { return V(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float vlen(v3 a) { return sqrtf(vdot(a, a)); }
__device__ __forceinline__ v3 vcross(v3 a, v3 b) {
  return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ v3 mv(const m3& m, v3 v) {
  return V((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z,
           (m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z,
           (m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z);
}
__device__ __forceinline__ m3 mm(const m3& a, const m3& b) {
  m3 r; r.c[0] = mv(a, b.c[0]); r.c[1] = mv(a, b.c[1]); r.c[2] = mv(a, b.c[2]); return r;
}
__device__ __forceinline__ m3 mT(const m3& a) {
  m3 r;
  r.c[0] = V(a.c[0].x, a.c[1].x, a.c[2].x);
  r.c[1] = V(a.c[0].y, a.c[1].y, a.c[2].y);
  r.c[2] = V(a.c[0].z, a.c[1].z, a.c[2].z);
  return r;
}
__device__ __forceinline__ float det3(const m3& m) {
  float a = m.c[0].x * (m.c[1].y * m.c[2].z - m.c[2].y * m.c[1].z);
  float b = m.c[1].x * (m.c[0].y * m.c[2].z - m.c[2].y * m.c[0].z);
  float c = m.c[2].x * (m.c[0].y * m.c[1].z - m.c[1].y * m.c[0].z);
  return (a - b) + c;
}
// (U diag(s)) with the zero terms dropped
__device__ __forceinline__ m3 mdiag_right(const m3& u, v3 s) {
  m3 r;
  r.c[0] = V(u.c[0].x * s.x, u.c[0].y * s.x, u.c[0].z * s.x);
  r.c[1] = V(u.c[1].x * s.y, u.c[1].y * s.y, u.c[1].z * s.y);
  r.c[2] = V(u.c[2].x * s.z, u.c[2].y * s.z, u.c[2].z * s.z);
  return r;
}
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// i32(round(clamp(x * 2^22, -2e9, 2e9))), mpm.js:66 (round = nearest-even)
__device__ __forceinline__ int32_t to_fixed(float x) {
  return __float2int_rn(clampf(x * 4194304.0f, -2.0e9f, 2.0e9f));
}

__device__ __forceinline__ uint32_t part1by2(uint32_t x) {
  uint32_t v = x & 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
// block key of mpm.js:567-568; keys past the table (positions outside the grid) clamp to the last bin
__device__ __forceinline__ uint32_t block_key(float x, float y, float z, uint32_t num_blocks) {
  uint32_t bx = ((uint32_t)fminf(fmaxf(x, 0.0f), 16777216.0f)) / 4u;
  uint32_t by = ((uint32_t)fminf(fmaxf(y, 0.0f), 16777216.0f)) / 4u;
  uint32_t bz = ((uint32_t)fminf(fmaxf(z, 0.0f), 16777216.0f)) / 4u;
  uint32_t k = part1by2(bx) | (part1by2(by) << 1) | (part1by2(bz) << 2);
  return k < num_blocks ? k : num_blocks - 1u;
}

// quadratic B-spline weights, mpm.js:67-69
__device__ __forceinline__ void bspline(float f, float w[3]) {
  float a = 1.5f - f, b = f - 1.0f, c = f - 0.5f;
  w[0] = (0.5f * a) * a;
  w[1] = 0.75f - b * b;
  w[2] = (0.5f * c) * c;
}
// floor(x - 0.5); outside the grid (or NaN) -> far outside, so the whole stencil is skipped
__device__ __forceinline__ int32_t base_of(float x, int32_t dim) {
  float b = floorf(x - 0.5f);
  if (!(b >= -4.0f && b <= (float)(dim + 4))) return -1000000;
  return (int32_t)b;
}

// ---- log / exp: Cody & Waite (1980) argument reduction; log m = 2 atanh((m-1)/(m+1)) by its
// Taylor series to s^9, e^r by its Taylor series to r^7. Within 2 ulp; identical bits to the oracle.
__device__ __forceinline__ float si_logf(float x) {
  if (!(x > 0.0f)) return x == 0.0f ? -__int_as_float(0x7f800000) : __int_as_float(0x7fc00000);
  if (x == __int_as_float(0x7f800000)) return x;
  uint32_t b = __float_as_uint(x);
  int32_t e = 0;
  if (b < 0x00800000u) { x = x * 0x1p24f; b = __float_as_uint(x); e = -24; }
  e += (int32_t)(b >> 23) - 127;
  float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
  if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float z = s * s;
  float p = 0x1.c71c72p-4f;
  p = p * z + 0x1.24924ap-3f;
  p = p * z + 0x1.99999ap-3f;
  p = p * z + 0x1.555556p-2f;
  float t = s + s;
  float r = t + t * (z * p);
  float fe = (float)e;
  return fe * 0x1.62e4p-1f + (fe * 0x1.7f7d1cp-20f + r);
}
__device__ __forceinline__ float si_expf(float x) {
  if (x != x) return x;
  if (x > 0x1.62e430p+6f) return __int_as_float(0x7f800000);
  if (x < -0x1.9fe368p+6f) return 0.0f;
  float kf = rintf(x * 0x1.715476p+0f);
  int32_t k = (int32_t)kf;
  float r = (x - kf * 0x1.62e4p-1f) - kf * 0x1.7f7d1cp-20f;
  float p = 0x1.a01a02p-13f;
  p = p * r + 0x1.6c16c2p-10f;
  p = p * r + 0x1.111112p-7f;
  p = p * r + 0x1.555556p-5f;
  p = p * r + 0x1.555556p-3f;
  p = p * r + 0.5f;
  float y = 1.0f + (r + (r * r) * p);
  if (k > 127) { y = y * 2.0f; k -= 1; }
  if (k < -126) {
    y = y * __uint_as_float((uint32_t)(k + 64 + 127) << 23);
    return y * 0x1p-64f;
  }
  return y * __uint_as_float((uint32_t)(k + 127) << 23);
}

// ---- Jacobi rotation of linalg.js:14-25 with the identity terms of J dropped
__device__ __forceinline__ float get(const v3& v, int r) { return r == 0 ? v.x : (r == 1 ? v.y : v.z); }
__device__ __forceinline__ void put(v3& v, int r, float x) { if (r == 0) v.x = x; else if (r == 1) v.y = x; else v.z = x; }

// sg / y with sg = +-1 is +-(1 / y) exactly, and 1 / y is the correctly rounded reciprocal
// (__frcp_rn), cheaper than a general IEEE division. (Packing the rotation updates into FP32 pairs
// was bit-exact too but raised the kernel's spills and cost more on the scenes without SVD.)
template <int p, int q>
__device__ __forceinline__ void jacobi_rotate(m3& A, m3& Vm) {
  float apq = get(A.c[q], p);
  if (fabsf(apq) < 1e-30f) return;
  float theta = (get(A.c[q], q) - get(A.c[p], p)) / (2.0f * apq);
  float sg = theta >= 0.0f ? 1.0f : -1.0f;
  float t = sg * __frcp_rn(fabsf(theta) + sqrtf(theta * theta + 1.0f));
  float c = __frcp_rn(sqrtf(t * t + 1.0f));
  float s = t * c;
  float ns = -s;
  // T = J^T A: rows p and q of every column
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const float ap = get(A.c[j], p), aq = get(A.c[j], q);
    put(A.c[j], p, c * ap + ns * aq);
    put(A.c[j], q, s * ap + c * aq);
  }
  // A' = T J: columns p and q
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float tp = get(A.c[p], i), tq = get(A.c[q], i);
    put(A.c[p], i, tp * c + tq * ns);
    put(A.c[q], i, tp * s + tq * c);
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float vp = get(Vm.c[p], i), vq = get(Vm.c[q], i);
    put(Vm.c[p], i, vp * c + vq * ns);
    put(Vm.c[q], i, vp * s + vq * c);
  }
}

// svd3 of linalg.js:46-69
__device__ __forceinline__ void svd3(const m3& F, m3& U, v3& s_out, m3& Vm) {
  m3 A = mm(mT(F), F);
  Vm.c[0] = V(1.0f, 0.0f, 0.0f); Vm.c[1] = V(0.0f, 1.0f, 0.0f); Vm.c[2] = V(0.0f, 0.0f, 1.0f);
#pragma unroll 1
  for (int sweep = 0; sweep < 4; sweep++) {
    jacobi_rotate<0, 1>(A, Vm);
    jacobi_rotate<0, 2>(A, Vm);
    jacobi_rotate<1, 2>(A, Vm);
  }
  v3 e = V(A.c[0].x, A.c[1].y, A.c[2].z);
  if (e.x < e.y) { e = V(e.y, e.x, e.z); v3 c0 = Vm.c[0]; Vm.c[0] = Vm.c[1]; Vm.c[1] = c0; Vm.c[2] = vneg(Vm.c[2]); }
  if (e.x < e.z) { e = V(e.z, e.y, e.x); v3 c0 = Vm.c[0]; Vm.c[0] = Vm.c[2]; Vm.c[1] = vneg(Vm.c[1]); Vm.c[2] = c0; }
  if (e.y < e.z) { e = V(e.x, e.z, e.y); v3 c1 = Vm.c[1]; Vm.c[0] = vneg(Vm.c[0]); Vm.c[1] = Vm.c[2]; Vm.c[2] = c1; }
  if (det3(Vm) < 0.0f) Vm.c[2] = vneg(Vm.c[2]);
  v3 s = V(sqrtf(fmaxf(e.x, 0.0f)), sqrtf(fmaxf(e.y, 0.0f)), sqrtf(fmaxf(e.z, 0.0f)));
  v3 u0 = mv(F, Vm.c[0]);
  float l0 = vlen(u0);
  v3 u0n = V(u0.x / l0, u0.y / l0, u0.z / l0);
  u0 = l0 > 1e-12f ? u0n : V(1.0f, 0.0f, 0.0f);
  v3 u1 = mv(F, Vm.c[1]);
  float d01 = vdot(u1, u0);
  u1 = vsub(u1, vscale(d01, u0));
  float l1 = vlen(u1);
  if (l1 > 1e-12f) {
    u1 = V(u1.x / l1, u1.y / l1, u1.z / l1);
  } else {
    u1 = fabsf(u0.x) < 0.9f ? V(1.0f, 0.0f, 0.0f) : V(0.0f, 1.0f, 0.0f);
    float d = vdot(u1, u0);
    u1 = vsub(u1, vscale(d, u0));
    float l = vlen(u1);
    u1 = V(u1.x / l, u1.y / l, u1.z / l);
  }
  v3 u2 = vcross(u0, u1);
  if (vdot(mv(F, Vm.c[2]), u2) < 0.0f) s.z = -s.z;
  U.c[0] = u0; U.c[1] = u1; U.c[2] = u2;
  s_out = s;
}

// ---- svd3 to a tolerance instead of bit for bit (worlds with si_world_set_svd_tolerance): the same
// four cyclic Jacobi sweeps on F^T F, eigen sort and Gram-Schmidt U as svd3, but with fused
// multiply-adds, the hardware reciprocal square root and fast division in place of IEEE division and
// square root, and F^T F kept as its six distinct entries. A rotation of the (p, q) plane that zeroes
// a_pq changes a_pp and a_qq by -/+ t a_pq (t = tan of the angle) and mixes a_rp and a_rq (r the third
// index); the other entries do not move. (A float32 model of the sweeps on snow and sand states of the
// plasticity scene leaves off-diagonal residues below 3e-9 of the largest eigenvalue after four
// sweeps, against 1.5e-7 with the rotation applied to all rows and columns.)
struct Sym3 { float d[3]; float o[3]; };   // diagonal, then a_01, a_02, a_12
template <int p, int q> __device__ __forceinline__ constexpr int sym_off() { return p + q - 1; }
template <int p, int q>
__device__ __forceinline__ void jacobi_rotate_fast(Sym3& A, m3& Vm) {
  constexpr int r = 3 - p - q;
  constexpr int pq = sym_off<p, q>();
  constexpr int rp = sym_off<(r < p ? r : p), (r < p ? p : r)>();
  constexpr int rq = sym_off<(r < q ? r : q), (r < q ? q : r)>();
  const float apq = A.o[pq];
  if (fabsf(apq) < 1e-30f) return;
  const float theta = __fdividef(A.d[q] - A.d[p], 2.0f * apq);
  const float h = __fmaf_rn(theta, theta, 1.0f);
  const float root_h = h < 1e30f ? h * rsqrtf(h) : fabsf(theta);   // sqrt(1 + theta^2), also for huge theta
  const float t = __fdividef(theta >= 0.0f ? 1.0f : -1.0f, fabsf(theta) + root_h);
  const float c = rsqrtf(__fmaf_rn(t, t, 1.0f));
  const float s = t * c;
  A.d[p] = __fmaf_rn(-t, apq, A.d[p]);
  A.d[q] = __fmaf_rn(t, apq, A.d[q]);
  A.o[pq] = 0.0f;
  const float arp = A.o[rp], arq = A.o[rq];
  A.o[rp] = __fmaf_rn(c, arp, -s * arq);
  A.o[rq] = __fmaf_rn(s, arp, c * arq);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float vp = get(Vm.c[p], i), vq = get(Vm.c[q], i);
    put(Vm.c[p], i, __fmaf_rn(vp, c, -vq * s));
    put(Vm.c[q], i, __fmaf_rn(vp, s, vq * c));
  }
}

__device__ __forceinline__ float dot_fma(v3 a, v3 b) { return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, a.x * b.x)); }
__device__ __forceinline__ v3 mv_fma(const m3& m, v3 v) {
  return V(__fmaf_rn(m.c[2].x, v.z, __fmaf_rn(m.c[1].x, v.y, m.c[0].x * v.x)),
           __fmaf_rn(m.c[2].y, v.z, __fmaf_rn(m.c[1].y, v.y, m.c[0].y * v.x)),
           __fmaf_rn(m.c[2].z, v.z, __fmaf_rn(m.c[1].z, v.y, m.c[0].z * v.x)));
}

__device__ __forceinline__ m3 mm_fma(const m3& a, const m3& b) {
  m3 r; r.c[0] = mv_fma(a, b.c[0]); r.c[1] = mv_fma(a, b.c[1]); r.c[2] = mv_fma(a, b.c[2]); return r;
}
// The products and transcendental functions of the snow and sand updates: the bit-exact forms, or
// (FAST) fused products and the hardware approximations of log and exp (absolute error below 2^-21
// for log on [0.5, 2], 2 ulp plus a term in |x| for exp).
template <bool FAST> __device__ __forceinline__ m3 mmx(const m3& a, const m3& b) { return FAST ? mm_fma(a, b) : mm(a, b); }
template <bool FAST> __device__ __forceinline__ float logx(float x) { return FAST ? __logf(x) : si_logf(x); }
template <bool FAST> __device__ __forceinline__ float expx(float x) { return FAST ? __expf(x) : si_expf(x); }
// Division and square root: IEEE, or (FAST) the fast division and x rsqrt(x) (x >= 0).
template <bool FAST> __device__ __forceinline__ float divx(float a, float b) { return FAST ? __fdividef(a, b) : a / b; }
template <bool FAST> __device__ __forceinline__ float sqrtx(float x) { return FAST ? (x > 0.0f ? x * rsqrtf(x) : 0.0f) : sqrtf(x); }

__device__ __forceinline__ void svd3_fast(const m3& F, m3& U, v3& s_out, m3& Vm) {
  Sym3 A;
  A.d[0] = dot_fma(F.c[0], F.c[0]); A.d[1] = dot_fma(F.c[1], F.c[1]); A.d[2] = dot_fma(F.c[2], F.c[2]);
  A.o[0] = dot_fma(F.c[0], F.c[1]); A.o[1] = dot_fma(F.c[0], F.c[2]); A.o[2] = dot_fma(F.c[1], F.c[2]);
  Vm.c[0] = V(1.0f, 0.0f, 0.0f); Vm.c[1] = V(0.0f, 1.0f, 0.0f); Vm.c[2] = V(0.0f, 0.0f, 1.0f);
  // Two sweeps bring 95 % of the particles, and three all but a few in ten thousand, to
  // off-diagonals below 2^-24 of the trace (snow and sand states of a deformed scene), where another
  // sweep changes the result only at rounding level; a particle still above that takes the next one,
  // up to four. The test reads the particle's own matrix only, so the result does not depend on the
  // warp it runs in.
#pragma unroll 1
  for (int sweep = 0; sweep < 4; sweep++) {
    if (sweep >= 2 && fmaxf(fabsf(A.o[0]), fmaxf(fabsf(A.o[1]), fabsf(A.o[2]))) <=
                          0x1p-24f * (A.d[0] + A.d[1] + A.d[2]))
      break;
    jacobi_rotate_fast<0, 1>(A, Vm);
    jacobi_rotate_fast<0, 2>(A, Vm);
    jacobi_rotate_fast<1, 2>(A, Vm);
  }
  v3 e = V(A.d[0], A.d[1], A.d[2]);
  if (e.x < e.y) { e = V(e.y, e.x, e.z); v3 c0 = Vm.c[0]; Vm.c[0] = Vm.c[1]; Vm.c[1] = c0; Vm.c[2] = vneg(Vm.c[2]); }
  if (e.x < e.z) { e = V(e.z, e.y, e.x); v3 c0 = Vm.c[0]; Vm.c[0] = Vm.c[2]; Vm.c[1] = vneg(Vm.c[1]); Vm.c[2] = c0; }
  if (e.y < e.z) { e = V(e.x, e.z, e.y); v3 c1 = Vm.c[1]; Vm.c[0] = vneg(Vm.c[0]); Vm.c[1] = Vm.c[2]; Vm.c[2] = c1; }
  if (det3(Vm) < 0.0f) Vm.c[2] = vneg(Vm.c[2]);
  auto root = [](float x) { return x > 0.0f ? x * rsqrtf(x) : 0.0f; };
  v3 s = V(root(e.x), root(e.y), root(e.z));
  v3 u0 = mv_fma(F, Vm.c[0]);
  const float q0 = dot_fma(u0, u0);
  u0 = q0 > 1e-24f ? vscale(rsqrtf(q0), u0) : V(1.0f, 0.0f, 0.0f);
  v3 u1 = mv_fma(F, Vm.c[1]);
  u1 = vsub(u1, vscale(dot_fma(u1, u0), u0));
  const float q1 = dot_fma(u1, u1);
  if (q1 > 1e-24f) {
    u1 = vscale(rsqrtf(q1), u1);
  } else {
    u1 = fabsf(u0.x) < 0.9f ? V(1.0f, 0.0f, 0.0f) : V(0.0f, 1.0f, 0.0f);
    u1 = vsub(u1, vscale(dot_fma(u1, u0), u0));
    u1 = vscale(rsqrtf(dot_fma(u1, u1)), u1);
  }
  const v3 u2 = vcross(u0, u1);
  if (dot_fma(mv_fma(F, Vm.c[2]), u2) < 0.0f) s.z = -s.z;
  U.c[0] = u0; U.c[1] = u1; U.c[2] = u2;
  s_out = s;
}

}  // namespace si
