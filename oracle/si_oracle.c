/*
 * si_oracle.c — CPU restatement of the ShaderIntel MLS-MPM substep (TEST INFRASTRUCTURE ONLY).
 * See si_oracle.h for the file:line map into the reference and the canonical evaluation order.
 * Build: -std=c11 -O2 -ffp-contract=off -Wdouble-promotion (every literal is an f32 literal).
 */
#include "si_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FP_SCALE 4194304.0f              /* 2^22, mpm.js:64 */
#define INV_FP (1.0f / 4194304.0f)       /* mpm.js:65 */

typedef struct { float x, y, z; } v3;
typedef struct { v3 c[3]; } m3;          /* columns */

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline int32_t f2i_bits(float f) { int32_t i; memcpy(&i, &f, 4); return i; }
static inline float i2f_bits(int32_t i) { float f; memcpy(&f, &i, 4); return f; }

static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline float vget(v3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vscale(float s, v3 a) { return V(s * a.x, s * a.y, s * a.z); }
static inline float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline float vlen(v3 a) { return sqrtf(vdot(a, a)); }
static inline v3 vcross(v3 a, v3 b) {
  return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* mat * vec: (c0*v.x + c1*v.y) + c2*v.z per component */
static inline v3 mv(m3 m, v3 v) {
  return V((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z,
           (m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z,
           (m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z);
}
static inline m3 mm(m3 a, m3 b) { m3 r; for (int j = 0; j < 3; j++) r.c[j] = mv(a, b.c[j]); return r; }
static inline m3 mT(m3 a) {
  m3 r;
  r.c[0] = V(a.c[0].x, a.c[1].x, a.c[2].x);
  r.c[1] = V(a.c[0].y, a.c[1].y, a.c[2].y);
  r.c[2] = V(a.c[0].z, a.c[1].z, a.c[2].z);
  return r;
}
static inline float mel(m3 a, int col, int row) { return vget(a.c[col], row); }
static inline void mset(m3* a, int col, int row, float v) {
  if (row == 0) a->c[col].x = v; else if (row == 1) a->c[col].y = v; else a->c[col].z = v;
}
static inline float sio_det3(m3 m) {
  float a = m.c[0].x * (m.c[1].y * m.c[2].z - m.c[2].y * m.c[1].z);
  float b = m.c[1].x * (m.c[0].y * m.c[2].z - m.c[2].y * m.c[0].z);
  float c = m.c[2].x * (m.c[0].y * m.c[1].z - m.c[1].y * m.c[0].z);
  return (a - b) + c;
}
static inline float trace3(m3 m) { return (m.c[0].x + m.c[1].y) + m.c[2].z; }
/* (U diag(s)) with the zero terms dropped: column j = U_j * s_j */
static inline m3 mdiag_right(m3 u, v3 s) {
  m3 r;
  r.c[0] = V(u.c[0].x * s.x, u.c[0].y * s.x, u.c[0].z * s.x);
  r.c[1] = V(u.c[1].x * s.y, u.c[1].y * s.y, u.c[1].z * s.y);
  r.c[2] = V(u.c[2].x * s.z, u.c[2].y * s.z, u.c[2].z * s.z);
  return r;
}
static inline float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

/* ------------------------------------------------------------------ log / exp */
/* Natural log for finite x > 0 (Cody & Waite 1980 reduction x = 2^e m, m in [sqrt(1/2), sqrt(2));
 * log m = 2 atanh((m-1)/(m+1)) by its Taylor series to s^9). */
float sio_logf(float x) {
  if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
  if (x == INFINITY) return x;
  uint32_t b = f2u(x);
  int32_t e = 0;
  if (b < 0x00800000u) { x = x * 0x1p24f; b = f2u(x); e = -24; }
  e += (int32_t)(b >> 23) - 127;
  float m = u2f((b & 0x007fffffu) | 0x3f800000u);
  if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float z = s * s;
  float p = 0x1.c71c72p-4f;            /* 1/9 */
  p = p * z + 0x1.24924ap-3f;          /* 1/7 */
  p = p * z + 0x1.99999ap-3f;          /* 1/5 */
  p = p * z + 0x1.555556p-2f;          /* 1/3 */
  float t = s + s;
  float r = t + t * (z * p);
  float fe = (float)e;
  return fe * 0x1.62e4p-1f + (fe * 0x1.7f7d1cp-20f + r);
}

/* e^x (Cody & Waite reduction x = k ln2 + r, |r| <= ln2/2; Taylor series of e^r to r^7). */
float sio_expf(float x) {
  if (x != x) return x;
  if (x > 0x1.62e430p+6f) return INFINITY;
  if (x < -0x1.9fe368p+6f) return 0.0f;
  float kf = rintf(x * 0x1.715476p+0f);
  int32_t k = (int32_t)kf;
  float r = (x - kf * 0x1.62e4p-1f) - kf * 0x1.7f7d1cp-20f;
  float p = 0x1.a01a02p-13f;           /* 1/5040 */
  p = p * r + 0x1.6c16c2p-10f;         /* 1/720 */
  p = p * r + 0x1.111112p-7f;          /* 1/120 */
  p = p * r + 0x1.555556p-5f;          /* 1/24 */
  p = p * r + 0x1.555556p-3f;          /* 1/6 */
  p = p * r + 0.5f;
  float y = 1.0f + (r + (r * r) * p);
  if (k > 127) { y = y * 2.0f; k -= 1; }
  if (k < -126) {
    y = y * u2f((uint32_t)(k + 64 + 127) << 23);
    return y * 0x1p-64f;
  }
  return y * u2f((uint32_t)(k + 127) << 23);
}

/* ------------------------------------------------------------------ linalg.js */
/* si_jacobiRotate, linalg.js:14-25: A = Jᵀ A J, V = V J with the rotation's identity terms dropped. */
static void jacobi_rotate(m3* A, m3* Vm, int p, int q) {
  float apq = mel(*A, q, p);
  if (fabsf(apq) < 1e-30f) return;
  float theta = (mel(*A, q, q) - mel(*A, p, p)) / (2.0f * apq);
  float sg = theta >= 0.0f ? 1.0f : -1.0f;
  float t = sg / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
  float c = 1.0f / sqrtf(t * t + 1.0f);
  float s = t * c;
  float ns = -s;
  /* T = Jᵀ A: rows p and q change. T[j][p] = c*A[j][p] + (-s)*A[j][q]; T[j][q] = s*A[j][p] + c*A[j][q] */
  m3 T = *A;
  for (int j = 0; j < 3; j++) {
    float ap = mel(*A, j, p), aq = mel(*A, j, q);
    mset(&T, j, p, c * ap + ns * aq);
    mset(&T, j, q, s * ap + c * aq);
  }
  /* A' = T J: columns p and q change. A'[p][i] = T[p][i]*c + T[q][i]*(-s); A'[q][i] = T[p][i]*s + T[q][i]*c */
  m3 R = T;
  for (int i = 0; i < 3; i++) {
    float tp = mel(T, p, i), tq = mel(T, q, i);
    mset(&R, p, i, tp * c + tq * ns);
    mset(&R, q, i, tp * s + tq * c);
  }
  *A = R;
  m3 W = *Vm;
  for (int i = 0; i < 3; i++) {
    float vp = mel(*Vm, p, i), vq = mel(*Vm, q, i);
    mset(&W, p, i, vp * c + vq * ns);
    mset(&W, q, i, vp * s + vq * c);
  }
  *Vm = W;
}

static const m3 I3 = {{{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}}};

static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }

/* svd3, linalg.js:46-69 */
static void svd3(m3 F, m3* U, v3* s_out, m3* Vout) {
  m3 A = mm(mT(F), F);
  m3 Vm = I3;
  for (int sweep = 0; sweep < 4; sweep++) {
    jacobi_rotate(&A, &Vm, 0, 1);
    jacobi_rotate(&A, &Vm, 0, 2);
    jacobi_rotate(&A, &Vm, 1, 2);
  }
  v3 e = V(A.c[0].x, A.c[1].y, A.c[2].z);
  if (e.x < e.y) { e = V(e.y, e.x, e.z); m3 W = {{Vm.c[1], Vm.c[0], vneg(Vm.c[2])}}; Vm = W; }
  if (e.x < e.z) { e = V(e.z, e.y, e.x); m3 W = {{Vm.c[2], vneg(Vm.c[1]), Vm.c[0]}}; Vm = W; }
  if (e.y < e.z) { e = V(e.x, e.z, e.y); m3 W = {{vneg(Vm.c[0]), Vm.c[2], Vm.c[1]}}; Vm = W; }
  if (sio_det3(Vm) < 0.0f) Vm.c[2] = vneg(Vm.c[2]);
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
  U->c[0] = u0; U->c[1] = u1; U->c[2] = u2;
  *s_out = s;
  *Vout = Vm;
}

void sio_svd3(const float* F, float* U, float* s, float* Vo) {
  m3 f, u, vv; v3 sv;
  for (int j = 0; j < 3; j++) f.c[j] = V(F[3 * j], F[3 * j + 1], F[3 * j + 2]);
  svd3(f, &u, &sv, &vv);
  for (int j = 0; j < 3; j++) {
    U[3 * j] = u.c[j].x; U[3 * j + 1] = u.c[j].y; U[3 * j + 2] = u.c[j].z;
    Vo[3 * j] = vv.c[j].x; Vo[3 * j + 1] = vv.c[j].y; Vo[3 * j + 2] = vv.c[j].z;
  }
  s[0] = sv.x; s[1] = sv.y; s[2] = sv.z;
}

/* ------------------------------------------------------------------ mpm.js:64-78 */
static inline int32_t to_fixed(float x) {
  return (int32_t)rintf(clampf(x * FP_SCALE, -2.0e9f, 2.0e9f));
}
static inline uint32_t part1by2(uint32_t x) {
  uint32_t v = x & 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
uint32_t sio_morton3(uint32_t x, uint32_t y, uint32_t z) {
  return part1by2(x) | (part1by2(y) << 1) | (part1by2(z) << 2);
}
uint32_t sio_num_blocks(const int32_t dims[3]) {
  int32_t bmax = 0;
  for (int a = 0; a < 3; a++) { int32_t b = (dims[a] + 3) / 4; if (b > bmax) bmax = b; }
  uint32_t bpow = 1;
  while ((int32_t)bpow < bmax) bpow <<= 1;
  return bpow * bpow * bpow;
}

/* B-spline weights, mpm.js:67-69: w0 = 0.5(1.5-f)(1.5-f), w1 = 0.75-(f-1)(f-1), w2 = 0.5(f-0.5)(f-0.5) */
static inline void bspline(float f, float w[3]) {
  float a = 1.5f - f, b = f - 1.0f, c = f - 0.5f;
  w[0] = (0.5f * a) * a;
  w[1] = 0.75f - b * b;
  w[2] = (0.5f * c) * c;
}

/* base = floor(x - 0.5) with the stencil guard: out-of-grid or NaN positions get a base far
 * outside the grid, so every node of their stencil is skipped (P2G) or reads zero (G2P). */
static inline int32_t base_of(float x, int32_t dim) {
  float b = floorf(x - 0.5f);
  if (!(b >= -4.0f && b <= (float)(dim + 4))) return -1000000;
  return (int32_t)b;
}

/* ------------------------------------------------------------------ block sort, mpm.js:563-577 */
static inline uint32_t key_of(const float* p, uint32_t num_blocks) {
  uint32_t b[3];
  for (int a = 0; a < 3; a++) {
    float x = fminf(fmaxf(p[a], 0.0f), 16777216.0f);
    b[a] = ((uint32_t)x) / 4u;
  }
  uint32_t k = sio_morton3(b[0], b[1], b[2]);
  return k < num_blocks ? k : num_blocks - 1u;
}

void sio_keys(const float* P, int64_t n, uint32_t num_blocks, uint32_t* keys) {
  for (int64_t i = 0; i < n; i++) keys[i] = key_of(P + SIO_PF * i, num_blocks);
}

void sio_bins(const uint32_t* keys, int64_t n, uint32_t num_blocks, uint32_t* starts) {
  memset(starts, 0, sizeof(uint32_t) * ((size_t)num_blocks + 1));
  for (int64_t i = 0; i < n; i++) starts[keys[i]]++;
  uint32_t acc = 0;
  for (uint32_t k = 0; k <= num_blocks; k++) { uint32_t c = starts[k]; starts[k] = acc; acc += c; }
}

void sio_sort(const float* src, float* dst, int64_t n, uint32_t num_blocks,
              uint32_t* keys_out, uint32_t* starts_out, uint32_t* perm) {
  uint32_t* keys = keys_out ? keys_out : (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
  uint32_t* starts = starts_out ? starts_out : (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)num_blocks + 1));
  uint32_t* next = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)num_blocks + 1));
  sio_keys(src, n, num_blocks, keys);
  sio_bins(keys, n, num_blocks, starts);
  memcpy(next, starts, sizeof(uint32_t) * ((size_t)num_blocks + 1));
  for (int64_t i = 0; i < n; i++) {
    uint32_t d = next[keys[i]]++;
    if (dst) memcpy(dst + SIO_PF * (size_t)d, src + SIO_PF * (size_t)i, sizeof(float) * SIO_PF);
    if (perm) perm[d] = (uint32_t)i;
  }
  free(next);
  if (!keys_out) free(keys);
  if (!starts_out) free(starts);
}

/* ------------------------------------------------------------------ P2G, mpm.js:318-350 */
static void scatter_one(const float* p, const int32_t dims[3], const float* mats, float vol4,
                        uint32_t* grid) {
  v3 xp = V(p[0], p[1], p[2]);
  int32_t base[3] = {base_of(xp.x, dims[0]), base_of(xp.y, dims[1]), base_of(xp.z, dims[2])};
  v3 fx = V(xp.x - (float)base[0], xp.y - (float)base[1], xp.z - (float)base[2]);
  float w[3][3];
  bspline(fx.x, w[0]); bspline(fx.y, w[1]); bspline(fx.z, w[2]);
  uint32_t mid = f2u(p[3]) & 7u;
  float mass = mats[mid * 12 + 1];
  m3 tau = {{V(p[11], p[23], p[27]), V(p[23], p[15], p[31]), V(p[27], p[31], p[19])}};
  m3 C = {{V(p[8], p[9], p[10]), V(p[12], p[13], p[14]), V(p[16], p[17], p[18])}};
  float nv = -vol4;
  m3 aff;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) mset(&aff, j, i, nv * mel(tau, j, i) + mass * mel(C, j, i));
  v3 mvel = V(mass * p[4], mass * p[5], mass * p[6]);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 3; c++) {
        int32_t g[3] = {base[0] + a, base[1] + b, base[2] + c};
        if (g[0] < 0 || g[0] >= dims[0] || g[1] < 0 || g[1] >= dims[1] || g[2] < 0 || g[2] >= dims[2]) continue;
        v3 dpos = V((float)a - fx.x, (float)b - fx.y, (float)c - fx.z);
        float wt = (w[0][a] * w[1][b]) * w[2][c];
        v3 ad = mv(aff, dpos);
        v3 mom = V(wt * (mvel.x + ad.x), wt * (mvel.y + ad.y), wt * (mvel.z + ad.z));
        int32_t q[4] = {to_fixed(mom.x), to_fixed(mom.y), to_fixed(mom.z), to_fixed(wt * mass)};
        size_t gi = 4 * ((size_t)g[0] + (size_t)dims[0] * ((size_t)g[1] + (size_t)dims[1] * (size_t)g[2]));
        for (int k = 0; k < 4; k++) __atomic_fetch_add(&grid[gi + k], (uint32_t)q[k], __ATOMIC_RELAXED);
      }
}

void sio_p2g(const float* P, int64_t n, const int32_t dims[3], const float* mats, float vol4,
             int32_t* grid, int threads) {
  size_t nodes = (size_t)dims[0] * (size_t)dims[1] * (size_t)dims[2];
  memset(grid, 0, nodes * 16);
  (void)threads;
#pragma omp parallel for schedule(static, 4096) num_threads(threads > 0 ? threads : 1)
  for (int64_t i = 0; i < n; i++) scatter_one(P + SIO_PF * i, dims, mats, vol4, (uint32_t*)grid);
}

/* ------------------------------------------------------------------ grid update, mpm.js:419-470 */
static float collider_sdf(uint32_t kind, v3 d, const float* s) {
  if (kind == 0u) return vlen(d) - s[0];
  if (kind == 1u) {
    v3 q = V(fabsf(d.x) - s[0], fabsf(d.y) - s[1], fabsf(d.z) - s[2]);
    v3 qm = V(fmaxf(q.x, 0.0f), fmaxf(q.y, 0.0f), fmaxf(q.z, 0.0f));
    return vlen(qm) + fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f);
  }
  return vdot(d, V(s[0], s[1], s[2]));
}

static void grid_node(int32_t* g4, int64_t i, const int32_t dims[3], const float grav[3], float bound,
                      const float* cols, int ncol, float ff) {
  int32_t g[4] = {g4[0], g4[1], g4[2], g4[3]};
  float out[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  if (g[3] > 0) {
    float m = (float)g[3] * INV_FP;
    v3 v = V(((float)g[0] * INV_FP) / m + grav[0], ((float)g[1] * INV_FP) / m + grav[1],
             ((float)g[2] * INV_FP) / m + grav[2]);
    int64_t X = dims[0], Y = dims[1];
    v3 c = V((float)(i % X), (float)((i / X) % Y), (float)(i / (X * Y)));
    v3 hi = V((float)dims[0] - bound, (float)dims[1] - bound, (float)dims[2] - bound);
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
      const float* h = cols + 12 * k;
      const float* s = h + 4;
      v3 cv = V(h[8], h[9], h[10]);
      uint32_t kind = f2u(h[0]);
      v3 d = V(c.x - h[1], c.y - h[2], c.z - h[3]);
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
          if (vt > 1e-9f) vr = vscale(fmaxf(0.0f, 1.0f - (s[3] * -vn) / vt), vr);
          v = vadd(vr, cv);
        }
      }
    }
    out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = m;
  }
  for (int k = 0; k < 4; k++) g4[k] = f2i_bits(out[k]);
}

void sio_grid_update(int32_t* grid, const int32_t dims[3], const float gravity[3], float bound,
                     const float* cols, int ncol, float floor_friction, int threads) {
  int64_t nodes = (int64_t)dims[0] * dims[1] * dims[2];
  (void)threads;
#pragma omp parallel for schedule(static, 8192) num_threads(threads > 0 ? threads : 1)
  for (int64_t i = 0; i < nodes; i++)
    grid_node(grid + 4 * i, i, dims, gravity, bound, cols, ncol, floor_friction);
}

/* ------------------------------------------------------------------ G2P, mpm.js:479-559 */
static void g2p_one(float* p, const int32_t dims[3], const int32_t* grid, const float* mats,
                    float bound, float vmax) {
  v3 xp = V(p[0], p[1], p[2]);
  int32_t base[3] = {base_of(xp.x, dims[0]), base_of(xp.y, dims[1]), base_of(xp.z, dims[2])};
  v3 fx = V(xp.x - (float)base[0], xp.y - (float)base[1], xp.z - (float)base[2]);
  float w[3][3];
  bspline(fx.x, w[0]); bspline(fx.y, w[1]); bspline(fx.z, w[2]);
  v3 v = V(0.0f, 0.0f, 0.0f);
  m3 B = {{V(0.0f, 0.0f, 0.0f), V(0.0f, 0.0f, 0.0f), V(0.0f, 0.0f, 0.0f)}};
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 3; c++) {
        v3 dpos = V((float)a - fx.x, (float)b - fx.y, (float)c - fx.z);
        float wt = (w[0][a] * w[1][b]) * w[2][c];
        int32_t g[3] = {base[0] + a, base[1] + b, base[2] + c};
        v3 gv = V(0.0f, 0.0f, 0.0f);
        if (!(g[0] < 0 || g[0] >= dims[0] || g[1] < 0 || g[1] >= dims[1] || g[2] < 0 || g[2] >= dims[2])) {
          const int32_t* n = grid + 4 * ((size_t)g[0] + (size_t)dims[0] * ((size_t)g[1] + (size_t)dims[1] * (size_t)g[2]));
          gv = V(i2f_bits(n[0]), i2f_bits(n[1]), i2f_bits(n[2]));
        }
        v3 t = vscale(wt, gv);
        v = vadd(v, t);
        /* B += outer3(t, dpos) (linalg.js outer3: column k = t * dpos_k), unfused */
        B.c[0] = V(B.c[0].x + t.x * dpos.x, B.c[0].y + t.y * dpos.x, B.c[0].z + t.z * dpos.x);
        B.c[1] = V(B.c[1].x + t.x * dpos.y, B.c[1].y + t.y * dpos.y, B.c[1].z + t.z * dpos.y);
        B.c[2] = V(B.c[2].x + t.x * dpos.z, B.c[2].y + t.y * dpos.z, B.c[2].z + t.z * dpos.z);
      }
  m3 C;
  for (int j = 0; j < 3; j++) C.c[j] = vscale(4.0f, B.c[j]);
  float sp = vlen(v);
  if (sp > vmax) v = vscale(vmax / sp, v);
  float lo = bound - 1.0f;
  v3 x = V(clampf(xp.x + v.x, lo, ((float)dims[0] - bound) + 1.0f),
           clampf(xp.y + v.y, lo, ((float)dims[1] - bound) + 1.0f),
           clampf(xp.z + v.z, lo, ((float)dims[2] - bound) + 1.0f));
  uint32_t mid = f2u(p[3]) & 7u;
  const float* m0 = mats + mid * 12;
  const float* m1 = m0 + 4;
  const float* m2 = m0 + 8;
  uint32_t kind = f2u(m0[0]);
  m3 F = {{V(p[20], p[21], p[22]), V(p[24], p[25], p[26]), V(p[28], p[29], p[30])}};
  m3 tau = {{V(0.0f, 0.0f, 0.0f), V(0.0f, 0.0f, 0.0f), V(0.0f, 0.0f, 0.0f)}};
  float vw = p[7];
  if (kind == 0u) {
    float J = clampf(vw * (1.0f + trace3(C)), 0.6f, 1.4f);
    vw = J;
    float a = m0[2] * fminf(J - 1.0f, 0.02f);
    float b = m1[0] * J;
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++)
        mset(&tau, j, i, a * mel(I3, j, i) + b * (mel(C, j, i) + mel(C, i, j)));
    F = I3;
  } else {
    m3 IC;
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) mset(&IC, j, i, mel(I3, j, i) + mel(C, j, i));
    F = mm(IC, F);
    float mu0 = m0[2], la0 = m0[3];
    if (kind == 1u) {
      float J = fmaxf(sio_det3(F), 0.05f);
      m3 FFt = mm(F, mT(F));
      float l = la0 * sio_logf(J);
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++)
          mset(&tau, j, i, mu0 * (mel(FFt, j, i) - mel(I3, j, i)) + l * mel(I3, j, i));
    } else if (kind == 2u) {
      m3 U, Vm; v3 sv;
      svd3(F, &U, &sv, &Vm);
      float lo_s = 1.0f - m1[2], hi_s = 1.0f + m1[3];
      v3 s = V(clampf(sv.x, lo_s, hi_s), clampf(sv.y, lo_s, hi_s), clampf(sv.z, lo_s, hi_s));
      float Jold = (sv.x * sv.y) * sv.z;
      float Jnew = (s.x * s.y) * s.z;
      vw = clampf((vw * Jold) / Jnew, 0.6f, 20.0f);
      F = mm(mdiag_right(U, s), mT(Vm));
      float h = sio_expf(m1[1] * (1.0f - vw));
      float mu = mu0 * h, la = la0 * h;
      m3 R = mm(U, mT(Vm));
      float J = Jnew;
      float tm = 2.0f * mu;
      m3 FR;
      for (int j = 0; j < 3; j++) FR.c[j] = vscale(tm, vsub(F.c[j], R.c[j]));
      m3 P1 = mm(FR, mT(F));
      float l = (la * J) * (J - 1.0f);
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) mset(&tau, j, i, mel(P1, j, i) + l * mel(I3, j, i));
    } else {
      m3 U, Vm; v3 sv;
      svd3(F, &U, &sv, &Vm);
      v3 e = V(sio_logf(fmaxf(fabsf(sv.x), 1e-4f)), sio_logf(fmaxf(fabsf(sv.y), 1e-4f)),
               sio_logf(fmaxf(fabsf(sv.z), 1e-4f)));
      float tr = (e.x + e.y) + e.z;
      float tr3 = tr / 3.0f;
      v3 dev = V(e.x - tr3, e.y - tr3, e.z - tr3);
      float devn = vlen(dev);
      if (tr >= 0.0f) {
        e = V(0.0f, 0.0f, 0.0f);
      } else {
        float dg = devn + (((3.0f * la0 + 2.0f * mu0) / (2.0f * mu0)) * tr) * m2[0];
        if (dg > 0.0f && devn > 1e-12f)
          e = V(e.x - (dg * dev.x) / devn, e.y - (dg * dev.y) / devn, e.z - (dg * dev.z) / devn);
      }
      v3 s = V(sio_expf(e.x), sio_expf(e.y), sio_expf(e.z));
      F = mm(mdiag_right(U, s), mT(Vm));
      float te = (e.x + e.y) + e.z;
      float tm = 2.0f * mu0;
      float lt = la0 * te;
      v3 dd = V(tm * e.x + lt, tm * e.y + lt, tm * e.z + lt);
      tau = mm(mdiag_right(U, dd), mT(U));
    }
  }
  p[0] = x.x; p[1] = x.y; p[2] = x.z;
  p[4] = v.x; p[5] = v.y; p[6] = v.z; p[7] = vw;
  p[8] = C.c[0].x; p[9] = C.c[0].y; p[10] = C.c[0].z; p[11] = tau.c[0].x;
  p[12] = C.c[1].x; p[13] = C.c[1].y; p[14] = C.c[1].z; p[15] = tau.c[1].y;
  p[16] = C.c[2].x; p[17] = C.c[2].y; p[18] = C.c[2].z; p[19] = tau.c[2].z;
  p[20] = F.c[0].x; p[21] = F.c[0].y; p[22] = F.c[0].z; p[23] = tau.c[1].x;
  p[24] = F.c[1].x; p[25] = F.c[1].y; p[26] = F.c[1].z; p[27] = tau.c[2].x;
  p[28] = F.c[2].x; p[29] = F.c[2].y; p[30] = F.c[2].z; p[31] = tau.c[2].y;
}

void sio_g2p(float* P, int64_t n, const int32_t dims[3], const int32_t* grid, const float* mats,
             float bound, float vmax, int threads) {
  (void)threads;
#pragma omp parallel for schedule(static, 1024) num_threads(threads > 0 ? threads : 1)
  for (int64_t i = 0; i < n; i++) g2p_one(P + SIO_PF * i, dims, grid, mats, bound, vmax);
}

/* ------------------------------------------------------------------ retime, mpm.js:405-413 */
void sio_retime(float* P, int64_t n, float k) {
  for (int64_t i = 0; i < n; i++) {
    float* p = P + SIO_PF * i;
    for (int r = 1; r <= 4; r++)
      for (int a = 0; a < 3; a++) p[4 * r + a] = p[4 * r + a] * k;
  }
}

/* ------------------------------------------------------------------ coupling, coupling.js:31-196 */
#define SIO_MAXC 128          /* MAX_CAND, coupling.js:25 */
#define SIO_FPJ 16384.0f      /* coupling.js:26 */
#define SIO_FPL 1024.0f       /* coupling.js:27 */
#define SIO_F_SENSOR 2u       /* rigid-wgsl.js:35-36 */
#define SIO_F_DISABLED 4u

/* qmat, src/shaders/math.js:56-62 (columns) */
static m3 qmat(const float* q) {
  const float x = q[0], y = q[1], z = q[2], w = q[3];
  m3 r;
  r.c[0] = V(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + w * z), 2.0f * (x * z - w * y));
  r.c[1] = V(2.0f * (x * y - w * z), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + w * x));
  r.c[2] = V(2.0f * (x * z + w * y), 2.0f * (y * z - w * x), 1.0f - 2.0f * (x * x + y * y));
  return r;
}
static inline float wsign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
/* i32(e) of WGSL: truncation, saturating at the range ends, NaN -> 0 */
static inline int32_t wgsl_i32(float x) {
  if (x != x) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
  return (int32_t)x;
}

/* bodySDF, coupling.js:31-58: signed distance from p to body b centred at c and the outward normal */
static void body_sdf(const float* b, v3 c, v3 p, float* dist, v3* nrm) {
  const uint32_t s = (uint32_t)(b[35] + 0.5f);            /* shapeOf, rigid-wgsl.js:75 */
  const m3 R = qmat(b + 4);
  const v3 lp = mv(mT(R), vsub(p, c));
  if (s == 0u) {
    const float d = vlen(lp);
    const float m = fmaxf(d, 1e-6f);
    *dist = d - b[32];
    *nrm = mv(R, V(lp.x / m, lp.y / m, lp.z / m));
    return;
  }
  if (s == 2u) {
    const float h = b[33];
    const v3 q = V(lp.x, lp.y - clampf(lp.y, -h, h), lp.z);
    const float d = vlen(q);
    const float m = fmaxf(d, 1e-6f);
    const v3 t = V(q.x / m, q.y / m, q.z / m);
    *dist = d - b[32];
    *nrm = mv(R, d > 1e-6f ? t : V(0.0f, wsign(lp.y), 0.0f));
    return;
  }
  const v3 h = V(b[32], b[33], b[34]);
  const v3 q = V(fabsf(lp.x) - h.x, fabsf(lp.y) - h.y, fabsf(lp.z) - h.z);
  if (q.x > 0.0f || q.y > 0.0f || q.z > 0.0f) {
    const v3 dv = V(lp.x - clampf(lp.x, -h.x, h.x), lp.y - clampf(lp.y, -h.y, h.y), lp.z - clampf(lp.z, -h.z, h.z));
    const float d = vlen(dv);
    const float m = fmaxf(d, 1e-9f);
    *dist = d;
    *nrm = mv(R, V(dv.x / m, dv.y / m, dv.z / m));
    return;
  }
  int ax = 0;
  if (q.y > vget(q, ax)) ax = 1;
  if (q.z > vget(q, ax)) ax = 2;
  const float sg = vget(lp, ax) >= 0.0f ? 1.0f : -1.0f;
  *dist = vget(q, ax);
  *nrm = mv(R, V(ax == 0 ? sg : 0.0f, ax == 1 ? sg : 0.0f, ax == 2 ? sg : 0.0f));
}

void sio_couple(int32_t* grid, const int32_t dims[3], const float* bodies, int32_t n,
                const sio_couple_params* p, int32_t* acc) {
  const int32_t tiles[3] = {(dims[0] + 3) / 4, (dims[1] + 3) / 4, (dims[2] + 3) / 4};
  const v3 origin = V(p->origin[0], p->origin[1], p->origin[2]);
  int32_t cand[SIO_MAXC];
  int32_t accj[SIO_MAXC * 3], accl[SIO_MAXC * 3];
  for (int32_t tz = 0; tz < tiles[2]; tz++)
    for (int32_t ty = 0; ty < tiles[1]; ty++)
      for (int32_t tx = 0; tx < tiles[0]; tx++) {
        const float lo_off = p->band + 1.0f, hi_off = (3.0f + p->band) + 1.0f;
        const v3 tl = V((float)(tx * 4) - lo_off, (float)(ty * 4) - lo_off, (float)(tz * 4) - lo_off);
        const v3 th = V((float)(tx * 4) + hi_off, (float)(ty * 4) + hi_off, (float)(tz * 4) + hi_off);
        int nc = 0;   /* candidates in index order, at most MAXC (coupling.js:100-124) */
        for (int32_t bi = 0; bi < n && nc < SIO_MAXC; bi++) {
          const float* b = bodies + 48 * (size_t)bi;
          if ((f2u(b[46]) & (SIO_F_DISABLED | SIO_F_SENSOR)) != 0u || (f2u(b[44]) & p->mask) == 0u) continue;
          const v3 c = vscale(p->inv_dx, vsub(vadd(V(b[0], b[1], b[2]), vscale(p->lead, V(b[8], b[9], b[10]))), origin));
          const v3 q = V(clampf(c.x, tl.x, th.x), clampf(c.y, tl.y, th.y), clampf(c.z, tl.z, th.z));
          if (vlen(vsub(c, q)) <= b[3] * p->inv_dx) cand[nc++] = bi;
        }
        if (nc == 0) continue;
        memset(accj, 0, sizeof(int32_t) * 3 * (size_t)nc);
        memset(accl, 0, sizeof(int32_t) * 3 * (size_t)nc);
        for (int lz = 0; lz < 4; lz++)
          for (int ly = 0; ly < 4; ly++)
            for (int lx = 0; lx < 4; lx++) {
              const int32_t gx = tx * 4 + lx, gy = ty * 4 + ly, gz = tz * 4 + lz;
              if (gx >= dims[0] || gy >= dims[1] || gz >= dims[2]) continue;
              int32_t* node = grid + 4 * ((size_t)gx + (size_t)dims[0] * ((size_t)gy + (size_t)dims[1] * (size_t)gz));
              const float m = i2f_bits(node[3]);
              if (!(m > 0.0f)) continue;
              v3 v = V(i2f_bits(node[0]), i2f_bits(node[1]), i2f_bits(node[2]));
              const v3 pw = vadd(origin, vscale(p->dx, V((float)gx, (float)gy, (float)gz)));
              for (int c = 0; c < nc; c++) {
                const float* b = bodies + 48 * (size_t)cand[c];
                const v3 bc = vadd(V(b[0], b[1], b[2]), vscale(p->lead, V(b[8], b[9], b[10])));
                float dist;
                v3 nr;
                body_sdf(b, bc, pw, &dist, &nr);
                if (!(dist * p->inv_dx < p->band)) continue;
                const v3 r = vsub(pw, bc);
                const v3 vb = vscale(p->vel_to_lattice, vadd(V(b[8], b[9], b[10]), vcross(V(b[12], b[13], b[14]), r)));
                v3 vr = vsub(v, vb);
                const float vn = vdot(vr, nr);
                if (vn < 0.0f) {
                  vr = vsub(vr, vscale(vn, nr));
                  const float vt = vlen(vr);
                  if (vt > 1e-9f) vr = vscale(fmaxf(0.0f, 1.0f - (p->friction * -vn) / vt), vr);
                  const v3 vnew = vadd(vr, vb);
                  if (b[36] > 0.0f) {
                    const v3 J = vscale(-m, vsub(vnew, v));
                    const v3 L = vcross(vscale(p->inv_dx, r), J);
                    accj[c * 3] += wgsl_i32(rintf(J.x * SIO_FPJ));
                    accj[c * 3 + 1] += wgsl_i32(rintf(J.y * SIO_FPJ));
                    accj[c * 3 + 2] += wgsl_i32(rintf(J.z * SIO_FPJ));
                    accl[c * 3] += wgsl_i32(rintf(L.x * SIO_FPL));
                    accl[c * 3 + 1] += wgsl_i32(rintf(L.y * SIO_FPL));
                    accl[c * 3 + 2] += wgsl_i32(rintf(L.z * SIO_FPL));
                  }
                  v = vnew;
                }
              }
              node[0] = f2i_bits(v.x); node[1] = f2i_bits(v.y); node[2] = f2i_bits(v.z); node[3] = f2i_bits(m);
            }
        for (int k = 0; k < nc * 3; k++) {
          const int32_t bi = cand[k / 3], a = k % 3;
          acc[bi * 8 + a] = (int32_t)((uint32_t)acc[bi * 8 + a] + (uint32_t)accj[k]);
          acc[bi * 8 + 4 + a] = (int32_t)((uint32_t)acc[bi * 8 + 4 + a] + (uint32_t)accl[k]);
        }
      }
}

void sio_couple_apply(int32_t* acc, float* ext, int32_t n, float mom_to_world, float dx) {
  for (int32_t i = 0; i < n; i++) {
    int32_t* a = acc + 8 * (size_t)i;
    if (a[0] == 0 && a[1] == 0 && a[2] == 0 && a[4] == 0 && a[5] == 0 && a[6] == 0) continue;
    for (int k = 0; k < 3; k++) {
      ext[8 * i + k] = ext[8 * i + k] + ((float)a[k] / SIO_FPJ) * mom_to_world;
      ext[8 * i + 4 + k] = ext[8 * i + 4 + k] + (((float)a[4 + k] / SIO_FPL) * mom_to_world) * dx;
    }
    memset(a, 0, 8 * sizeof(int32_t));
  }
}

/* ------------------------------------------------------------------ emission, mpm.js:683-714 + 213-227 */
static inline double js_maxd(double a, double b) { return (a != a || b != b) ? (double)NAN : (a > b ? a : b); }
static inline double js_mind(double a, double b) { return (a != a || b != b) ? (double)NAN : (a < b ? a : b); }

int64_t sio_emit_box(const double lo[3], const double hi[3], double spacing, double jitter, uint32_t seed,
                     uint32_t material, const double vel[3], const int32_t dims[3], double dx,
                     const double origin[3], double substep_dt, float* out, int64_t cap) {
  uint32_t rnd = seed ? seed : 1u;
  int64_t n[3];
  for (int a = 0; a < 3; a++) {
    double q = floor((hi[a] - lo[a]) / spacing);
    n[a] = (int64_t)js_maxd(1.0, q);
  }
  const double s = substep_dt / dx;
  int64_t k = 0;
  for (int64_t z = 0; z < n[2]; z++)
    for (int64_t y = 0; y < n[1]; y++)
      for (int64_t x = 0; x < n[0]; x++) {
        double p[3];
        int64_t idx[3] = {x, y, z};
        for (int a = 0; a < 3; a++) {
          rnd ^= rnd << 13; rnd ^= rnd >> 17; rnd ^= rnd << 5;
          double r = (double)rnd / 4294967296.0;
          p[a] = lo[a] + ((double)idx[a] + 0.5 + (r - 0.5) * jitter) * spacing;
        }
        if (out && k < cap) {
          float* o = out + (size_t)SIO_PF * (size_t)k;
          memset(o, 0, sizeof(float) * SIO_PF);
          for (int a = 0; a < 3; a++) {
            double xw = (double)(float)p[a];      /* Float32Array of sampleShape */
            double xl = (xw - origin[a]) / dx;
            o[a] = (float)js_mind((double)(dims[a] - 3) - 1e-3, js_maxd(3.0 + 1e-3, xl));
          }
          memcpy(&o[3], &material, 4);
          for (int a = 0; a < 3; a++) o[4 + a] = (float)(vel[a] * s);
          o[7] = 1.0f; o[20] = 1.0f; o[25] = 1.0f; o[30] = 1.0f;
        }
        k++;
      }
  return k;
}

/* ------------------------------------------------------------------ step(), mpm.js:590-602 */
void sio_substeps(float* P, float* scratch, int64_t n, int32_t* grid, const sio_params* prm,
                  int64_t* step_count, int K, int threads) {
  float* cur = P;
  float* alt = scratch;
  for (int s = 0; s < K; s++) {
    if (prm->sort_every > 0 && (*step_count % prm->sort_every) == 0) {
      sio_sort(cur, alt, n, prm->num_blocks, NULL, NULL, NULL);
      float* t = cur; cur = alt; alt = t;
    }
    sio_p2g(cur, n, prm->dims, prm->mats, prm->vol4, grid, threads);
    sio_grid_update(grid, prm->dims, prm->gravity, prm->bound, prm->cols, prm->ncol, prm->floor_friction, threads);
    if (prm->nbodies > 0) {   /* coupling.substep(s), mpm.js:596 */
      sio_couple_params cp = prm->couple;
      cp.lead = (float)(((double)s + 0.5) * prm->substep_dt);
      sio_couple(grid, prm->dims, prm->bodies, prm->nbodies, &cp, prm->body_acc);
    }
    sio_g2p(cur, n, prm->dims, grid, prm->mats, prm->bound, prm->vmax, threads);
    (*step_count)++;
  }
  if (cur != P) memcpy(P, cur, sizeof(float) * SIO_PF * (size_t)n);
}
