/*
 * si_oracle — CPU restatement of the ShaderIntel MLS-MPM substep (TEST INFRASTRUCTURE).
 *
 * This library is the checker for the CUDA substep in shaderintel_gb300/csrc. Only the tests,
 * the smoke check and the timed CPU baseline of bench.py load it; no product code path calls it.
 *
 * It restates, in plain C11 on the reference's 128-byte AoS particle record, the WGSL kernels of
 * src/physics/mpm.js (ShaderIntel v0.3.0):
 *   record / fixed point / B-spline / Morton ........ mpm.js:54-78
 *   block sort (key, count, scan, reorder) .......... mpm.js:563-577, 614-621; src/prims/scan.js:288-306
 *   P2G scatter (tile and global paths sum alike) ... mpm.js:306-401
 *   retime ......................................... mpm.js:405-413
 *   grid update + collider SDFs ..................... mpm.js:414-471
 *   G2P + fluid / Neo-Hookean / snow / sand ......... mpm.js:474-560
 *   eigSym3 / svd3 (4 cyclic Jacobi sweeps) .......... src/shaders/linalg.js:14-69
 *   step() schedule ................................. mpm.js:582-604
 *   fluid <-> rigid coupling pass and apply ......... src/physics/coupling.js:31-60, 83-196
 *
 * Canonical f32 evaluation order. WGSL pins neither FMA contraction nor the reduction order of
 * matrix products, so this file fixes one order and the CUDA kernels follow it exactly:
 *   - every f32 operation is rounded on its own (built with -ffp-contract=off; no fused operation);
 *   - binary expressions evaluate left to right as written in the WGSL;
 *   - mat*vec: r_i = (M0_i*v0 + M1_i*v1) + M2_i*v2 (columns Mk); mat*mat likewise per column;
 *   - dot(a,b) = (a0*b0 + a1*b1) + a2*b2; length = sqrt(dot); normalize(v) = v_i / length(v);
 *   - determinant: first-column cofactor expansion (sio_det3);
 *   - products with diag3(s) and with a Jacobi rotation drop the exact zero and one terms;
 *   - inverseSqrt(x) = 1/sqrt(x); division and sqrt are IEEE correctly rounded;
 *   - log and exp are sio_logf / sio_expf (Cody & Waite argument reduction with the Taylor
 *     series of atanh and exp), within 2 ulp of the true value.
 * With this order the integer work (keys, counts, starts, grid i32 sums) and, because the same
 * f32 sequence runs on both sides, the whole particle state agree with the CUDA path bit for bit.
 *
 * Parity pin: the reference holds no golden vectors and runs only as WGSL in a browser. Its own
 * WGSL source is executed by tests/golden/wgsl_exec.py (IEEE f32, the same order as above) to make
 * the fixtures under tests/golden/, and this oracle is checked against them: keys, starts, sorted
 * records, P2G grid sums and the grid update bit for bit; G2P bit for bit in every field that does
 * not pass through log/exp, and within WGSL's accuracy bound of log/exp in the others.
 */
#ifndef SI_ORACLE_H
#define SI_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SIO_PF 32 /* floats per particle record (8 x vec4f, mpm.js:54-63) */

uint32_t sio_morton3(uint32_t x, uint32_t y, uint32_t z);
/* numBlocks of mpm.js:119-121 for grid dims. */
uint32_t sio_num_blocks(const int32_t dims[3]);

/* Keys of mpm.js:567-569 (morton3(u32(max(x,0))/4)), clamped to num_blocks-1 for particles
 * outside the grid (the reference would index out of bounds there). */
void sio_keys(const float* P, int64_t n, uint32_t num_blocks, uint32_t* keys);
/* Exclusive scan of the per-block counts, num_blocks+1 entries; starts[num_blocks] = n. */
void sio_bins(const uint32_t* keys, int64_t n, uint32_t num_blocks, uint32_t* starts);
/* Stable counting sort of src into dst by block key; keys/starts/perm outputs may be NULL.
 * perm[d] = source index of dst record d. */
void sio_sort(const float* src, float* dst, int64_t n, uint32_t num_blocks,
              uint32_t* keys, uint32_t* starts, uint32_t* perm);

/* Clear grid (4 x i32 per node) and scatter n particles into it. */
void sio_p2g(const float* P, int64_t n, const int32_t dims[3], const float* mats, float vol4,
             int32_t* grid, int threads);
/* In place: i32 sums -> bit pattern of vec4f(v, m). cols: ncol x 12 floats. */
void sio_grid_update(int32_t* grid, const int32_t dims[3], const float gravity[3], float bound,
                     const float* cols, int ncol, float floor_friction, int threads);
/* In place G2P on the particle records; grid holds vec4f(v, m) bit patterns. */
void sio_g2p(float* P, int64_t n, const int32_t dims[3], const int32_t* grid, const float* mats,
             float bound, float vmax, int threads);
void sio_retime(float* P, int64_t n, float k);

typedef struct {
  float origin[3];        /* world origin of node 0 */
  float dx, inv_dx;
  float lead;             /* body positions extrapolated by v * lead: (s + 0.5) * substep dt */
  float vel_to_lattice;   /* substep dt / dx */
  float friction, band;   /* fluid-body friction (0.2), band in cells (0.5) */
  uint32_t mask;          /* group bits of the bodies that interact */
} sio_couple_params;

typedef struct sio_params {
  int32_t dims[3];
  uint32_t num_blocks;
  float gravity[3];     /* lattice units per substep^2 (mpm.js:588) */
  float bound;          /* 3 */
  float floor_friction; /* 0.4 */
  float vmax;           /* 0.9 */
  float vol4;           /* 4 / ppcAxis^3 */
  int32_t sort_every;   /* 4 */
  int32_t ncol;
  const float* mats;    /* 8 x 12 */
  const float* cols;    /* 16 x 12 */
  /* rigid coupling (nbodies = 0: none): body records, pass parameters (lead is set per substep
   * as (s + 0.5) * substep_dt, s counted from the call's first substep), impulse sums */
  const float* bodies;
  int32_t nbodies;
  sio_couple_params couple;
  double substep_dt;
  int32_t* body_acc;
} sio_params;

/* K substeps of mpm.js:590-602 starting at *step_count. P holds the n records on entry and on
 * return; scratch (n records) and grid (nodes x 4 i32) are work space. */
void sio_substeps(float* P, float* scratch, int64_t n, int32_t* grid, const sio_params* prm,
                  int64_t* step_count, int K, int threads);

/* sampleShape({box}) + the record conversion of add() (mpm.js:683-714, 213-227) with bound 3:
 * writes up to cap records and returns the number of lattice points. */
int64_t sio_emit_box(const double lo[3], const double hi[3], double spacing, double jitter, uint32_t seed,
                     uint32_t material, const double vel[3], const int32_t dims[3], double dx,
                     const double origin[3], double substep_dt, float* out, int64_t cap);

float sio_logf(float x);
float sio_expf(float x);
/* svd3 of linalg.js:46-69 on a column-major 3x3 (m[col*3+row]); outputs U, s, V likewise. */
void sio_svd3(const float* F, float* U, float* s, float* V);

/* ---- fluid <-> rigid coupling, src/physics/coupling.js:83-196 (moving rigid boundaries of the grid)
 * bodies: n records of 48 floats, the reference's Body (src/physics/rigid-wgsl.js:20-33): x (w =
 * bounding radius), q (x y z w), v (w = friction), w (angular velocity), x0, q0, y, qy, size (w =
 * shape: 0 sphere, 1 box, 2 capsule), mass (x = m, 0 = static / kinematic), props, info (4 u32:
 * group bits, mask bits, flags, user). sio_couple runs the pass of one substep over a grid that
 * holds vec4f(v, m) bits (after the grid update): nodes with m > 0 within `band` cells of a body
 * lose their inward relative velocity (Coulomb friction on the tangent), and the reaction impulses
 * are added in fixed point to acc (n x 8 i32: J x 16384 in [0..2], L x 1024 in [4..6]). */

void sio_couple(int32_t* grid, const int32_t dims[3], const float* bodies, int32_t n,
                const sio_couple_params* p, int32_t* acc);
/* mpm-rigid-apply: ext (n x 8 f32: J xyz 0, L xyz 0) += acc in world units, acc zeroed. */
void sio_couple_apply(int32_t* acc, float* ext, int32_t n, float mom_to_world, float dx);

#ifdef __cplusplus
}
#endif
#endif
