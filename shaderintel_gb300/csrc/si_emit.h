// si_emit.h — parameters of the device emission (si_emit.cu), built by si_runtime.cpp.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace si {

struct EmitInfo {
  uint32_t jump[32][32];   // jump[i][j]: column j of M^(3 * 2^i), M one xorshift32 step over GF(2)
  uint32_t seed;           // `seed >>> 0 || 1`
  int32_t shape;           // 0 box, 1 sphere, 2 cylinder
  double a[3];             // sphere / cylinder centre
  double r;                // radius
  double lo[3];            // lattice origin (world)
  double spacing, jitter;
  int64_t n[3], total;     // lattice points per axis, their product
  // record conversion (add(), mpm.js:213-227)
  double origin[3], dx, bound, hi[3];   // hi = dims - bound
  float vel[3];            // velocity * substep dt / dx, as f32
  uint32_t material;
  float4* P;               // the scene's particle streams
  int64_t cap, offset;     // stream stride; first slot written (the current count)
  int64_t room;            // maxParticles - count
};

// Enqueues the three emission kernels; scratch holds ceil(total / 256) + 1 u32, and its last
// entry receives the number of points inside the shape.
int launch_emit(const EmitInfo& e, uint32_t* scratch, cudaStream_t st);

}  // namespace si
