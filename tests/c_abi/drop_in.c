/* A C host of libsi_cuda (what an N-API or JNI shim does): the MPM object's life cycle through the
 * C ABI only — create, materials, add, colliders, step(dt, K), read positions, destroy. Exit 0 when
 * every call succeeds and the particles moved and stayed finite. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "si_cuda.h"

#define CHECK(x)                                                                  \
  do {                                                                            \
    int rc_ = (x);                                                                \
    if (rc_ != SI_OK) {                                                           \
      fprintf(stderr, "%s failed (%d): %s\n", #x, rc_, si_last_error());          \
      return 1;                                                                   \
    }                                                                             \
  } while (0)

int main(void) {
  si_mpm_desc d;
  si_mpm_desc_default(&d);
  d.grid = 32;
  d.max_particles = 50000;
  si_mpm* h = NULL;
  CHECK(si_mpm_create(NULL, &d, &h));
  si_material_def water, jelly;
  CHECK(si_material_preset("water", &water));
  CHECK(si_material_preset("jelly", &jelly));
  float table[2 * SI_MATERIAL_FLOATS];
  CHECK(si_material_row(&water, d.ppc_axis, table));
  CHECK(si_material_row(&jelly, d.ppc_axis, table + SI_MATERIAL_FLOATS));
  CHECK(si_mpm_set_materials(h, table, 2));
  const double lo[3] = {0.1, 0.1, 0.1}, hi[3] = {0.5, 0.4, 0.6}, c[3] = {0.7, 0.6, 0.5}, v[3] = {0, -1, 0};
  int64_t a = 0, b = 0;
  CHECK(si_mpm_emit(h, 0, lo, hi, 0, 0, 0.6, 1, 0, NULL, &a));
  CHECK(si_mpm_emit(h, 1, c, NULL, 0.1, 0, 0.6, (uint32_t)(a + 1), 1, v, &b));
  float col[SI_COLLIDER_FLOATS];
  const double center[3] = {0.5, 0.2, 0.5};
  CHECK(si_collider_row(h, 0, center, NULL, 0.08, 0.3, NULL, 0, col));
  CHECK(si_mpm_set_colliders(h, col, 1));
  si_mpm_info info;
  CHECK(si_mpm_get_info(h, &info));
  const int64_t n = info.count;
  float* before = (float*)malloc(sizeof(float) * 3 * (size_t)n);
  float* after = (float*)malloc(sizeof(float) * 3 * (size_t)n);
  CHECK(si_mpm_read_positions(h, before, 0, n));
  CHECK(si_mpm_step(h, 0.0, 0));                  /* one frame */
  CHECK(si_mpm_step(h, info.substep_dt, 5));      /* step(dt, K) */
  uint64_t ticket = 0;
  CHECK(si_mpm_read_positions_async(h, after, 0, n, &ticket));
  CHECK(si_mpm_read_wait(h, ticket));
  double moved = 0;
  for (int64_t i = 0; i < 3 * n; i++) {
    if (!isfinite(after[i])) return 2;
    moved += fabs((double)after[i] - (double)before[i]);
  }
  CHECK(si_mpm_get_info(h, &info));
  printf("particles %lld (%lld + %lld) stepCount %lld mean displacement %.3e\n", (long long)n, (long long)a,
         (long long)b, (long long)info.step_count, moved / (double)n);
  if (info.step_count != 13 || !(moved > 0)) return 3;
  CHECK(si_mpm_destroy(h));
  if (si_mpm_step(h, 0.0, 0) != SI_EDESTROYED) return 4;   /* step after destroy (mpm.js:583) */
  si_mpm_free(h);
  free(before);
  free(after);
  return 0;
}
