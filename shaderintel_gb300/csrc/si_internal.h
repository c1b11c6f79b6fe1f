// si_internal.h — helpers shared by the host-side translation units of libsi_cuda.
#pragma once
#include <stdint.h>

#include <string>

#include "si_cuda.h"

// Records the message for si_last_error() (thread-local) and returns the code.
int si_fail(int code, const std::string& msg);

struct si_scene_geom {
  int32_t dims[3];
  double dx, origin[3], substep_dt;
  int32_t bound;
};
void si_scene_geometry(const si_mpm* h, si_scene_geom* g);
