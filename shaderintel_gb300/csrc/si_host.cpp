// si_host.cpp — the reference's host-side arithmetic for building scenes, in f64 with JavaScript
// semantics (Number = IEEE double; Float32Array stores round to nearest even), so every host
// that drives libsi_cuda builds bit-identical particle records and tables.
//   MATERIALS presets ............ src/physics/mpm.js:38-46
//   _material validation ......... mpm.js:148-168
//   _uploadMaterials row ......... mpm.js:170-199
//   sampleShape (xorshift32) ..... mpm.js:683-714
//   add() record conversion ...... mpm.js:207-232
//   _uploadColliders row ......... mpm.js:276-293
#include <cmath>
#include <cstring>
#include <string>

#include "si_cuda.h"
#include "si_internal.h"

namespace {

// Math.max / Math.min: NaN if either argument is NaN
double js_max(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : b); }
double js_min(double a, double b) { return (a != a || b != b) ? NAN : (a < b ? a : b); }
double or_default(double v, double d) { return std::isnan(v) ? d : v; }   // `v ?? d` with NaN for undefined

struct Preset { const char* name; si_material_def d; };
const Preset kPresets[] = {
    {"water", {0, 1.0, 1.0, NAN, 0.0, NAN, NAN, NAN, NAN}},
    {"oil", {0, 0.9, 0.9, NAN, 0.3, NAN, NAN, NAN, NAN}},
    {"honey", {0, 1.4, 0.9, NAN, 1.0, NAN, NAN, NAN, NAN}},
    {"jelly", {1, 1.0, 0.35, 0.3, NAN, NAN, NAN, NAN, NAN}},
    {"rubber", {1, 1.2, 0.7, 0.45, NAN, NAN, NAN, NAN, NAN}},
    {"snow", {2, 0.4, 0.6, 0.2, NAN, 10.0, 0.025, 0.0075, NAN}},
    {"sand", {3, 1.6, 0.6, 0.3, NAN, NAN, NAN, NAN, 33.0}},
};

}  // namespace

extern "C" {

int si_material_preset(const char* name, si_material_def* out) {
  if (!name || !out) return si_fail(SI_EINVAL, "si_material_preset: null argument");
  for (const Preset& p : kPresets)
    if (std::strcmp(p.name, name) == 0) { *out = p.d; return SI_OK; }
  return si_fail(SI_EINVAL, std::string("MPM: unknown material \"") + name +
                                "\" (use water, oil, honey, jelly, rubber, snow, sand or a definition with a kind)");
}

int si_material_row(const si_material_def* m, int32_t ppc_axis, float row[12]) {
  if (!m || !row) return si_fail(SI_EINVAL, "si_material_row: null argument");
  if (m->kind < 0 || m->kind > 3)
    return si_fail(SI_EINVAL, "MPM: material kind must be 0-3 (got " + std::to_string(m->kind) + ")");
  const double density = or_default(m->density, 1.0);
  if (!(density > 0 && density <= 50))
    return si_fail(SI_EINVAL, "MPM: density " + std::to_string(density) +
                                  " is outside (0, 50] - densities are relative to water (1), not kg/m3");
  if (ppc_axis <= 0) ppc_axis = 2;
  const double vol = 1.0 / std::pow((double)ppc_axis, 3.0);
  const double mass = density * vol;
  const double rho = mass / vol;
  const double c = 0.4 * js_min(1.0, js_max(0.01, or_default(m->stiffness, 1.0)));
  const double nu = js_min(0.49, js_max(0.0, or_default(m->poisson, 0.3)));
  const double Mmod = rho * c * c;
  const double mu = Mmod * (1 - 2 * nu) / (2 * (1 - nu));
  const double la = Mmod * nu / (1 - nu);
  std::memset(row, 0, 12 * sizeof(float));
  const uint32_t kind = (uint32_t)m->kind;
  std::memcpy(&row[0], &kind, 4);
  row[1] = (float)mass;
  row[2] = (float)(m->kind == 0 ? rho * c * c : mu);
  row[3] = (float)la;
  row[4] = (float)(js_min(4.0, js_max(0.0, or_default(m->viscosity, 0.0))) * 0.05 * rho);
  row[5] = (float)or_default(m->hardening, 10.0);
  row[6] = (float)or_default(m->compression, 0.025);
  row[7] = (float)or_default(m->stretch, 0.0075);
  const double phi = (or_default(m->friction_deg, 33.0) * M_PI) / 180;
  const double sinp = std::sin(phi);
  row[8] = (float)(std::sqrt(2.0 / 3.0) * (2 * sinp) / (3 - sinp));
  return SI_OK;
}

int si_sample_shape(int32_t shape, const double a[3], const double b[3], double r, double h, double spacing,
                    double jitter, uint32_t seed, float* out, int64_t cap, int64_t* n_out) {
  if (!a || !n_out) return si_fail(SI_EINVAL, "si_sample_shape: null argument");
  if (!(spacing > 0)) return si_fail(SI_EINVAL, "si_sample_shape: spacing must be > 0");
  uint32_t rnd = seed ? seed : 1u;   // `seed >>> 0 || 1`
  auto rand = [&rnd]() {
    rnd ^= rnd << 13; rnd ^= rnd >> 17; rnd ^= rnd << 5;
    return (double)rnd / 4294967296.0;
  };
  double lo[3], hi[3];
  if (shape == 0) {
    if (!b) return si_fail(SI_EINVAL, "si_sample_shape: box needs hi");
    for (int k = 0; k < 3; k++) { lo[k] = a[k]; hi[k] = b[k]; }
  } else if (shape == 1) {
    for (int k = 0; k < 3; k++) { lo[k] = a[k] - r; hi[k] = a[k] + r; }
  } else if (shape == 2) {
    lo[0] = a[0] - r; lo[1] = a[1] - h; lo[2] = a[2] - r;
    hi[0] = a[0] + r; hi[1] = a[1] + h; hi[2] = a[2] + r;
  } else {
    return si_fail(SI_EINVAL, "MPM.add: shape needs box | sphere | cylinder | sdf | points");
  }
  int64_t n[3];
  for (int k = 0; k < 3; k++) {
    double q = std::floor((hi[k] - lo[k]) / spacing);
    n[k] = (int64_t)js_max(1.0, q);
  }
  int64_t cnt = 0;
  double p[3];
  for (int64_t z = 0; z < n[2]; z++)
    for (int64_t y = 0; y < n[1]; y++)
      for (int64_t x = 0; x < n[0]; x++) {
        p[0] = lo[0] + ((double)x + 0.5 + (rand() - 0.5) * jitter) * spacing;
        p[1] = lo[1] + ((double)y + 0.5 + (rand() - 0.5) * jitter) * spacing;
        p[2] = lo[2] + ((double)z + 0.5 + (rand() - 0.5) * jitter) * spacing;
        bool inside = true;
        if (shape == 1) {
          double d0 = p[0] - a[0], d1 = p[1] - a[1], d2 = p[2] - a[2];
          inside = d0 * d0 + d1 * d1 + d2 * d2 <= r * r;
        } else if (shape == 2) {
          double d0 = p[0] - a[0], d2 = p[2] - a[2];
          inside = d0 * d0 + d2 * d2 <= r * r;
        }
        if (!inside) continue;
        if (out && cnt < cap) {
          out[3 * cnt] = (float)p[0]; out[3 * cnt + 1] = (float)p[1]; out[3 * cnt + 2] = (float)p[2];
        }
        cnt++;
      }
  *n_out = cnt;
  return SI_OK;
}

int si_make_records(const si_mpm* h, const float* xyz, int64_t n, int32_t material, const double velocity[3],
                    double substep_dt, float* records) {
  if (!h || (!xyz && n) || (!records && n)) return si_fail(SI_EINVAL, "si_make_records: null argument");
  si_scene_geom g;
  si_scene_geometry(h, &g);
  const double dt = substep_dt > 0 ? substep_dt : g.substep_dt;
  const double s = dt / g.dx;
  const double vel[3] = {velocity ? velocity[0] : 0.0, velocity ? velocity[1] : 0.0, velocity ? velocity[2] : 0.0};
  const uint32_t mat = (uint32_t)material;
  for (int64_t k = 0; k < n; k++) {
    float* o = records + 32 * k;
    std::memset(o, 0, 32 * sizeof(float));
    for (int a = 0; a < 3; a++) {
      const double x = ((double)xyz[3 * k + a] - g.origin[a]) / g.dx;
      const double lo = g.bound, hi = g.dims[a] - g.bound;
      o[a] = (float)js_min(hi - 1e-3, js_max(lo + 1e-3, x));
    }
    std::memcpy(&o[3], &mat, 4);
    o[4] = (float)(vel[0] * s); o[5] = (float)(vel[1] * s); o[6] = (float)(vel[2] * s);
    o[7] = 1.0f;
    o[20] = 1.0f; o[25] = 1.0f; o[30] = 1.0f;
  }
  return SI_OK;
}

int si_collider_row(const si_mpm* h, int32_t type, const double center[3], const double vec3[3], double radius,
                    double friction, const double velocity[3], double substep_dt, float row[12]) {
  if (!h || !row) return si_fail(SI_EINVAL, "si_collider_row: null argument");
  if (type < 0 || type > 2) return si_fail(SI_EINVAL, "MPM collider type must be sphere (0), box (1) or plane (2)");
  si_scene_geom g;
  si_scene_geometry(h, &g);
  const double dt = substep_dt > 0 ? substep_dt : g.substep_dt;
  const double s = dt / g.dx;
  std::memset(row, 0, 12 * sizeof(float));
  const uint32_t t = (uint32_t)type;
  std::memcpy(&row[0], &t, 4);
  const double ctr[3] = {center ? center[0] : 0.0, center ? center[1] : 0.0, center ? center[2] : 0.0};
  for (int a = 0; a < 3; a++) row[1 + a] = (float)((ctr[a] - g.origin[a]) / g.dx);
  if (type == 2) {
    const double nrm[3] = {vec3 ? vec3[0] : 0.0, vec3 ? vec3[1] : 1.0, vec3 ? vec3[2] : 0.0};
    row[4] = (float)nrm[0]; row[5] = (float)nrm[1]; row[6] = (float)nrm[2];
  } else if (type == 1) {
    const double hh[3] = {vec3 ? vec3[0] : 0.1, vec3 ? vec3[1] : 0.1, vec3 ? vec3[2] : 0.1};
    row[4] = (float)(hh[0] / g.dx); row[5] = (float)(hh[1] / g.dx); row[6] = (float)(hh[2] / g.dx);
  } else {
    row[4] = (float)(or_default(radius, 0.1) / g.dx);
  }
  row[7] = (float)or_default(friction, 0.3);
  const double v[3] = {velocity ? velocity[0] : 0.0, velocity ? velocity[1] : 0.0, velocity ? velocity[2] : 0.0};
  row[8] = (float)(v[0] * s); row[9] = (float)(v[1] * s); row[10] = (float)(v[2] * s);
  return SI_OK;
}

}  // extern "C"
