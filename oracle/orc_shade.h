// Oracle — TEST INFRASTRUCTURE ONLY (see orc_math.h).
//
// Restatement of the shading steps of the reference's path tracer that produce
// the secondary rays of the wavefront workloads:
//   pcg / xxhash32 / PCGRandomSampler    scene/rendering/gpu-ray-tracing/src/sampler.rs:11-72
//   next_2d = (next(), next())           math/statistics/src/sampling/mod.rs:25-27
//   concentric_sample_disk              math/statistics/src/distribution_map.rs:10-27
//   cosine_sample_hemisphere(_in_dir)   math/statistics/src/distribution_map.rs:29-58
//   offset_ray_hit                      scene/rendering/gpu-ray-tracing/src/ray_util.rs:5-40
//   hit_world_position = o + d * t      shader/ray-tracing/src/api/ctx.rs:209-211
//   shadow ray [EPSILON, light dist] with ACCEPT_FIRST_HIT_AND_END_SEARCH
//                                        scene/rendering/gpu-ray-tracing/src/feature/path_tracing/ray_hit.rs:21-44
//
// One deliberate difference: the reference evaluates cos/sin with the
// platform's f32 libm (which differs between platforms in the last bit); here
// both this oracle and the CUDA kernels use the same fixed Taylor polynomials on
// [-pi/4, pi/4] (sin to x^9, cos to x^10, truncation error < 3e-9) and use
// cos(pi/2 - phi) = sin(phi) for the second branch of the concentric mapping, so
// host and device produce identical secondary rays.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "orc_math.h"

namespace orc {

static inline uint32_t pcg_next(uint32_t& state) {
  uint32_t prev = state * 747796405u + 2891336453u;
  uint32_t word = ((prev >> ((prev >> 28u) + 4u)) ^ prev) * 277803737u;
  state = prev;
  return (word >> 22u) ^ word;
}
static inline float bits_f(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static inline uint32_t f_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}
static inline float sample_next(uint32_t& state) {
  uint32_t r = pcg_next(state);
  return bits_f(0x3f800000u | (r >> 9u)) - 1.0f;
}
static inline uint32_t xxhash32(uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t p0 = 2246822519u, p1 = 3266489917u, p2 = 668265263u, p3 = 374761393u;
  uint32_t h = z + p3 + x * p1;
  h = p2 * ((h << 17) | (h >> (32 - 17)));
  h = h + y * p1;
  h = p2 * ((h << 17) | (h >> (32 - 17)));
  h = p0 * (h ^ (h >> 15));
  h = p1 * (h ^ (h >> 13));
  return h ^ (h >> 16);
}

static inline float poly_sin(float x) {
  float x2 = x * x;
  float p = 2.7557319e-6f;            // 1/9!
  p = -1.9841270e-4f + x2 * p;        // -1/7!
  p = 8.3333333e-3f + x2 * p;         // 1/5!
  p = -1.6666667e-1f + x2 * p;        // -1/3!
  return x + x * (x2 * p);
}
static inline float poly_cos(float x) {
  float x2 = x * x;
  float p = -2.7557319e-7f;           // -1/10!
  p = 2.4801587e-5f + x2 * p;         // 1/8!
  p = -1.3888889e-3f + x2 * p;        // -1/6!
  p = 4.1666667e-2f + x2 * p;         // 1/4!
  p = -0.5f + x2 * p;                 // -1/2!
  return 1.0f + x2 * p;
}

static const float PI_OVER_4 = 0.78539819f;  // std::f32::consts::PI / 4.0

static inline void concentric_sample_disk(float sx, float sy, float* dx, float* dy) {
  float ux = sx * 2.0f - 1.0f;
  float uy = sy * 2.0f - 1.0f;
  if (ux == 0.0f && uy == 0.0f) {
    *dx = 0.0f;
    *dy = 0.0f;
    return;
  }
  float r, c, s;
  if (std::fabs(ux) > std::fabs(uy)) {
    r = ux;
    float phi = PI_OVER_4 * (uy / ux);
    c = poly_cos(phi);
    s = poly_sin(phi);
  } else {
    r = uy;
    float phi = PI_OVER_4 * (ux / uy);  // theta = pi/2 - phi
    c = poly_sin(phi);
    s = poly_cos(phi);
  }
  *dx = c * r;
  *dy = s * r;
}

// cosine_sample_hemisphere_in_dir: direction around `dir` (normalized).
static inline V3 cosine_sample_in_dir(V3 dir, float sx, float sy) {
  float dx, dy;
  concentric_sample_disk(sx, sy, &dx, &dy);
  float oz = std::sqrt(rmax(0.0f, 1.0f - dx * dx - dy * dy));
  V3 left = normalize(cross(v3(0.0f, 1.0f, 0.0f), dir));
  V3 up = cross(left, dir);
  float xy_r = std::sqrt(dx * dx + dy * dy);
  if (xy_r == 0.0f) return dir;
  float cos_phi = dx / xy_r;
  float sin_phi = dy / xy_r;
  float cos_theta = oz;
  float sin_theta = xy_r;
  V3 v = left * sin_theta * cos_phi + up * sin_theta * sin_phi + dir * cos_theta;
  return normalize(v);
}

// offset_ray_hit (Ray Tracing Gems ch. 6): integer ULP offset away from the surface.
static inline float offset_axis(float p, float n) {
  const float int_scale = 256.0f, float_scale = 1.0f / 65536.0f, origin = 1.0f / 32.0f;
  int32_t of_i = (int32_t)(n * int_scale);  // truncation toward zero
  uint32_t pi = f_bits(p) + (uint32_t)((p < 0.0f) ? -of_i : of_i);  // wrapping i32 add
  float p_i = bits_f(pi);
  return (std::fabs(p) < origin) ? (p + float_scale * n) : p_i;
}
static inline V3 offset_ray_hit(V3 p, V3 n) { return v3(offset_axis(p.x, n.x), offset_axis(p.y, n.y), offset_axis(p.z, n.z)); }

}  // namespace orc
