// Shading helpers shared by the wavefront and path kernels: the reference
// path tracer's sampler and sampling functions restated for the device.
//   pcg / xxhash32 / next()                scene/rendering/gpu-ray-tracing/src/sampler.rs:11-72
//   concentric disk + cosine hemisphere     math/statistics/src/distribution_map.rs:10-58
//   offset_ray_hit                          scene/rendering/gpu-ray-tracing/src/ray_util.rs:5-40
// cos/sin are fixed Taylor polynomials on [-pi/4, pi/4] evaluated identically
// on host (oracle) and device; every unit including this header is built with
// -fmad=false so that all of it is bit-reproducible.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "traverse.cuh"

namespace rdn {
namespace dev {

constexpr float F32_EPSILON = 1.1920929e-7f;
constexpr float F32_MAX = 3.40282347e+38f;

__device__ __forceinline__ uint32_t pcg_next(uint32_t& state) {
  const uint32_t prev = state * 747796405u + 2891336453u;
  const uint32_t word = ((prev >> ((prev >> 28u) + 4u)) ^ prev) * 277803737u;
  state = prev;
  return (word >> 22u) ^ word;
}
__device__ __forceinline__ float sample_next(uint32_t& state) {
  return __uint_as_float(0x3f800000u | (pcg_next(state) >> 9u)) - 1.0f;
}
__device__ __forceinline__ uint32_t rotl17(uint32_t h) { return (h << 17) | (h >> 15); }
__device__ __forceinline__ uint32_t xxhash32(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t h = z + 374761393u + x * 3266489917u;
  h = 668265263u * rotl17(h);
  h = h + y * 3266489917u;
  h = 668265263u * rotl17(h);
  h = 2246822519u * (h ^ (h >> 15));
  h = 3266489917u * (h ^ (h >> 13));
  return h ^ (h >> 16);
}
// Taylor polynomials on [-pi/4, pi/4], evaluated identically on host and device.
__device__ __forceinline__ float poly_sin(float x) {
  const float x2 = x * x;
  float p = 2.7557319e-6f;
  p = -1.9841270e-4f + x2 * p;
  p = 8.3333333e-3f + x2 * p;
  p = -1.6666667e-1f + x2 * p;
  return x + x * (x2 * p);
}
__device__ __forceinline__ float poly_cos(float x) {
  const float x2 = x * x;
  float p = -2.7557319e-7f;
  p = 2.4801587e-5f + x2 * p;
  p = -1.3888889e-3f + x2 * p;
  p = 4.1666667e-2f + x2 * p;
  p = -0.5f + x2 * p;
  return 1.0f + x2 * p;
}

__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize3(float3 v) {
  const float mag_sq = dot3(v, v);
  if (mag_sq > 0.0f) return v * (1.0f / sqrtf(mag_sq));
  return v;
}

// cosine_sample_hemisphere_in_dir (math/statistics/src/distribution_map.rs:29-58)
__device__ __forceinline__ float3 cosine_sample_in_dir(float3 dir, float sx, float sy) {
  const float ux = sx * 2.0f - 1.0f, uy = sy * 2.0f - 1.0f;
  float dx = 0.0f, dy = 0.0f;
  if (!(ux == 0.0f && uy == 0.0f)) {
    float r, c, s;
    if (fabsf(ux) > fabsf(uy)) {
      r = ux;
      const float phi = 0.78539819f * (uy / ux);
      c = poly_cos(phi);
      s = poly_sin(phi);
    } else {
      r = uy;
      const float phi = 0.78539819f * (ux / uy);
      c = poly_sin(phi);
      s = poly_cos(phi);
    }
    dx = c * r;
    dy = s * r;
  }
  const float oz = sqrtf(fmaxf(0.0f, 1.0f - dx * dx - dy * dy));
  const float3 left = normalize3(cross3(make_float3(0.0f, 1.0f, 0.0f), dir));
  const float3 up = cross3(left, dir);
  const float xy_r = sqrtf(dx * dx + dy * dy);
  if (xy_r == 0.0f) return dir;
  const float cos_phi = dx / xy_r, sin_phi = dy / xy_r;
  const float3 v = left * xy_r * cos_phi + up * xy_r * sin_phi + dir * oz;
  return normalize3(v);
}

// offset_ray_hit (scene/rendering/gpu-ray-tracing/src/ray_util.rs:5-40)
__device__ __forceinline__ float offset_axis(float p, float n) {
  const int32_t of_i = (int32_t)(n * 256.0f);
  const float p_i = __uint_as_float(__float_as_uint(p) + (uint32_t)((p < 0.0f) ? -of_i : of_i));
  return (fabsf(p) < 0.03125f) ? (p + 1.52587891e-5f * n) : p_i;
}
__device__ __forceinline__ float3 offset_ray_hit(float3 p, float3 n) {
  return make_float3(offset_axis(p.x, n.x), offset_axis(p.y, n.y), offset_axis(p.z, n.z));
}

// Warp-aggregated append: every lane with `want` gets a unique slot.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want) {
  const uint32_t active = __activemask();
  const uint32_t mask = __ballot_sync(active, want);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t leader = __ffs(active) - 1;
  uint32_t base = 0;
  if (lane == leader && mask) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(active, base, leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

// Geometric normal of a hit in world space, flipped to face the incoming ray:
// normalize(transpose(transform_inv) * n) with n from the triangle record.
__device__ __forceinline__ float3 facing_normal(const TraceParams& p, uint32_t k, uint32_t inst, float3 d) {
  const float4* rec = p.tris + 4 * (size_t)k;
  const float3 n = make_float3(__ldg(&rec[0].w), __ldg(&rec[1].w), __ldg(&rec[2].w));
  const float* m = p.tlas_data[inst].transform_inv;
  const float3 nw = normalize3(make_float3(n.x * __ldg(m + 0) + n.y * __ldg(m + 1) + n.z * __ldg(m + 2),
                                           n.x * __ldg(m + 4) + n.y * __ldg(m + 5) + n.z * __ldg(m + 6),
                                           n.x * __ldg(m + 8) + n.y * __ldg(m + 9) + n.z * __ldg(m + 10)));
  return dot3(nw, d) < 0.0f ? nw : make_float3(-nw.x, -nw.y, -nw.z);
}

}  // namespace dev
}  // namespace rdn
