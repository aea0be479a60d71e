// Ambient-occlusion shading of the reference's ray-traced AO renderer
// (scene/rendering/gpu-ray-tracing/src/feature/ao.rs), restated for the device:
//   camera ray with PCG jitter           feature/ao.rs:193-213, camera.rs:66-100,
//                                        sampler.rs:48-78, shader/library/src/lib.rs:18-28
//   world shading / geometric normal     bindless_mesh_bridge.rs:43-61,86-123
//   hit position                         shader/ray-tracing/src/api/ctx.rs:209-211
//   tbn, hammersley, cosine hemisphere   shader/library/src/sampling.rs:33-83
//   occlusion ray, payload 1 / 0         feature/ao.rs:244-296
//   progressive average into RGBA8       feature/ao.rs:215-237
// Every unit that includes this header is built with -fmad=false; cos / sin
// of the hemisphere sample use a Cody-Waite reduction by pi/2 and the fixed
// Taylor polynomials of shade.cuh, evaluated identically by the oracle.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "shade.cuh"
#include "task_graph.h"

namespace rdn {
namespace dev {

constexpr uint32_t AO_MAX_SAMPLE = 256;  // feature/ao.rs:7
constexpr float AO_TEST_MIN = 0.01f, AO_TEST_MAX = 100.0f;
constexpr uint32_t RAY_FLAG_END_SEARCH = 0x04u, RAY_FLAG_CULL_BACK = 0x10u, RAY_FLAG_SKIP_CLOSEST = 0x08u;

// (sin, cos) of phi >= 0: k = nearest integer of phi / (pi/2), r = phi - k*pi/2
// in two steps (Cody-Waite, pi/2 = C1 + C2), then the quadrant's polynomials.
__device__ __forceinline__ void sincos_reduced(float phi, float& s, float& c) {
  const float k = rintf(phi * 0.636619772f);
  const float r = (phi - k * 1.57079637f) - k * -4.37113883e-8f;
  const float ps = poly_sin(r), pc = poly_cos(r);
  const int q = ((int)k) & 3;
  if (q == 0) {
    s = ps;
    c = pc;
  } else if (q == 1) {
    s = pc;
    c = -ps;
  } else if (q == 2) {
    s = -ps;
    c = -pc;
  } else {
    s = -pc;
    c = ps;
  }
}

// Pixel of dispatch index i: each run of 32 indices covers a 4x8 tile (4 wide,
// 8 tall), tiles in row order (a warp traces one tile). Indices of the tiles' overhang past
// the frame return false.
__device__ __forceinline__ bool ao_pixel(const AoEnv& A, uint32_t i, uint32_t& x, uint32_t& y) {
  const uint32_t tiles_x = (A.width + 3) / 4, t = i >> 5, lane = i & 31u;
  x = (t % tiles_x) * 4 + (lane & 3u);
  y = (t / tiles_x) * 8 + (lane >> 2);
  return x < A.width && y < A.height;
}

// Mat4 * (x, y, z, w), Mat4 in the reference's column order.
__device__ __forceinline__ float4 mat4_mul(const float* m, float x, float y, float z, float w) {
  return make_float4(x * m[0] + y * m[4] + z * m[8] + w * m[12], x * m[1] + y * m[5] + z * m[9] + w * m[13],
                     x * m[2] + y * m[6] + z * m[10] + w * m[14], x * m[3] + y * m[7] + z * m[11] + w * m[15]);
}

// Sample index of the frame: the device counter when the frame reads one.
__device__ __forceinline__ uint32_t ao_sample(const AoEnv& A) { return A.sample_dev ? *A.sample_dev : A.sample_count; }

// DefaultRtxCameraInvocation::generate_ray with PCGRandomSampler seeded by
// xxhash32(x, y, sample index); next_2d = (next(), next()).
__device__ __forceinline__ void ao_camera_ray(const AoEnv& A, uint32_t x, uint32_t y, float3& o, float3& d) {
  uint32_t state = xxhash32(x, y, ao_sample(A));
  const float j0 = sample_next(state);
  const float j1 = sample_next(state);
  const float fw = (float)A.width, fh = (float)A.height;
  const float ux = (float)x / fw + j0 / fw;
  const float uy = (float)y / fh + j1 / fh;
  const float nx = (ux * 2.0f - 1.0f) * 1.0f;
  const float ny = (uy * 2.0f - 1.0f) * -1.0f;
  const float4 r = mat4_mul(A.vp_inv, nx, ny, 1.0f, 1.0f);
  const float3 target = make_float3(r.x / r.w, r.y / r.w, r.z / r.w);
  o = make_float3(A.cam[0], A.cam[1], A.cam[2]);
  d = normalize3(target - o);
}

__device__ __forceinline__ float3 ld_vertex(const float* v, uint32_t i) {
  return make_float3(__ldg(v + 3 * (size_t)i), __ldg(v + 3 * (size_t)i + 1), __ldg(v + 3 * (size_t)i + 2));
}
// transpose(shrink_to_3(world_to_object)) * n
__device__ __forceinline__ float3 normal_mat_mul(const float* m, float3 n) {
  return make_float3(n.x * __ldg(m + 0) + n.y * __ldg(m + 1) + n.z * __ldg(m + 2),
                     n.x * __ldg(m + 4) + n.y * __ldg(m + 5) + n.z * __ldg(m + 6),
                     n.x * __ldg(m + 8) + n.y * __ldg(m + 9) + n.z * __ldg(m + 10));
}

// Shading and geometric normals of a hit (get_world_normal_impl), oriented like
// the reference: the geometric normal towards the ray origin, the shading
// normal into the geometric normal's hemisphere. Without vertex normals the
// shading normal is the oriented geometric normal.
__device__ __forceinline__ float3 hit_normals(const AoEnv& A, const DeviceInstance* inst, uint32_t tri, float u,
                                              float v, float3 ro, float3 hit, float3& geom) {
  const uint32_t i0 = __ldg(A.indices + 3 * (size_t)tri), i1 = __ldg(A.indices + 3 * (size_t)tri + 1),
                 i2 = __ldg(A.indices + 3 * (size_t)tri + 2);
  const float* m = inst->transform_inv;
  const float3 pa = ld_vertex(A.vertices, i0), pb = ld_vertex(A.vertices, i1), pc = ld_vertex(A.vertices, i2);
  geom = normalize3(normal_mat_mul(m, cross3(pa - pb, pa - pc)));
  const float3 hto = ro - hit;
  if (dot3(hto, geom) < 0.0f) geom = make_float3(-geom.x, -geom.y, -geom.z);
  if (!A.normals) return geom;
  const float b0 = (1.0f - u) - v;
  const float3 na = ld_vertex(A.normals, i0), nb = ld_vertex(A.normals, i1), nc = ld_vertex(A.normals, i2);
  const float3 n = (na * b0 + nb * u) + nc * v;
  float3 shading = normalize3(normal_mat_mul(m, n));
  if (dot3(geom, shading) < 0.0f) shading = make_float3(-shading.x, -shading.y, -shading.z);
  return shading;
}
__device__ __forceinline__ float3 ao_shading_normal(const AoEnv& A, const DeviceInstance* inst, uint32_t tri,
                                                    float u, float v, float3 ro, float3 hit) {
  float3 geom;
  return hit_normals(A, inst, tri, u, v, ro, hit, geom);
}

// radical_inverse_vdc: bit reversal, times 2^-32
__device__ __forceinline__ float radical_inverse(uint32_t bits) {
  bits = (bits << 16) | (bits >> 16);
  bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
  bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
  bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
  bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
  return __uint2float_rn(bits) * 2.3283064e-10f;
}

// tbn(normal) * sample_hemisphere_cos(hammersley_2d(sample, 256))
__device__ __forceinline__ float3 ao_direction(float3 n, uint32_t sample) {
  const float hx = __uint2float_rn(sample) / __uint2float_rn(AO_MAX_SAMPLE);
  const float hy = radical_inverse(sample);
  const float phi = 6.28318548f * hy;
  const float cos_theta = sqrtf(1.0f - hx);
  const float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
  float sp, cp;
  sincos_reduced(phi, sp, cp);
  const float lx = cp * sin_theta, ly = sp * sin_theta, lz = cos_theta;
  const float sign = n.z < 0.0f ? -1.0f : 1.0f;
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  const float3 t = normalize3(make_float3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x));
  const float3 bt = normalize3(make_float3(b, sign + n.y * n.y * a, -n.y));
  return make_float3(t.x * lx + bt.x * ly + n.x * lz, t.y * lx + bt.y * ly + n.y * lz,
                     t.z * lx + bt.z * ly + n.z * lz);
}

// Adds the lanes that want it to counter k of the AO ray counts, one atomic per warp.
__device__ __forceinline__ void ao_count(const AoEnv& A, uint32_t k, bool want) {
  if (!A.ray_counts) return;
  const uint32_t active = __activemask();
  const uint32_t mask = __ballot_sync(active, want);
  if ((threadIdx.x & 31u) == (uint32_t)(__ffs(active) - 1) && mask) atomicAdd(A.ray_counts + k, __popc(mask));
}

__device__ __forceinline__ uint32_t to_unorm8(float x) {
  return (uint32_t)rintf(fminf(fmaxf(x, 0.0f), 1.0f) * 255.0f);
}

// Ray-gen map of the AO renderer: running average of the occlusion payloads
// in an RGBA8 unorm texel (alpha 1), frozen after AO_MAX_SAMPLE samples.
__device__ __forceinline__ void ao_accumulate(const AoEnv& A, uint32_t pixel, float payload) {
  uint32_t* texel = reinterpret_cast<uint32_t*>(A.image) + pixel;
  const uint32_t old = *texel;
  const float prev = (float)(old & 0xFFu) / 255.0f;
  const uint32_t count = ao_sample(A);
  const float prev_count = (float)count;
  const float all = prev_count + 1.0f;
  const float next = (prev * prev_count + payload) / all;
  const float w = count < AO_MAX_SAMPLE ? next : prev;
  const uint32_t q = to_unorm8(w);
  *texel = q | (q << 8) | (q << 16) | (255u << 24);
}

}  // namespace dev
}  // namespace rdn
