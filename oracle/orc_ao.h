// Oracle — TEST INFRASTRUCTURE ONLY (see orc_math.h).
//
// Restatement of the reference's ray-traced ambient occlusion
// (scene/rendering/gpu-ray-tracing/src/feature/ao.rs) for one pixel and one
// sample:
//   camera ray: uv = pixel / size + (next(), next()) / size with
//     PCGRandomSampler(xxhash32(x, y, sample_count))      feature/ao.rs:193-203,
//     sampler.rs:48-78; DefaultRtxCameraInvocation::generate_ray camera.rs:66-100;
//     shader_uv_space_to_render_space shader/library/src/lib.rs:18-28
//   primary trace: CULL_BACK_FACING_TRIANGLES, [f32::EPSILON, f32::MAX]
//                                                         feature/ao.rs:205-213, api/ty.rs:49-56
//   shading normal: get_world_normal_impl                bindless_mesh_bridge.rs:43-61,86-123
//   occlusion ray: tbn(n) * sample_hemisphere_cos(hammersley_2d(sample, 256)) from
//     the hit position, ACCEPT_FIRST_HIT_AND_END_SEARCH over [0.01, 100]
//                                                         feature/ao.rs:244-276,
//                                                         shader/library/src/sampling.rs:33-83
//   payload 0 on an occlusion hit, 1 on a miss (camera miss: 1)
//                                                         feature/ao.rs:278-297
//   progressive average into an RGBA8 unorm texel        feature/ao.rs:215-237
// The reference's shaders compute cos / sin and the f32 -> unorm8 store with
// the GPU's own builtins (implementation precision); this oracle and the CUDA
// kernels both use a Cody-Waite reduction by pi/2 with the Taylor polynomials
// of orc_shade.h, and round-to-nearest-even for the unorm store.
#pragma once
#include <cmath>
#include <cstdint>

#include "orc_math.h"
#include "orc_shade.h"

namespace orc {

static const uint32_t AO_MAX_SAMPLE = 256;

static inline void sincos_reduced(float phi, float* s, float* c) {
  const float k = std::rint(phi * 0.636619772f);
  const float r = (phi - k * 1.57079637f) - k * -4.37113883e-8f;
  const float ps = poly_sin(r), pc = poly_cos(r);
  const int q = ((int)k) & 3;
  if (q == 0) {
    *s = ps;
    *c = pc;
  } else if (q == 1) {
    *s = pc;
    *c = -ps;
  } else if (q == 2) {
    *s = -ps;
    *c = -pc;
  } else {
    *s = -pc;
    *c = ps;
  }
}

struct AoView {
  float vp_inv[16];
  float cam[3];
  uint32_t width, height, sample_count;
};

static inline void ao_camera_ray(const AoView& A, uint32_t x, uint32_t y, V3* o, V3* d) {
  uint32_t state = xxhash32(x, y, A.sample_count);
  const float j0 = sample_next(state);
  const float j1 = sample_next(state);
  const float fw = (float)A.width, fh = (float)A.height;
  const float ux = (float)x / fw + j0 / fw;
  const float uy = (float)y / fh + j1 / fh;
  const float nx = (ux * 2.0f - 1.0f) * 1.0f;
  const float ny = (uy * 2.0f - 1.0f) * -1.0f;
  const float* m = A.vp_inv;
  const float rx = nx * m[0] + ny * m[4] + 1.0f * m[8] + 1.0f * m[12];
  const float ry = nx * m[1] + ny * m[5] + 1.0f * m[9] + 1.0f * m[13];
  const float rz = nx * m[2] + ny * m[6] + 1.0f * m[10] + 1.0f * m[14];
  const float rw = nx * m[3] + ny * m[7] + 1.0f * m[11] + 1.0f * m[15];
  const V3 target = v3(rx / rw, ry / rw, rz / rw);
  *o = v3(A.cam[0], A.cam[1], A.cam[2]);
  *d = normalize(target - *o);
}

static inline V3 normal_mat_mul(const float* m, V3 n) {
  return v3(n.x * m[0] + n.y * m[1] + n.z * m[2], n.x * m[4] + n.y * m[5] + n.z * m[6],
            n.x * m[8] + n.y * m[9] + n.z * m[10]);
}

// indices / vertices / normals: built arrays; m: the instance's transform_inv.
static inline V3 ao_shading_normal(const uint32_t* indices, const float* vertices, const float* normals,
                                   const float* m, uint32_t tri, float u, float v, V3 ro, V3 hit) {
  const uint32_t i0 = indices[3 * (size_t)tri], i1 = indices[3 * (size_t)tri + 1], i2 = indices[3 * (size_t)tri + 2];
  const V3 pa = v3(vertices[3 * (size_t)i0], vertices[3 * (size_t)i0 + 1], vertices[3 * (size_t)i0 + 2]);
  const V3 pb = v3(vertices[3 * (size_t)i1], vertices[3 * (size_t)i1 + 1], vertices[3 * (size_t)i1 + 2]);
  const V3 pc = v3(vertices[3 * (size_t)i2], vertices[3 * (size_t)i2 + 1], vertices[3 * (size_t)i2 + 2]);
  V3 geom = normalize(normal_mat_mul(m, cross(pa - pb, pa - pc)));
  const V3 hto = ro - hit;
  if (dot(hto, geom) < 0.0f) geom = v3(-geom.x, -geom.y, -geom.z);
  if (!normals) return geom;
  const float b0 = (1.0f - u) - v;
  const V3 na = v3(normals[3 * (size_t)i0], normals[3 * (size_t)i0 + 1], normals[3 * (size_t)i0 + 2]);
  const V3 nb = v3(normals[3 * (size_t)i1], normals[3 * (size_t)i1 + 1], normals[3 * (size_t)i1 + 2]);
  const V3 nc = v3(normals[3 * (size_t)i2], normals[3 * (size_t)i2 + 1], normals[3 * (size_t)i2 + 2]);
  const V3 n = (na * b0 + nb * u) + nc * v;
  V3 shading = normalize(normal_mat_mul(m, n));
  if (dot(geom, shading) < 0.0f) shading = v3(-shading.x, -shading.y, -shading.z);
  return shading;
}

static inline float radical_inverse(uint32_t bits) {
  bits = (bits << 16) | (bits >> 16);
  bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
  bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
  bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
  bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
  return (float)bits * 2.3283064e-10f;
}

static inline V3 ao_direction(V3 n, uint32_t sample) {
  const float hx = (float)sample / (float)AO_MAX_SAMPLE;
  const float hy = radical_inverse(sample);
  const float phi = 6.28318548f * hy;
  const float cos_theta = std::sqrt(1.0f - hx);
  const float sin_theta = std::sqrt(1.0f - cos_theta * cos_theta);
  float sp, cp;
  sincos_reduced(phi, &sp, &cp);
  const float lx = cp * sin_theta, ly = sp * sin_theta, lz = cos_theta;
  const float sign = n.z < 0.0f ? -1.0f : 1.0f;
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  const V3 t = normalize(v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x));
  const V3 bt = normalize(v3(b, sign + n.y * n.y * a, -n.y));
  return v3(t.x * lx + bt.x * ly + n.x * lz, t.y * lx + bt.y * ly + n.y * lz, t.z * lx + bt.z * ly + n.z * lz);
}

static inline uint32_t to_unorm8(float x) {
  return (uint32_t)std::rint(rmin(rmax(x, 0.0f), 1.0f) * 255.0f);
}

static inline uint32_t ao_accumulate(uint32_t old, uint32_t sample_count, float payload) {
  const float prev = (float)(old & 0xFFu) / 255.0f;
  const float prev_count = (float)sample_count;
  const float all = prev_count + 1.0f;
  const float next = (prev * prev_count + payload) / all;
  const float w = sample_count < AO_MAX_SAMPLE ? next : prev;
  const uint32_t q = to_unorm8(w);
  return q | (q << 8) | (q << 16) | (255u << 24);
}

}  // namespace orc
