// Oracle — TEST INFRASTRUCTURE ONLY (see orc_math.h).
//
// Restatement of the reference path tracer
// (scene/rendering/gpu-ray-tracing/src/feature/path_tracing) for one pixel and
// one sample:
//   camera ray: as the AO renderer (orc_ao.h), sampler xxhash32(x, y, sample_count)
//                                                        ray_gen.rs:95-102, camera.rs:66-100
//   core ray: CULL_BACK_FACING_TRIANGLES over [f32::EPSILON, f32::MAX], TLAS 0
//                                                        ray_gen.rs:141-159, api/ty.rs:49-56
//   miss: solid colour, the test gradient or the environment cube
//                                                        ray_miss.rs:10-28,136-152
//   closest hit: world position o + d t, shading / geometric normal
//     (get_world_normal_impl), light sample with PCGRandomSampler(xxhash32(x, y,
//     2 sample_count)), shadow ray ACCEPT_FIRST_HIT_AND_END_SEARCH over
//     [f32::EPSILON, light distance] from offset_ray_hit(position, geometric
//     normal), payload radiance = radiance / pdf (0 when the light sample is
//     invalid, 0 on a shadow hit)                        ray_hit.rs:12-57, mod.rs:197-209
//   uniform light choice: floor(next * count), clamped to count - 1, pmf 1/count
//                                                        lighting_sampler.rs:86-125
//   directional light: direction -dir, distance f32::MAX, radiance illuminance,
//     pdf 1 (times the pmf)                              lighting_sampler.rs:46-69,
//                                                        lighting_bridge.rs:213-258
//   map: surface from the material channels, BRDF importance sample with
//     PCGRandomSampler(xxhash32(x, y, 3 sample_count)), sampled radiance
//     |n.l| bsdf(v, l) radiance                          ray_hit.rs:58-102, surface_bridge.rs:152-224,
//                                                        direct_lighting.rs:14-59
//   physical material: bsdf / pdf = mix(diffuse, specular, specular_estimate),
//     sample chooses specular when next() < estimate     microfacet/device/mod.rs:12-70
//   Lambertian: albedo / pi, cosine sample by Malley's method, pdf max(n.l, 0) / pi
//                                                        microfacet/device/diffuse.rs
//   specular: GGX D, Smith-GGX-correlated G, Schlick F; microfacet normal
//     sample theta = atan(alpha sqrt(u / (1 - u))), reflect; pdf D(m) (n.m) / (4 |m.v|)
//                                                        microfacet/device/specular.rs
//   tbn, concentric disk                                 shader/library/src/sampling.rs:72-119
//   ray generation: hit -> depth + 1 (max_depth when pdf == 0), throughput *=
//     cos brdf / max(pdf, 1e-4), radiance += throughput sampled; miss ->
//     radiance += throughput sampled + surface radiance (0) and the path ends
//                                                        ray_gen.rs:101-150
//   resolve: tone map, (old count + ldr) / (count + 1) into RGBA8, alpha 1
//                                                        ray_gen.rs:160-177, tonemap.rs:53-200
//
// Deliberate differences from the reference's shaders (which use the GPU
// backend's builtins at implementation precision): atan, sin / cos and pow are
// fixed evaluations shared with the CUDA kernels — atan by Cody-Waite reduction
// and the Taylor series to x^15, sin / cos by the pi/2 reduction and Taylor
// polynomials of orc_ao.h / orc_shade.h (the concentric disk uses
// cos(pi/2 - phi) = sin(phi)), pow(x, 5) as (x^2)^2 x, pow(x, 2.2) as
// exp2(2.2 log2 x) from frexp, the atanh series and the Taylor series of
// e^(f ln 2); the unorm8 store rounds to nearest even.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "orc_ao.h"
#include "orc_math.h"
#include "orc_shade.h"

namespace orc {

static const float PT_PI = 3.14159274f;
static const float PT_INV_PI = 0.318309873f;
static const float PT_EPS_SHADING = 0.0001f;

struct PtMaterial {
  float base_color[3];
  float perceptual_roughness;
  float emissive[3];
  float metallic;
  float specular[3];
  float reflectance;
  uint32_t workflow;
  uint32_t reserved[3];
};
struct PtLight {
  float illuminance[3];
  float direction[3];
};
struct PtScene {
  uint32_t max_depth, tone_map, background;
  float exposure;
  float bg[3];
  const PtLight* lights;
  uint32_t light_count;
  const PtMaterial* materials;
  uint32_t material_count;
  const uint32_t* sm_to_material;
  uint32_t sm_count;
  const float* env;  // 6 faces (+X -X +Y -Y +Z -Z) x env_size rows x env_size RGBA texels
  uint32_t env_size;
  float env_transform[16];
  float env_intensity;
};

static inline float pt_mix(float lo, float hi, float t) { return lo * (1.0f - t) + hi * t; }
static inline float saturate(float x) { return rmin(rmax(x, 0.0f), 1.0f); }
// reflect(i, n) = i - 2 dot(n, i) n
static inline V3 pt_reflect(V3 i, V3 n) {
  const float k = 2.0f * dot(n, i);
  return i - n * k;
}

static inline float pt_atan(float x) {
  const bool neg = x < 0.0f;
  float a = std::fabs(x);
  const bool inv = a > 1.0f;
  if (inv) a = 1.0f / a;
  const bool shift = a > 0.267949194f;  // tan(pi/12)
  if (shift) a = (1.73205078f * a - 1.0f) / (a + 1.73205078f);
  const float a2 = a * a;
  float p = -6.66666667e-2f;
  p = 7.69230769e-2f + a2 * p;
  p = -9.09090909e-2f + a2 * p;
  p = 1.11111111e-1f + a2 * p;
  p = -1.42857143e-1f + a2 * p;
  p = 2.00000000e-1f + a2 * p;
  p = -3.33333333e-1f + a2 * p;
  float r = a + a * (a2 * p);
  if (shift) r = 0.52359879f + r;
  if (inv) r = 1.57079637f - r;
  return neg ? -r : r;
}

static inline float pt_log2(float x) {
  int e;
  float m = std::frexp(x, &e);
  if (m < 0.707106769f) {
    m = m * 2.0f;
    e = e - 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = 7.69230769e-2f;
  p = 9.09090909e-2f + s2 * p;
  p = 1.11111111e-1f + s2 * p;
  p = 1.42857143e-1f + s2 * p;
  p = 2.00000000e-1f + s2 * p;
  p = 3.33333333e-1f + s2 * p;
  const float ln_m = 2.0f * (s + s * (s2 * p));
  return (float)e + ln_m * 1.44269502f;
}
static inline float pt_exp2(float y) {
  if (!(y < 128.0f)) return std::isnan(y) ? y : INFINITY;
  if (y < -150.0f) return 0.0f;
  const float n = std::rint(y);
  const float f = (y - n) * 0.693147182f;
  float p = 2.75573192e-7f;
  p = 2.75573192e-6f + f * p;
  p = 2.48015873e-5f + f * p;
  p = 1.98412698e-4f + f * p;
  p = 1.38888889e-3f + f * p;
  p = 8.33333333e-3f + f * p;
  p = 4.16666667e-2f + f * p;
  p = 1.66666667e-1f + f * p;
  p = 0.5f + f * p;
  p = 1.0f + f * p;
  p = 1.0f + f * p;
  return std::ldexp(p, (int)n);
}
static inline float pt_pow(float x, float y) {
  if (x == 0.0f) return 0.0f;
  if (std::isnan(x)) return x;
  return pt_exp2(y * pt_log2(x));
}
static inline float pow5(float x) {
  const float x2 = x * x;
  return (x2 * x2) * x;
}

static inline V3 tbn_mul(V3 n, V3 v) {
  const float sign = n.z < 0.0f ? -1.0f : 1.0f;
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  const V3 t = normalize(v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x));
  const V3 bt = normalize(v3(b, sign + n.y * n.y * a, -n.y));
  return v3(t.x * v.x + bt.x * v.y + n.x * v.z, t.y * v.x + bt.y * v.y + n.y * v.z,
            t.z * v.x + bt.z * v.y + n.z * v.z);
}

struct PtSurface {
  V3 albedo, f0, emissive;
  float alpha, estimate;
};

static inline PtSurface pt_surface(const PtScene& S, uint32_t sm_id) {
  V3 base = v3(0.5f, 0.5f, 0.5f), emissive = v3(0.0f, 0.0f, 0.0f), specular = emissive;
  float pr = 0.5f, metallic = 0.0f, reflectance = 0.5f;
  uint32_t workflow = 0;
  uint32_t idx = 0xFFFFFFFFu;
  if (S.sm_to_material) {
    if (sm_id < S.sm_count) idx = S.sm_to_material[sm_id];
  } else {
    idx = sm_id;
  }
  if (S.materials && idx < S.material_count) {
    const PtMaterial& m = S.materials[idx];
    base = v3(m.base_color[0], m.base_color[1], m.base_color[2]);
    pr = m.perceptual_roughness;
    emissive = v3(m.emissive[0], m.emissive[1], m.emissive[2]);
    metallic = m.metallic;
    specular = v3(m.specular[0], m.specular[1], m.specular[2]);
    reflectance = m.reflectance;
    workflow = m.workflow;
  }
  PtSurface s;
  if (workflow == 1u) {  // specular workflow: metallic = max channel of the specular colour
    const float mt = max_channel(specular);
    s.albedo = base * (1.0f - mt);
    s.f0 = specular;
  } else {
    const float dielectric_f0 = (0.16f * reflectance) * reflectance;  // compute_dielectric_f0
    const float k = dielectric_f0 * (1.0f - metallic);
    s.f0 = v3(base.x * metallic + k, base.y * metallic + k, base.z * metallic + k);
    s.albedo = base * (1.0f - metallic);
  }
  s.emissive = emissive;
  s.alpha = pr * pr;
  s.estimate = pt_mix(0.2f, 1.0f, max_channel(s.f0));
  return s;
}

static inline float ggx_d(float alpha, V3 n, V3 h) {
  const float n_o_h = rmax(dot(n, h), PT_EPS_SHADING);
  const float r2 = alpha * alpha;
  const float d = (n_o_h * r2 - n_o_h) * n_o_h + 1.0f;
  return r2 / ((PT_PI * d) * d);
}

static inline V3 pt_bsdf(const PtSurface& s, V3 v, V3 l, V3 n) {
  const V3 h = normalize(l + v);
  const float p5 = pow5(1.0f - dot(v, h));  // Schlick
  const V3 f = v3(s.f0.x + (1.0f - s.f0.x) * p5, s.f0.y + (1.0f - s.f0.y) * p5, s.f0.z + (1.0f - s.f0.z) * p5);
  // Smith GGX correlated, multiplied back by 4 (n.l) (n.v)
  const float gl = rmax(dot(l, n), PT_EPS_SHADING);
  const float gv = rmax(dot(v, n), PT_EPS_SHADING);
  const float r2 = s.alpha * s.alpha;
  const float vis_v = gv * std::sqrt(gv * (gv - gv * r2) + r2);
  const float vis_l = gl * std::sqrt(gl * (gl - gl * r2) + r2);
  const float g = ((0.5f / (vis_v + vis_l)) * 4.0f * gl) * gv;
  const float d = ggx_d(s.alpha, n, h);
  const float n_dot_l = rmax(dot(l, n), PT_EPS_SHADING);
  const float n_dot_v = rmax(dot(v, n), PT_EPS_SHADING);
  const float dg = d * g;
  const float den = (4.0f * n_dot_l) * n_dot_v;
  const V3 spec = v3((dg * f.x) / den, (dg * f.y) / den, (dg * f.z) / den);
  const V3 diff = v3(s.albedo.x / PT_PI, s.albedo.y / PT_PI, s.albedo.z / PT_PI);
  return v3(pt_mix(diff.x, spec.x, s.estimate), pt_mix(diff.y, spec.y, s.estimate),
            pt_mix(diff.z, spec.z, s.estimate));
}

static inline float pt_pdf(const PtSurface& s, V3 v, V3 l, V3 n) {
  const V3 m = normalize(v + l);
  const float normal_pdf = dot(n, m) * ggx_d(s.alpha, n, m);
  const float spec = normal_pdf / (4.0f * std::fabs(dot(m, v)));
  const float diff = rmax(dot(l, n), 0.0f) * PT_INV_PI;
  return pt_mix(diff, spec, s.estimate);
}

static inline V3 pt_sample(const PtSurface& s, V3 v, V3 n, uint32_t& state, V3* brdf, float* pdf) {
  V3 l;
  if (sample_next(state) < s.estimate) {
    const float u = sample_next(state);
    const float theta = pt_atan(s.alpha * std::sqrt(u / (1.0f - u)));
    float sin_t, cos_t;
    sincos_reduced(theta, &sin_t, &cos_t);
    const float sx = sample_next(state);
    const float sy = sample_next(state);
    float x, y;
    concentric_sample_disk(sx, sy, &x, &y);
    const V3 m = tbn_mul(n, v3(x * sin_t, y * sin_t, cos_t));
    l = pt_reflect(v3(-v.x, -v.y, -v.z), m);
  } else {
    const float sx = sample_next(state);
    const float sy = sample_next(state);
    float x, y;
    concentric_sample_disk(sx, sy, &x, &y);
    const float z = std::sqrt((1.0f - x * x) - y * y);
    l = tbn_mul(n, v3(x, y, z));
  }
  *pdf = pt_pdf(s, v, l, n);
  *brdf = pt_bsdf(s, v, l, n);
  return l;
}

// PTRayMissCtx::EnvCube (ray_miss.rs:139-147): transform_dir (M (d, 1) / w,
// shader/library/src/lib.rs:13-16), the major axis's face (ties x, y, z) with
// the standard face coordinates, bilinear over texel centres clamped to the
// face's edge, f32 weights; black for a non-finite or zero direction.
static inline V3 env_texel(const PtScene& S, uint32_t f, int i, int j) {
  const float* t = S.env + 4 * (((size_t)f * S.env_size + (uint32_t)j) * S.env_size + (uint32_t)i);
  return v3(t[0], t[1], t[2]);
}
static inline V3 lerp3(V3 a, V3 b, float f) {
  return v3(a.x * (1.0f - f) + b.x * f, a.y * (1.0f - f) + b.y * f, a.z * (1.0f - f) + b.z * f);
}
static inline V3 pt_env(const PtScene& S, V3 d) {
  const float* m = S.env_transform;
  const float rx = d.x * m[0] + d.y * m[4] + d.z * m[8] + 1.0f * m[12];
  const float ry = d.x * m[1] + d.y * m[5] + d.z * m[9] + 1.0f * m[13];
  const float rz = d.x * m[2] + d.y * m[6] + d.z * m[10] + 1.0f * m[14];
  const float rw = d.x * m[3] + d.y * m[7] + d.z * m[11] + 1.0f * m[15];
  const float x = rx / rw, y = ry / rw, z = rz / rw;
  const float ax = std::fabs(x), ay = std::fabs(y), az = std::fabs(z);
  if (!(ax <= 3.0e38f && ay <= 3.0e38f && az <= 3.0e38f) || (ax == 0.0f && ay == 0.0f && az == 0.0f))
    return v3(0.0f, 0.0f, 0.0f);
  uint32_t face;
  float sc, tc, ma;
  if (ax >= ay && ax >= az) {
    face = x >= 0.0f ? 0u : 1u;
    sc = x >= 0.0f ? -z : z;
    tc = -y;
    ma = ax;
  } else if (ay >= az) {
    face = y >= 0.0f ? 2u : 3u;
    sc = x;
    tc = y >= 0.0f ? z : -z;
    ma = ay;
  } else {
    face = z >= 0.0f ? 4u : 5u;
    sc = z >= 0.0f ? x : -x;
    tc = -y;
    ma = az;
  }
  const float n = (float)S.env_size;
  const float u = ((sc / ma + 1.0f) * 0.5f) * n - 0.5f;
  const float v = ((tc / ma + 1.0f) * 0.5f) * n - 0.5f;
  const float u0 = std::floor(u), v0 = std::floor(v);
  const float fu = u - u0, fv = v - v0;
  const int last = (int)S.env_size - 1;
  const int i0 = std::min(std::max((int)u0, 0), last), i1 = std::min(std::max((int)u0 + 1, 0), last);
  const int j0 = std::min(std::max((int)v0, 0), last), j1 = std::min(std::max((int)v0 + 1, 0), last);
  const V3 c = lerp3(lerp3(env_texel(S, face, i0, j0), env_texel(S, face, i1, j0), fu),
                     lerp3(env_texel(S, face, i0, j1), env_texel(S, face, i1, j1), fu), fv);
  return c * S.env_intensity;
}

static inline V3 pt_miss(const PtScene& S, V3 d) {
  if (S.background == 1u) return d.y > 0.0f ? v3(0.7f, 0.7f, 0.7f) : v3(0.3f, 0.3f, 0.3f);
  if (S.background == 2u) return pt_env(S, d);
  return v3(S.bg[0], S.bg[1], S.bg[2]);
}

static inline V3 mat3_cols(V3 c0, V3 c1, V3 c2, V3 v) {
  return v3(c0.x * v.x + c1.x * v.y + c2.x * v.z, c0.y * v.x + c1.y * v.y + c2.y * v.z,
            c0.z * v.x + c1.z * v.y + c2.z * v.z);
}

static inline V3 pt_tone_map(const PtScene& S, V3 c) {
  const float ex = S.exposure;
  switch (S.tone_map) {
    case 0:
      return c;
    case 1:
      return v3(ex * c.x, ex * c.y, ex * c.z);
    case 2: {
      const V3 e = v3(ex * c.x, ex * c.y, ex * c.z);
      return v3(saturate(e.x / (1.0f + e.x)), saturate(e.y / (1.0f + e.y)), saturate(e.z / (1.0f + e.z)));
    }
    case 3: {
      V3 e = v3(ex * c.x, ex * c.y, ex * c.z);
      e = v3(rmax(e.x - 0.004f, 0.0f), rmax(e.y - 0.004f, 0.0f), rmax(e.z - 0.004f, 0.0f));
      const V3 num = v3(e.x * (6.2f * e.x + 0.5f), e.y * (6.2f * e.y + 0.5f), e.z * (6.2f * e.z + 0.5f));
      const V3 den = v3(e.x * (6.2f * e.x + 1.7f) + 0.06f, e.y * (6.2f * e.y + 1.7f) + 0.06f,
                        e.z * (6.2f * e.z + 1.7f) + 0.06f);
      return v3(pt_pow(num.x / den.x, 2.2f), pt_pow(num.y / den.y, 2.2f), pt_pow(num.z / den.z, 2.2f));
    }
    default: {  // ACES filmic, the matrices given by their columns
      const float k = ex / 0.6f;
      V3 v = c * k;
      v = mat3_cols(v3(0.59719f, 0.07600f, 0.02840f), v3(0.35458f, 0.90834f, 0.13383f),
                    v3(0.04823f, 0.01566f, 0.83777f), v);
      const V3 a = v3(v.x * (v.x + 0.0245786f) - 0.000090537f, v.y * (v.y + 0.0245786f) - 0.000090537f,
                      v.z * (v.z + 0.0245786f) - 0.000090537f);
      const V3 b = v3(v.x * (0.983729f * v.x + 0.432951f) + 0.238081f, v.y * (0.983729f * v.y + 0.432951f) + 0.238081f,
                      v.z * (0.983729f * v.z + 0.432951f) + 0.238081f);
      v = v3(a.x / b.x, a.y / b.y, a.z / b.z);
      v = mat3_cols(v3(1.60475f, -0.10208f, -0.00327f), v3(-0.53108f, 1.10813f, -0.07276f),
                    v3(-0.07367f, -0.00605f, 1.07602f), v);
      return v3(saturate(v.x), saturate(v.y), saturate(v.z));
    }
  }
}

static inline uint32_t pt_accumulate(uint32_t old, uint32_t sample_count, V3 ldr) {
  const float cnt = (float)sample_count;
  const float all = cnt + 1.0f;
  const float r = ((float)(old & 0xFFu) / 255.0f * cnt + ldr.x) / all;
  const float g = ((float)((old >> 8) & 0xFFu) / 255.0f * cnt + ldr.y) / all;
  const float b = ((float)((old >> 16) & 0xFFu) / 255.0f * cnt + ldr.z) / all;
  return to_unorm8(r) | (to_unorm8(g) << 8) | (to_unorm8(b) << 16) | (255u << 24);
}

}  // namespace orc
