// Shading of the reference path tracer, restated for the device:
//   PCGRandomSampler(xxhash32(x, y, k * sample_count)), k = 2 for the light
//   sample, 3 for the BRDF sample        path_tracing/ray_hit.rs:17-19,62-64, sampler.rs:48-72
//   uniform light index, pmf 1/count     path_tracing/lighting_sampler.rs:86-125
//   directional light: -direction, f32::MAX, illuminance, pdf 1
//                                        path_tracing/lighting_bridge.rs:213-258
//   physical shading from the material   lighting/transport/.../device/direct_lighting.rs:14-59
//   surface point (alpha = roughness^2)  path_tracing/surface_bridge.rs:171-224
//   Lambertian + GGX / Smith-GGX-correlated / Schlick specular mixed by
//   mix(0.2, 1, max f0): bsdf, pdf and importance sample
//                                        lighting/transport/src/surface/microfacet/device/{mod,diffuse,specular}.rs
//   tbn, concentric disk                 shader/library/src/sampling.rs:72-119
//   miss radiance (solid colour, test, environment cube)
//                                        path_tracing/ray_miss.rs:136-152
//   tone maps                            content/texture/gpu-process/src/tonemap.rs:53-200
//
// The reference's shaders evaluate atan, sin, cos and pow with the GPU
// backend's builtins (implementation precision). Here atan, pow and cos/sin are
// written from published methods and evaluated identically by the oracle:
//   atan: Cody-Waite argument reduction (x > 1 -> pi/2 - atan(1/x), then
//     x > tan(pi/12) -> pi/6 + atan((sqrt3 x - 1) / (x + sqrt3))) and the Taylor
//     series to x^15 (|x| <= tan(pi/12): truncation < 2e-11);
//   sin / cos: the pi/2 reduction and Taylor polynomials of ao.cuh / shade.cuh;
//   pow(x, 5) in Schlick's term as (x^2)^2 x; pow(x, 2.2) of the Cineon curve
//     as exp2(2.2 log2 x) with log2 from frexp and the atanh series
//     (ln m = 2 atanh((m-1)/(m+1)), m in [sqrt(1/2), sqrt(2))) and exp2 from
//     rint + the Taylor series of e^(f ln 2) to degree 10, scaled by ldexp.
// Every unit that includes this header is built with -fmad=false.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "ao.cuh"
#include "pt.h"

namespace rdn {
namespace dev {

constexpr float PT_PI = 3.14159274f;
constexpr float PT_INV_PI = 0.318309873f;
constexpr float PT_EPSILON_SHADING = 0.0001f;
constexpr float PT_MIN_PDF = 0.0001f;

__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 splat3(float s) { return make_float3(s, s, s); }
__device__ __forceinline__ float3 neg3(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float max_ch(float3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
__device__ __forceinline__ float saturate1(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
// WGSL mix(lo, hi, t) = lo * (1 - t) + hi * t
__device__ __forceinline__ float mix1(float lo, float hi, float t) { return lo * (1.0f - t) + hi * t; }
__device__ __forceinline__ float3 mix3(float3 lo, float3 hi, float t) {
  return make_float3(mix1(lo.x, hi.x, t), mix1(lo.y, hi.y, t), mix1(lo.z, hi.z, t));
}
// WGSL reflect(i, n) = i - 2 dot(n, i) n  (Node::reflect: self is the normal)
__device__ __forceinline__ float3 reflect3(float3 i, float3 n) {
  const float k = 2.0f * dot3(n, i);
  return i - n * k;
}

// atan(x), x >= 0 (the GGX sample's argument is never negative; odd symmetry otherwise)
__device__ __forceinline__ float pt_atan(float x) {
  const bool neg = x < 0.0f;
  float a = fabsf(x);
  const bool inv = a > 1.0f;
  if (inv) a = 1.0f / a;
  const bool shift = a > 0.267949194f;  // tan(pi/12)
  if (shift) a = (1.73205078f * a - 1.0f) / (a + 1.73205078f);
  const float a2 = a * a;
  float p = -6.66666667e-2f;   // -1/15
  p = 7.69230769e-2f + a2 * p;  // 1/13
  p = -9.09090909e-2f + a2 * p; // -1/11
  p = 1.11111111e-1f + a2 * p;  // 1/9
  p = -1.42857143e-1f + a2 * p; // -1/7
  p = 2.00000000e-1f + a2 * p;  // 1/5
  p = -3.33333333e-1f + a2 * p; // -1/3
  float r = a + a * (a2 * p);
  if (shift) r = 0.52359879f + r;
  if (inv) r = 1.57079637f - r;
  return neg ? -r : r;
}

// log2(x), x > 0 finite
__device__ __forceinline__ float pt_log2(float x) {
  int e;
  float m = frexpf(x, &e);  // x = m 2^e, m in [1/2, 1)
  if (m < 0.707106769f) {
    m = m * 2.0f;
    e = e - 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = 7.69230769e-2f;     // 1/13
  p = 9.09090909e-2f + s2 * p;  // 1/11
  p = 1.11111111e-1f + s2 * p;  // 1/9
  p = 1.42857143e-1f + s2 * p;  // 1/7
  p = 2.00000000e-1f + s2 * p;  // 1/5
  p = 3.33333333e-1f + s2 * p;  // 1/3
  const float ln_m = 2.0f * (s + s * (s2 * p));
  return (float)e + ln_m * 1.44269502f;
}
// 2^y
__device__ __forceinline__ float pt_exp2(float y) {
  if (!(y < 128.0f)) return y != y ? y : __int_as_float(0x7f800000);
  if (y < -150.0f) return 0.0f;
  const float n = rintf(y);
  const float f = (y - n) * 0.693147182f;
  float p = 2.75573192e-7f;     // 1/10!
  p = 2.75573192e-6f + f * p;   // 1/9!
  p = 2.48015873e-5f + f * p;   // 1/8!
  p = 1.98412698e-4f + f * p;   // 1/7!
  p = 1.38888889e-3f + f * p;   // 1/6!
  p = 8.33333333e-3f + f * p;   // 1/5!
  p = 4.16666667e-2f + f * p;   // 1/4!
  p = 1.66666667e-1f + f * p;   // 1/3!
  p = 0.5f + f * p;             // 1/2!
  p = 1.0f + f * p;
  p = 1.0f + f * p;
  return ldexpf(p, (int)n);
}
// pow(x, y) for x >= 0 (WGSL pow is undefined below 0)
__device__ __forceinline__ float pt_pow(float x, float y) {
  if (x == 0.0f) return 0.0f;
  if (x != x) return x;
  return pt_exp2(y * pt_log2(x));
}
__device__ __forceinline__ float pow5(float x) {
  const float x2 = x * x;
  return (x2 * x2) * x;
}

// tbn(normal) * v: the orthonormal basis of Duff et al. 2017 ("Building an
// Orthonormal Basis, Revisited"), as shader/library/src/sampling.rs:70-83 builds it
__device__ __forceinline__ float3 tbn_mul(float3 n, float3 v) {
  const float sign = n.z < 0.0f ? -1.0f : 1.0f;
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  const float3 t = normalize3(make_float3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x));
  const float3 bt = normalize3(make_float3(b, sign + n.y * n.y * a, -n.y));
  return make_float3(t.x * v.x + bt.x * v.y + n.x * v.z, t.y * v.x + bt.y * v.y + n.y * v.z,
                     t.z * v.x + bt.z * v.y + n.z * v.z);
}

// concentric_sample_disk_device of (next(), next())
__device__ __forceinline__ void concentric_disk(uint32_t& state, float& dx, float& dy) {
  const float sx = sample_next(state);
  const float sy = sample_next(state);
  const float ux = sx * 2.0f - 1.0f, uy = sy * 2.0f - 1.0f;
  dx = 0.0f;
  dy = 0.0f;
  if (ux == 0.0f && uy == 0.0f) return;
  float r, c, s;
  if (fabsf(ux) > fabsf(uy)) {
    r = ux;
    const float phi = 0.78539819f * (uy / ux);
    c = poly_cos(phi);
    s = poly_sin(phi);
  } else {
    r = uy;
    const float phi = 0.78539819f * (ux / uy);  // theta = pi/2 - phi
    c = poly_sin(phi);
    s = poly_cos(phi);
  }
  dx = c * r;
  dy = s * r;
}

// ShaderPhysicalShading -> the surface point's parameters
struct PtSurface {
  float3 albedo, f0, emissive;
  float alpha;     // alpha roughness = perceptual^2
  float estimate;  // specular_estimate = mix(0.2, 1, max channel of f0)
};

__device__ __forceinline__ PtSurface pt_surface(const PtEnv& E, uint32_t sm_id) {
  float3 base = splat3(0.5f), emissive = splat3(0.0f), specular = splat3(0.0f);
  float pr = 0.5f, metallic = 0.0f, reflectance = 0.5f;
  uint32_t workflow = 0;
  uint32_t idx = 0xFFFFFFFFu;
  if (E.sm_to_material) {
    if (sm_id < E.sm_count) idx = __ldg(E.sm_to_material + sm_id);
  } else {
    idx = sm_id;
  }
  if (E.materials && idx < E.material_count) {
    const float* m = reinterpret_cast<const float*>(E.materials + idx);
    base = make_float3(__ldg(m + 0), __ldg(m + 1), __ldg(m + 2));
    pr = __ldg(m + 3);
    emissive = make_float3(__ldg(m + 4), __ldg(m + 5), __ldg(m + 6));
    metallic = __ldg(m + 7);
    specular = make_float3(__ldg(m + 8), __ldg(m + 9), __ldg(m + 10));
    reflectance = __ldg(m + 11);
    workflow = __ldg(reinterpret_cast<const uint32_t*>(m) + 12);
  }
  PtSurface s;
  if (workflow == 1u) {
    const float mt = max_ch(specular);
    s.albedo = base * (1.0f - mt);
    s.f0 = specular;
  } else {
    const float dielectric_f0 = (0.16f * reflectance) * reflectance;
    const float k = dielectric_f0 * (1.0f - metallic);
    s.f0 = make_float3(base.x * metallic + k, base.y * metallic + k, base.z * metallic + k);
    s.albedo = base * (1.0f - metallic);
  }
  s.emissive = emissive;
  s.alpha = pr * pr;
  s.estimate = mix1(0.2f, 1.0f, max_ch(s.f0));
  return s;
}

// ShaderGGX::d
__device__ __forceinline__ float ggx_d(float alpha, float3 n, float3 h) {
  const float n_o_h = fmaxf(dot3(n, h), PT_EPSILON_SHADING);
  const float r2 = alpha * alpha;
  const float d = (n_o_h * r2 - n_o_h) * n_o_h + 1.0f;
  return r2 / ((PT_PI * d) * d);
}

// ShaderRtxPhysicalMaterial::bsdf
__device__ __forceinline__ float3 pt_bsdf(const PtSurface& s, float3 v, float3 l, float3 n) {
  const float3 h = normalize3(l + v);
  const float p5 = pow5(1.0f - dot3(v, h));
  const float3 f = make_float3(s.f0.x + (1.0f - s.f0.x) * p5, s.f0.y + (1.0f - s.f0.y) * p5,
                               s.f0.z + (1.0f - s.f0.z) * p5);
  const float n_dot_l_g = fmaxf(dot3(l, n), PT_EPSILON_SHADING);
  const float n_dot_v_g = fmaxf(dot3(v, n), PT_EPSILON_SHADING);
  const float r2 = s.alpha * s.alpha;
  const float vis_v = n_dot_v_g * sqrtf(n_dot_v_g * (n_dot_v_g - n_dot_v_g * r2) + r2);
  const float vis_l = n_dot_l_g * sqrtf(n_dot_l_g * (n_dot_l_g - n_dot_l_g * r2) + r2);
  const float g = ((0.5f / (vis_v + vis_l)) * 4.0f * n_dot_l_g) * n_dot_v_g;
  const float d = ggx_d(s.alpha, n, h);
  const float n_dot_l = fmaxf(dot3(l, n), PT_EPSILON_SHADING);
  const float n_dot_v = fmaxf(dot3(v, n), PT_EPSILON_SHADING);
  const float dg = d * g;
  const float den = (4.0f * n_dot_l) * n_dot_v;
  const float3 spec = make_float3((dg * f.x) / den, (dg * f.y) / den, (dg * f.z) / den);
  const float3 diff = s.albedo / PT_PI;
  return mix3(diff, spec, s.estimate);
}

// ShaderRtxPhysicalMaterial::pdf
__device__ __forceinline__ float pt_pdf(const PtSurface& s, float3 v, float3 l, float3 n) {
  const float3 m = normalize3(v + l);
  const float normal_pdf = dot3(n, m) * ggx_d(s.alpha, n, m);
  const float spec = normal_pdf / (4.0f * fabsf(dot3(m, v)));
  const float diff = fmaxf(dot3(l, n), 0.0f) * PT_INV_PI;
  return mix1(diff, spec, s.estimate);
}

// sample_light_dir_use_bsdf_importance: direction, bsdf and pdf
__device__ __forceinline__ float3 pt_sample(const PtSurface& s, float3 v, float3 n, uint32_t& state, float3& brdf,
                                            float& pdf) {
  float3 l;
  if (sample_next(state) < s.estimate) {
    const float u = sample_next(state);
    const float theta = pt_atan(s.alpha * sqrtf(u / (1.0f - u)));
    float sin_t, cos_t;
    sincos_reduced(theta, sin_t, cos_t);
    float x, y;
    concentric_disk(state, x, y);
    const float3 m = tbn_mul(n, make_float3(x * sin_t, y * sin_t, cos_t));
    l = reflect3(neg3(v), m);
  } else {
    float x, y;
    concentric_disk(state, x, y);
    const float z = sqrtf((1.0f - x * x) - y * y);
    l = tbn_mul(n, make_float3(x, y, z));
  }
  pdf = pt_pdf(s, v, l, n);
  brdf = pt_bsdf(s, v, l, n);
  return l;
}

// Texel (i, j) of cube face f.
__device__ __forceinline__ float3 env_texel(const PtEnv& E, uint32_t f, int i, int j) {
  const float4 c = __ldg(E.env + ((size_t)f * E.env_size + (uint32_t)j) * E.env_size + (uint32_t)i);
  return make_float3(c.x, c.y, c.z);
}
__device__ __forceinline__ float3 lerp3(float3 a, float3 b, float f) {
  return make_float3(a.x * (1.0f - f) + b.x * f, a.y * (1.0f - f) + b.y * f, a.z * (1.0f - f) + b.z * f);
}

// EnvCube: transform_dir (shader/library/src/lib.rs:13-16: M (d, 1), divided
// by w), then the cube face of the major axis (ties: x before y before z) with
// the standard face coordinates, bilinear over texel centres, clamped to the
// face's edge, at level 0; times the intensity (ray_miss.rs:139-147). The
// reference samples a GPU cube texture: its filter weights are the texture
// unit's fixed-point ones and it blends across face edges; here the weights
// are f32 and each face is clamped to its own edge. A non-finite or zero
// direction samples black.
__device__ __forceinline__ float3 pt_env(const PtEnv& E, float3 d) {
  const float* m = E.env_transform;
  const float rx = d.x * m[0] + d.y * m[4] + d.z * m[8] + 1.0f * m[12];
  const float ry = d.x * m[1] + d.y * m[5] + d.z * m[9] + 1.0f * m[13];
  const float rz = d.x * m[2] + d.y * m[6] + d.z * m[10] + 1.0f * m[14];
  const float rw = d.x * m[3] + d.y * m[7] + d.z * m[11] + 1.0f * m[15];
  const float x = rx / rw, y = ry / rw, z = rz / rw;
  const float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
  if (!(ax <= 3.0e38f && ay <= 3.0e38f && az <= 3.0e38f) || (ax == 0.0f && ay == 0.0f && az == 0.0f))
    return splat3(0.0f);
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
  const float n = (float)E.env_size;
  const float u = ((sc / ma + 1.0f) * 0.5f) * n - 0.5f;
  const float v = ((tc / ma + 1.0f) * 0.5f) * n - 0.5f;
  const float u0 = floorf(u), v0 = floorf(v);
  const float fu = u - u0, fv = v - v0;
  const int last = (int)E.env_size - 1;
  const int i0 = min(max((int)u0, 0), last), i1 = min(max((int)u0 + 1, 0), last);
  const int j0 = min(max((int)v0, 0), last), j1 = min(max((int)v0 + 1, 0), last);
  const float3 c = lerp3(lerp3(env_texel(E, face, i0, j0), env_texel(E, face, i1, j0), fu),
                         lerp3(env_texel(E, face, i0, j1), env_texel(E, face, i1, j1), fu), fv);
  return c * E.env_intensity;
}

// PTRayMissCtxInvocation::sample_radiance
__device__ __forceinline__ float3 pt_miss(const PtEnv& E, float3 d) {
  if (E.background == PT_BACKGROUND_TEST) return d.y > 0.0f ? splat3(0.7f) : splat3(0.3f);
  if (E.background == PT_BACKGROUND_ENV_CUBE) return pt_env(E, d);
  return make_float3(E.bg[0], E.bg[1], E.bg[2]);
}

__device__ __forceinline__ float3 rrt_odt_fit(float3 v) {
  const float3 a = make_float3(v.x * (v.x + 0.0245786f) - 0.000090537f, v.y * (v.y + 0.0245786f) - 0.000090537f,
                               v.z * (v.z + 0.0245786f) - 0.000090537f);
  const float3 b = make_float3(v.x * (0.983729f * v.x + 0.432951f) + 0.238081f,
                               v.y * (0.983729f * v.y + 0.432951f) + 0.238081f,
                               v.z * (0.983729f * v.z + 0.432951f) + 0.238081f);
  return make_float3(a.x / b.x, a.y / b.y, a.z / b.z);
}
// Mat3 given by its columns c0, c1, c2, times v
__device__ __forceinline__ float3 mat3_cols(float3 c0, float3 c1, float3 c2, float3 v) {
  return make_float3(c0.x * v.x + c1.x * v.y + c2.x * v.z, c0.y * v.x + c1.y * v.y + c2.y * v.z,
                     c0.z * v.x + c1.z * v.y + c2.z * v.z);
}

// ToneMapInvocation::compute_ldr
__device__ __forceinline__ float3 pt_tone_map(const PtEnv& E, float3 c) {
  const float ex = E.exposure;
  switch (E.tone_map) {
    case PT_TONE_NONE:
      return c;
    case PT_TONE_LINEAR:
      return make_float3(ex * c.x, ex * c.y, ex * c.z);
    case PT_TONE_REINHARD: {
      const float3 e = make_float3(ex * c.x, ex * c.y, ex * c.z);
      return make_float3(saturate1(e.x / (1.0f + e.x)), saturate1(e.y / (1.0f + e.y)), saturate1(e.z / (1.0f + e.z)));
    }
    case PT_TONE_CINEON: {
      float3 e = make_float3(ex * c.x, ex * c.y, ex * c.z);
      e = make_float3(fmaxf(e.x - 0.004f, 0.0f), fmaxf(e.y - 0.004f, 0.0f), fmaxf(e.z - 0.004f, 0.0f));
      const float3 num = make_float3(e.x * (6.2f * e.x + 0.5f), e.y * (6.2f * e.y + 0.5f), e.z * (6.2f * e.z + 0.5f));
      const float3 den = make_float3(e.x * (6.2f * e.x + 1.7f) + 0.06f, e.y * (6.2f * e.y + 1.7f) + 0.06f,
                                     e.z * (6.2f * e.z + 1.7f) + 0.06f);
      return make_float3(pt_pow(num.x / den.x, 2.2f), pt_pow(num.y / den.y, 2.2f), pt_pow(num.z / den.z, 2.2f));
    }
    default: {  // ACES filmic
      const float k = ex / 0.6f;
      float3 v = c * k;
      v = mat3_cols(make_float3(0.59719f, 0.07600f, 0.02840f), make_float3(0.35458f, 0.90834f, 0.13383f),
                    make_float3(0.04823f, 0.01566f, 0.83777f), v);
      v = rrt_odt_fit(v);
      v = mat3_cols(make_float3(1.60475f, -0.10208f, -0.00327f), make_float3(-0.53108f, 1.10813f, -0.07276f),
                    make_float3(-0.07367f, -0.00605f, 1.07602f), v);
      return make_float3(saturate1(v.x), saturate1(v.y), saturate1(v.z));
    }
  }
}

// Ray-gen resolve: (old * sample_count + ldr) / (sample_count + 1) into the
// RGBA8 unorm texel, alpha 1.
__device__ __forceinline__ void pt_accumulate(const PtEnv& E, uint32_t pixel, float3 ldr) {
  uint32_t* texel = reinterpret_cast<uint32_t*>(E.view.image) + pixel;
  const uint32_t old = *texel;
  const float cnt = (float)ao_sample(E.view);
  const float all = cnt + 1.0f;
  const float r = ((float)(old & 0xFFu) / 255.0f * cnt + ldr.x) / all;
  const float g = ((float)((old >> 8) & 0xFFu) / 255.0f * cnt + ldr.y) / all;
  const float b = ((float)((old >> 16) & 0xFFu) / 255.0f * cnt + ldr.z) / all;
  *texel = to_unorm8(r) | (to_unorm8(g) << 8) | (to_unorm8(b) << 16) | (255u << 24);
}

}  // namespace dev
}  // namespace rdn
