// Oracle — TEST INFRASTRUCTURE ONLY. Nothing in the product (rendiation_gb300/,
// include/) may include, link or call this code; only tests/, the smoke check and
// bench.py's cpu_baseline / reference arm use it, and only as the checker.
//
// f32 math restated from the reference crates with the exact operation order of
// the Rust source (Rust never contracts a*b+c into an FMA, so this file must be
// compiled with -ffp-contract=off and without fast-math).
//
//   Vec3 ops / dot / cross     math/algebra/src/vec/vec3.rs:26-28,116-122
//   normalize (zero unchanged)  math/algebra/src/vec/dimension.rs:98-105
//   min/max (NaN-ignoring)      math/algebra/src/vec/dimension.rs:53-60 (f32::min/max)
//   Box3 empty/expand/union     math/geometry/src/hyper_aabb.rs:20-68
//   Box3 centre / SA / axis     math/geometry/src/dimension3/box3.rs:5-11,90-93,117-133
//   Box3 apply_matrix           math/geometry/src/dimension3/box3.rs:20-39
//   Mat4 * Vec4, det, inverse   math/algebra/src/mat/mat4.rs:40-104,155-169
//   Mat3 * Vec3, det            math/algebra/src/mat/mat3.rs:37-42,97-110
#pragma once
#include <cmath>
#include <cstdint>
#include <cstddef>
#include <limits>

namespace orc {

struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
static inline V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }

// Rust f32::min / f32::max: if one operand is NaN the other is returned.
static inline float rmin(float a, float b) { return std::fmin(a, b); }
static inline float rmax(float a, float b) { return std::fmax(a, b); }
static inline V3 vmin(V3 a, V3 b) { return v3(rmin(a.x, b.x), rmin(a.y, b.y), rmin(a.z, b.z)); }
static inline V3 vmax(V3 a, V3 b) { return v3(rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z)); }
static inline float max_channel(V3 a) { return rmax(rmax(a.x, a.y), a.z); }
static inline float min_channel(V3 a) { return rmin(rmin(a.x, a.y), a.z); }

static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline V3 normalize(V3 v) {
  float mag_sq = dot(v, v);
  if (mag_sq > 0.0f) {
    float inv_sqrt = 1.0f / std::sqrt(mag_sq);
    return v * inv_sqrt;
  }
  return v;
}
static inline float length(V3 v) { return std::sqrt(dot(v, v)); }

// Rust f32::signum: +1 for +0 and positives, -1 for -0 and negatives, NaN for NaN.
static inline float signum(float x) {
  if (std::isnan(x)) return x;
  return std::signbit(x) ? -1.0f : 1.0f;
}

// Rust `f as usize` saturating cast (NaN and negatives give 0).
static inline size_t sat_usize(float f) {
  if (!(f > 0.0f)) return 0;
  if (f >= 18446744073709551616.0f) return SIZE_MAX;
  return (size_t)f;
}

static const float F_INF = std::numeric_limits<float>::infinity();

struct Box3 {
  V3 min, max;
};
static inline Box3 box_empty() { return Box3{v3(F_INF, F_INF, F_INF), v3(-F_INF, -F_INF, -F_INF)}; }
static inline void box_expand_point(Box3& b, V3 p) { b.min = vmin(b.min, p); b.max = vmax(b.max, p); }
static inline void box_union(Box3& b, const Box3& o) { b.min = vmin(b.min, o.min); b.max = vmax(b.max, o.max); }
static inline V3 box_center(const Box3& b) { return (b.min + b.max) * 0.5f; }
static inline bool box_is_empty(const Box3& b) {
  return (b.max.x < b.min.x) || (b.max.y < b.min.y) || (b.max.z < b.min.z);
}
// LebesgueMeasurable<T, 2>::measure: 2 * (w*h + w*d + h*d)
static inline float box_surface_area(const Box3& b) {
  float w = b.max.x - b.min.x, h = b.max.y - b.min.y, d = b.max.z - b.min.z;
  return 2.0f * (w * h + w * d + h * d);
}
// 0 = X, 1 = Y, 2 = Z
static inline int box_longest_axis(const Box3& b) {
  float xl = b.max.x - b.min.x, yl = b.max.y - b.min.y, zl = b.max.z - b.min.z;
  if (xl > yl) return xl > zl ? 0 : 2;
  return yl > zl ? 1 : 2;
}
static inline float axis_of(V3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// Mat4 in the reference's field order a1..a4, b1..b4, c1..c4, d1..d4 (column-major).
struct M4 { float m[16]; };
#define A1 m[0]
#define A2 m[1]
#define A3 m[2]
#define A4 m[3]
#define B1 m[4]
#define B2 m[5]
#define B3 m[6]
#define B4 m[7]
#define C1 m[8]
#define C2 m[9]
#define C3 m[10]
#define C4 m[11]
#define D1 m[12]
#define D2 m[13]
#define D3 m[14]
#define D4 m[15]

static inline V4 m4_mul_v4(const M4& M, V4 v) {
  const float* m = M.m;
  return V4{v.x * A1 + v.y * B1 + v.z * C1 + v.w * D1, v.x * A2 + v.y * B2 + v.z * C2 + v.w * D2,
            v.x * A3 + v.y * B3 + v.z * C3 + v.w * D3, v.x * A4 + v.y * B4 + v.z * C4 + v.w * D4};
}
// Mat4 * Vec3 (point): expand with one, divide xyz by w.
static inline V3 m4_mul_point(const M4& M, V3 p) {
  V4 r = m4_mul_v4(M, V4{p.x, p.y, p.z, 1.0f});
  return v3(r.x, r.y, r.z) / r.w;
}
// to_mat3() * Vec3
static inline V3 m3_mul_v3(const M4& M, V3 v) {
  const float* m = M.m;
  return v3(v.x * A1 + v.y * B1 + v.z * C1, v.x * A2 + v.y * B2 + v.z * C2, v.x * A3 + v.y * B3 + v.z * C3);
}
static inline float m3_det(const M4& M) {
  const float* m = M.m;
  float t11 = C3 * B2 - B3 * C2;
  float t12 = B3 * C1 - C3 * B1;
  float t13 = C2 * B1 - B2 * C1;
  return A1 * t11 + A2 * t12 + A3 * t13;
}
static inline float m4_det(const M4& M) {
  const float* m = M.m;
  return A1 * B2 * C3 * D4 - A1 * B2 * C4 * D3 + A1 * B3 * C4 * D2 - A1 * B3 * C2 * D4 +
         A1 * B4 * C2 * D3 - A1 * B4 * C3 * D2
         - A2 * B3 * C4 * D1 + A2 * B3 * C1 * D4 - A2 * B4 * C1 * D3 + A2 * B4 * C3 * D1 -
         A2 * B1 * C3 * D4 + A2 * B1 * C4 * D3
         + A3 * B4 * C1 * D2 - A3 * B4 * C2 * D1 + A3 * B1 * C2 * D4 - A3 * B1 * C4 * D2 +
         A3 * B2 * C4 * D1 - A3 * B2 * C1 * D4
         - A4 * B1 * C2 * D3 + A4 * B1 * C3 * D2 - A4 * B2 * C3 * D1 + A4 * B2 * C1 * D3 -
         A4 * B3 * C1 * D2 + A4 * B3 * C2 * D1;
}
static inline M4 m4_identity() {
  M4 r{};
  r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
  return r;
}
// inverse_or_identity: cofactor expansion, identity when det == 0.
static inline M4 m4_inverse_or_identity(const M4& M) {
  float det = m4_det(M);
  if (det == 0.0f) return m4_identity();
  const float* m = M.m;
  float i = 1.0f / det;
  float n = -i;
  M4 r;
  r.m[0] = i * (B2 * (C3 * D4 - C4 * D3) + B3 * (C4 * D2 - C2 * D4) + B4 * (C2 * D3 - C3 * D2));
  r.m[1] = n * (A2 * (C3 * D4 - C4 * D3) + A3 * (C4 * D2 - C2 * D4) + A4 * (C2 * D3 - C3 * D2));
  r.m[2] = i * (A2 * (B3 * D4 - B4 * D3) + A3 * (B4 * D2 - B2 * D4) + A4 * (B2 * D3 - B3 * D2));
  r.m[3] = n * (A2 * (B3 * C4 - B4 * C3) + A3 * (B4 * C2 - B2 * C4) + A4 * (B2 * C3 - B3 * C2));
  r.m[4] = n * (B1 * (C3 * D4 - C4 * D3) + B3 * (C4 * D1 - C1 * D4) + B4 * (C1 * D3 - C3 * D1));
  r.m[5] = i * (A1 * (C3 * D4 - C4 * D3) + A3 * (C4 * D1 - C1 * D4) + A4 * (C1 * D3 - C3 * D1));
  r.m[6] = n * (A1 * (B3 * D4 - B4 * D3) + A3 * (B4 * D1 - B1 * D4) + A4 * (B1 * D3 - B3 * D1));
  r.m[7] = i * (A1 * (B3 * C4 - B4 * C3) + A3 * (B4 * C1 - B1 * C4) + A4 * (B1 * C3 - B3 * C1));
  r.m[8] = i * (B1 * (C2 * D4 - C4 * D2) + B2 * (C4 * D1 - C1 * D4) + B4 * (C1 * D2 - C2 * D1));
  r.m[9] = n * (A1 * (C2 * D4 - C4 * D2) + A2 * (C4 * D1 - C1 * D4) + A4 * (C1 * D2 - C2 * D1));
  r.m[10] = i * (A1 * (B2 * D4 - B4 * D2) + A2 * (B4 * D1 - B1 * D4) + A4 * (B1 * D2 - B2 * D1));
  r.m[11] = n * (A1 * (B2 * C4 - B4 * C2) + A2 * (B4 * C1 - B1 * C4) + A4 * (B1 * C2 - B2 * C1));
  r.m[12] = n * (B1 * (C2 * D3 - C3 * D2) + B2 * (C3 * D1 - C1 * D3) + B3 * (C1 * D2 - C2 * D1));
  r.m[13] = i * (A1 * (C2 * D3 - C3 * D2) + A2 * (C3 * D1 - C1 * D3) + A3 * (C1 * D2 - C2 * D1));
  r.m[14] = n * (A1 * (B2 * D3 - B3 * D2) + A2 * (B3 * D1 - B1 * D3) + A3 * (B1 * D2 - B2 * D1));
  r.m[15] = i * (A1 * (B2 * C3 - B3 * C2) + A2 * (B3 * C1 - B1 * C3) + A3 * (B1 * C2 - B2 * C1));
  return r;
}
#undef A1
#undef A2
#undef A3
#undef A4
#undef B1
#undef B2
#undef B3
#undef B4
#undef C1
#undef C2
#undef C3
#undef C4
#undef D1
#undef D2
#undef D3
#undef D4

static inline Box3 box_apply_matrix(Box3 b, const M4& M) {
  if (box_is_empty(b)) return b;
  V3 pts[8] = {
      v3(b.min.x, b.min.y, b.min.z), v3(b.min.x, b.min.y, b.max.z), v3(b.min.x, b.max.y, b.min.z),
      v3(b.min.x, b.max.y, b.max.z), v3(b.max.x, b.min.y, b.min.z), v3(b.max.x, b.min.y, b.max.z),
      v3(b.max.x, b.max.y, b.min.z), v3(b.max.x, b.max.y, b.max.z)};
  Box3 r = box_empty();
  for (int k = 0; k < 8; k++) box_expand_point(r, m4_mul_point(M, pts[k]));
  return r;
}

}  // namespace orc
