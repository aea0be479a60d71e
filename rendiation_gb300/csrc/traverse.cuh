// Device-side traversal shared by the batch trace and the wavefront kernels.
//
// Semantics: NaiveSahBvhCpu::traverse (shader/ray-tracing/src/backend/
// wavefront_compute/geometry/naive/traverse_cpu.rs:52-245) — TLAS threaded walk,
// per-instance AABB + mask test, object-space ray with distance scaling, flag
// merging and culling (naive/flag.rs:24-117), BLAS walk, triangle tests
// (geometry/mod.rs:104-155), commit / any-hit / end-search, shared far.
//
// Arithmetic: IEEE f32 exactly as the reference orders it. Every translation
// unit including this header is built with -fmad=false (no contraction of
// a*b+c), IEEE division and square root, and min/max with NaN-ignoring
// fminf/fmaxf (Rust f32::min/max), so every intersection value equals the
// reference CPU's bit for bit.
//
// Traversal orders over the same tree (the reference's SAH build):
//   threaded: the reference's stackless hit/miss walk over its 48 B
//     DeviceBVHNode forest (traverse_cpu.rs:291-319); identical results,
//     including equal-distance ties and which hit ends a first-hit search.
//   ordered (binary / wide4): nearest-child-first traversal over 64 B two-child
//     or 128 B four-child nodes with a per-thread stack in shared memory, and
//     speculative leaf postponement (a lane that reaches a leaf keeps
//     descending until its whole warp holds leaves). Every child box is tested
//     with the reference's slab test; popped entries are re-checked against the
//     current far with the reference's strict `t_near_max < t_max`.
// Both read triangles as 64 B precomputed records (v0, e1, e2, normal, uu, uv,
// vv, 1/(uv^2-uu*vv)) — values the reference recomputes for every test.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "rdn_core.h"
#include "trace_kernels.h"

// Per-thread traversal stack of a kernel: with LOCAL in the thread's local
// memory (kLocalStackEntries entries, L1-cached), else a column of the
// dynamic shared-memory block (stride blockDim.x).
#define RDN_TRAVERSAL_STACK(LOCAL)                                                   \
  extern __shared__ uint2 smem_stack[];                                              \
  uint2 local_stack_[(LOCAL) ? ::rdn::kLocalStackEntries : 1];                       \
  uint2* const stack_ptr = (LOCAL) ? local_stack_ : smem_stack + threadIdx.x;        \
  const uint32_t stack_stride = (LOCAL) ? 1u : blockDim.x

namespace rdn {
namespace dev {

constexpr uint32_t TF_FORCE_OPAQUE = 0x01, TF_FORCE_NON_OPAQUE = 0x02, TF_END_SEARCH = 0x04;
constexpr uint32_t TF_CULL_BACK = 0x10, TF_CULL_FRONT = 0x20, TF_CULL_OPAQUE = 0x40, TF_CULL_NON_OPAQUE = 0x80;
constexpr uint32_t TF_SKIP_TRIANGLES = 0x100, TF_FLIP = 0x400;
constexpr uint32_t ANYHIT_ACCEPT = 1, ANYHIT_END = 2;

__device__ __forceinline__ uint32_t merge_instance_flags(uint32_t f, uint32_t gi) {
  if (gi & 0x1u) f &= ~(TF_CULL_BACK | TF_CULL_FRONT);
  if (gi & 0x2u) f ^= TF_FLIP;
  if (gi & 0x4u) f |= TF_FORCE_OPAQUE;
  if (gi & 0x8u) f |= TF_FORCE_NON_OPAQUE;
  return f;
}

__device__ __forceinline__ float signum_f(float x) {
  if (isnan(x)) return x;
  return signbit(x) ? -1.0f : 1.0f;
}

// intersect_ray_aabb_cpu with the reciprocal direction precomputed (1/d is
// the same IEEE value the reference forms per test). WT (the watertight
// triangle test) multiplies the box's exit distance by kWatertightBoxFarScale,
// so that rounding cannot reject a box the ray touches (Ize, "Robust BVH Ray
// Traversal", JCGT 2(2), 2013: t_far * (1 + 2 gamma_3)); without it a ray
// through a shared vertex or edge on a box face can skip the box that holds
// its triangle. Without WT the test is exactly the reference's.
template <bool WT = false>
__device__ __forceinline__ bool slab(float3 o, float3 inv_d, float tmin, float tmax, float lx, float ly, float lz,
                                     float hx, float hy, float hz, float& t_near_max) {
  const float t0x = (lx - o.x) * inv_d.x, t0y = (ly - o.y) * inv_d.y, t0z = (lz - o.z) * inv_d.z;
  const float t1x = (hx - o.x) * inv_d.x, t1y = (hy - o.y) * inv_d.y, t1z = (hz - o.z) * inv_d.z;
  const float nx = fminf(t0x, t1x), ny = fminf(t0y, t1y), nz = fminf(t0z, t1z);
  const float fx = fmaxf(t0x, t1x), fy = fmaxf(t0y, t1y), fz = fmaxf(t0z, t1z);
  const float tn = fmaxf(fmaxf(nx, ny), nz);
  const float tf = WT ? fminf(fminf(fx, fy), fz) * kWatertightBoxFarScale : fminf(fminf(fx, fy), fz);
  t_near_max = tn;
  return tn <= tf && tmin < tf && tn < tmax;
}

struct TriOut {
  float t, u, v, s;
};

// intersect_ray_triangle_cpu on a precomputed record.
__device__ __forceinline__ bool tri_test(const float4* __restrict__ rec, float3 o, float3 d, float near_, float far_,
                                         bool cull_enable, bool cull_back, TriOut& r) {
  const float4 q0 = __ldg(rec), q1 = __ldg(rec + 1), q2 = __ldg(rec + 2);
  const float b = q0.w * d.x + q1.w * d.y + q2.w * d.z;
  if (cull_enable) {
    const bool pass = cull_back != (b < 0.0f);
    if (!pass) return false;
  }
  const float w0x = o.x - q0.x, w0y = o.y - q0.y, w0z = o.z - q0.z;
  const float a = -(q0.w * w0x + q1.w * w0y + q2.w * w0z);
  const float t = a / b;
  if (t < near_ || t > far_) return false;
  const float4 q3 = __ldg(rec + 3);
  const float px = o.x + t * d.x, py = o.y + t * d.y, pz = o.z + t * d.z;
  const float wx = px - q0.x, wy = py - q0.y, wz = pz - q0.z;
  const float wu = wx * q1.x + wy * q1.y + wz * q1.z;
  const float wv = wx * q2.x + wy * q2.y + wz * q2.z;
  const float uu = q3.x, uv = q3.y, vv = q3.z, inv_d = q3.w;
  const float u = (uv * wv - vv * wu) * inv_d;
  if (u < 0.0f || u > 1.0f) return false;
  const float v = (uv * wu - uu * wv) * inv_d;
  if (v < 0.0f || (u + v) > 1.0f) return false;
  r.t = t;
  r.u = u;
  r.v = v;
  r.s = signum_f(b);
  return true;
}

// ---- watertight triangle test ----------------------------------------------
// Woop, Benthin and Wald, "Watertight Ray/Triangle Intersection", Journal of
// Computer Graphics Techniques 2(1), 2013: the ray is made the +z axis of a
// sheared frame (kz = the largest |d| component, kx and ky the next two,
// swapped when d[kz] < 0 to keep the winding), the triangle's vertices are
// transformed into it and tested with 2D edge functions U, V, W. Two triangles
// sharing an edge evaluate that edge's function on the same two vertices in
// opposite order, and a*b - c*d in f32 is exactly antisymmetric under that
// swap, so a ray can pass between them only if both see exactly 0 (then both
// accept it): no ray leaks through a shared edge. Where a function rounds to 0
// the three are recomputed as exact-sign differences of products (TwoProduct
// by FMA), in place of the paper's double-precision fallback: every step stays
// f32. Differences from the paper's listing: Sx = d[kx] * (1/d[kz]) (the
// reciprocal the slab test already holds), t and the barycentrics from one
// reciprocal of det, and NaN never hits. Facing: det has the opposite sign of
// the reference's b = n.d, so culling and the hit kind follow b's rules.
struct Shear {
  uint32_t kx, ky, kz;
  float sx, sy, sz;
};

__device__ __forceinline__ float pick(float3 v, uint32_t k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// kz = the largest |component| (the lowest axis among equals).
__device__ __forceinline__ Shear make_shear(float3 d, float3 inv_d) {
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  Shear s;
  s.kz = ax >= ay ? (ax >= az ? 0u : 2u) : (ay >= az ? 1u : 2u);
  uint32_t kx = s.kz == 2u ? 0u : s.kz + 1u;
  uint32_t ky = kx == 2u ? 0u : kx + 1u;
  if (pick(d, s.kz) < 0.0f) {
    const uint32_t t = kx;
    kx = ky;
    ky = t;
  }
  s.kx = kx;
  s.ky = ky;
  s.sz = pick(inv_d, s.kz);
  s.sx = pick(d, kx) * s.sz;
  s.sy = pick(d, ky) * s.sz;
  return s;
}

// a*b - c*d with the exact sign: the products' rounding errors by FMA
// (TwoProduct), then (p - q) + (e - f). Antisymmetric like the plain form.
__device__ __forceinline__ float diff_products(float a, float b, float c, float d) {
  const float p = a * b, q = c * d;
  const float e = __fmaf_rn(a, b, -p), f = __fmaf_rn(c, d, -q);
  return (p - q) + (e - f);
}

__device__ __forceinline__ bool tri_test_watertight(const float4* __restrict__ rec, float3 o, const Shear& sh,
                                                    float near_, float far_, bool cull_enable, bool cull_back,
                                                    TriOut& r) {
  const float4 q0 = __ldg(rec), q1 = __ldg(rec + 1), q2 = __ldg(rec + 2);
  const float3 A = make_float3(q0.x - o.x, q0.y - o.y, q0.z - o.z);
  const float3 B = make_float3(q0.w - o.x, q1.x - o.y, q1.y - o.z);
  const float3 C = make_float3(q1.z - o.x, q1.w - o.y, q2.x - o.z);
  const float akz = pick(A, sh.kz), bkz = pick(B, sh.kz), ckz = pick(C, sh.kz);
  const float ax = pick(A, sh.kx) - sh.sx * akz, ay = pick(A, sh.ky) - sh.sy * akz;
  const float bx = pick(B, sh.kx) - sh.sx * bkz, by = pick(B, sh.ky) - sh.sy * bkz;
  const float cx = pick(C, sh.kx) - sh.sx * ckz, cy = pick(C, sh.ky) - sh.sy * ckz;
  float U = cx * by - cy * bx, V = ax * cy - ay * cx, W = bx * ay - by * ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = diff_products(cx, by, cy, bx);
    V = diff_products(ax, cy, ay, cx);
    W = diff_products(bx, ay, by, ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  const float det = (U + V) + W;
  if (!(fabsf(det) > 0.0f)) return false;
  if (cull_enable) {
    const bool pass = cull_back != (det > 0.0f);  // det > 0 <=> the reference's b < 0
    if (!pass) return false;
  }
  const float T = (U * (sh.sz * akz) + V * (sh.sz * bkz)) + W * (sh.sz * ckz);
  const float rcp = 1.0f / det;
  const float t = T * rcp;
  if (!(t >= near_ && t <= far_)) return false;
  r.t = t;
  r.u = V * rcp;
  r.v = W * rcp;
  r.s = det > 0.0f ? -1.0f : 1.0f;
  return true;
}

struct Best {
  float t, u, v, s;
  uint32_t k, geom_slot, inst;
  bool have;
};

struct InstanceRay {
  float3 o, d, inv_d;
  float scaling;
  uint32_t flags;
};

// Object-space ray: transform_inv * (o, 1) / w, to_mat3() * d, scaling = |d'|,
// d' normalised (traverse_cpu.rs:99-104).
__device__ __forceinline__ InstanceRay to_instance(const DeviceInstance* __restrict__ inst, float3 o, float3 d,
                                                   uint32_t ray_flags) {
  const float* m = inst->transform_inv;
  const float x = o.x * __ldg(m + 0) + o.y * __ldg(m + 4) + o.z * __ldg(m + 8) + 1.0f * __ldg(m + 12);
  const float y = o.x * __ldg(m + 1) + o.y * __ldg(m + 5) + o.z * __ldg(m + 9) + 1.0f * __ldg(m + 13);
  const float z = o.x * __ldg(m + 2) + o.y * __ldg(m + 6) + o.z * __ldg(m + 10) + 1.0f * __ldg(m + 14);
  const float w = o.x * __ldg(m + 3) + o.y * __ldg(m + 7) + o.z * __ldg(m + 11) + 1.0f * __ldg(m + 15);
  InstanceRay r;
  r.o = make_float3(x / w, y / w, z / w);
  float dx = d.x * __ldg(m + 0) + d.y * __ldg(m + 4) + d.z * __ldg(m + 8);
  float dy = d.x * __ldg(m + 1) + d.y * __ldg(m + 5) + d.z * __ldg(m + 9);
  float dz = d.x * __ldg(m + 2) + d.y * __ldg(m + 6) + d.z * __ldg(m + 10);
  const float mag_sq = dx * dx + dy * dy + dz * dz;
  r.scaling = sqrtf(mag_sq);
  if (mag_sq > 0.0f) {
    const float inv = 1.0f / sqrtf(mag_sq);
    dx = dx * inv;
    dy = dy * inv;
    dz = dz * inv;
  }
  r.d = make_float3(dx, dy, dz);
  r.inv_d = make_float3(1.0f / dx, 1.0f / dy, 1.0f / dz);
  r.flags = merge_instance_flags(ray_flags, __ldg(&inst->flags));
  return r;
}

__device__ __forceinline__ void geometry_cull(uint32_t f, uint32_t gf, bool& pass, bool& is_opaque, bool& cull_enable,
                                              bool& cull_back) {
  const bool geometry_opaque = (gf & 1u) != 0;
  const bool op = (geometry_opaque || (f & TF_FORCE_OPAQUE)) && !(f & TF_FORCE_NON_OPAQUE);
  pass = (op && !(f & TF_CULL_OPAQUE)) || (!op && !(f & TF_CULL_NON_OPAQUE));
  is_opaque = op;
  const bool flip = (f & TF_FLIP) != 0, cf = (f & TF_CULL_FRONT) != 0, cb = (f & TF_CULL_BACK) != 0;
  cull_enable = cf || cb;
  cull_back = (flip && cb) || (!flip && cf);
}

// Policies in place of a user any-hit shader: 0 accept, 1 accept and end the
// search, 2 accept even primitive ids, 3 accept when bit `tri` (built
// triangle index) of the mask is set.
__device__ __forceinline__ uint32_t anyhit_policy(uint32_t mode, uint32_t primitive_idx, uint32_t tri,
                                                  const uint32_t* __restrict__ mask) {
  if (mode == 1) return ANYHIT_ACCEPT | ANYHIT_END;
  if (mode == 2) return (primitive_idx & 1u) ? 0u : ANYHIT_ACCEPT;
  if (mode == 3) return (__ldg(mask + (tri >> 5)) >> (tri & 31u)) & 1u ? ANYHIT_ACCEPT : 0u;
  return ANYHIT_ACCEPT;
}

// A candidate hit on non-opaque geometry, as an any-hit program sees it.
struct AnyHitInfo {
  uint32_t primitive;  // index within its geometry
  uint32_t triangle;   // built triangle index
  uint32_t instance;   // TLAS instance slot
  uint32_t geometry;   // geometry slot
  float t, u, v;       // world distance, barycentrics of vertices 1 and 2
  bool front_facing;
};

// The fixed policies of anyhit_policy; traversals take any functor with the
// same call (behaviour bits ANYHIT_ACCEPT / ANYHIT_END) in its place.
struct BuiltinAnyHit {
  __device__ __forceinline__ uint32_t operator()(const TraceParams& p, const AnyHitInfo& h) const {
    return anyhit_policy(p.anyhit_mode, h.primitive, h.triangle, p.anyhit_mask);
  }
};

struct RayCtx {
  float3 o, d, inv_d;
  float tmin, tmax;
  float far_world;  // the shared far of RayRange
  uint32_t cull_mask, ray_flags;
  Best best;
  uint32_t node_visits, tri_tests, tri_hits;
  bool end_search;
};

// Tests the triangles of sorted range [k0, k1) and commits hits; returns true
// when the search must end. Follows traverse_cpu.rs:133-193.
template <bool COUNT, class AH = BuiltinAnyHit, bool WT = false>
__device__ __forceinline__ bool leaf_triangles(const TraceParams& p, RayCtx& R, const InstanceRay& ir, uint32_t k0,
                                               uint32_t k1, uint32_t gslot, uint32_t inst_slot, bool is_opaque,
                                               bool cull_enable, bool cull_back, uint32_t prim_start,
                                               const AH& anyhit = AH()) {
  Shear sh;
  if (WT) sh = make_shear(ir.d, ir.inv_d);
  for (uint32_t k = k0; k < k1; k++) {
    if (COUNT) R.tri_tests++;
    TriOut h;
    const float near_ = R.tmin * ir.scaling, far_ = R.far_world * ir.scaling;
    if (WT) {
      if (!tri_test_watertight(p.verts + 3 * (size_t)k, ir.o, sh, near_, far_, cull_enable, cull_back, h)) continue;
    } else if (!tri_test(p.tris + 4 * (size_t)k, ir.o, ir.d, near_, far_, cull_enable, cull_back, h)) {
      continue;
    }
    if (COUNT) R.tri_hits++;
    const float distance = h.t / ir.scaling;
    uint32_t behavior = ANYHIT_ACCEPT;
    if (!is_opaque) {
      const uint32_t tri = __ldg(p.redirect + k);
      behavior = anyhit(p, AnyHitInfo{tri - prim_start, tri, inst_slot, gslot, distance, h.u, h.v, !(h.s < 0.0f)});
    }
    if (behavior & ANYHIT_ACCEPT) {
      R.far_world = distance;
      R.best.t = distance;
      R.best.u = h.u;
      R.best.v = h.v;
      R.best.s = h.s;
      R.best.k = k;
      R.best.geom_slot = gslot;
      R.best.inst = inst_slot;
      R.best.have = true;
      if (ir.flags & TF_END_SEARCH) behavior |= ANYHIT_END;
    }
    if (behavior & ANYHIT_END) return true;
  }
  return false;
}

// BLAS of one geometry, reference threaded order (traverse_cpu.rs:122-195).
template <bool COUNT, class AH = BuiltinAnyHit, bool WT = false>
__device__ __forceinline__ bool blas_threaded(const TraceParams& p, RayCtx& R, const InstanceRay& ir, uint32_t root,
                                              uint32_t gslot, uint32_t inst_slot, bool is_opaque, bool cull_enable,
                                              bool cull_back, uint32_t prim_start, const AH& anyhit = AH()) {
  uint32_t curr = root;
  while (curr != INVALID_NEXT) {
    if (COUNT) R.node_visits++;
    const float4* nd = reinterpret_cast<const float4*>(p.tri_forest + curr);
    const float4 a = __ldg(nd), b = __ldg(nd + 1);
    float tn;
    const uint32_t hit_next = __float_as_uint(a.w), miss_next = __float_as_uint(b.w);
    if (slab<WT>(ir.o, ir.inv_d, R.tmin * ir.scaling, R.far_world * ir.scaling, a.x, a.y, a.z, b.x, b.y, b.z, tn)) {
      curr = hit_next;
      if (hit_next == miss_next) {  // a leaf: hit and miss links are the same node
        const uint2 cr = __ldg(reinterpret_cast<const uint2*>(nd + 2));
        if (leaf_triangles<COUNT, AH, WT>(p, R, ir, cr.x, cr.y, gslot, inst_slot, is_opaque, cull_enable,
                                          cull_back, prim_start, anyhit))
          return true;
      }
    } else {
      curr = miss_next;
    }
  }
  return false;
}

__device__ __forceinline__ void cswap(float& ta, uint32_t& ca, float& tb, uint32_t& cb) {
  if (tb < ta) {
    const float t = ta;
    ta = tb;
    tb = t;
    const uint32_t c = ca;
    ca = cb;
    cb = c;
  }
}

// Pops the next pending child whose box still passes `t_near_max < t_max`
// against the current far; EMPTY_SLOT when the stack is exhausted.
__device__ __forceinline__ uint32_t pop_live(const uint2* stack, uint32_t stride, uint32_t& sp, float far_,
                                             float& code_tn) {
  while (sp) {
    sp--;
    const uint2 e = stack[sp * stride];
    if (__uint_as_float(e.y) < far_) {
      code_tn = __uint_as_float(e.y);
      return e.x;
    }
  }
  return EMPTY_SLOT;
}

__device__ __forceinline__ void push_entry(const TraceParams& p, uint2* stack, uint32_t stride, uint32_t& sp,
                                           uint32_t depth, uint32_t code, float tn) {
  if (sp < depth) stack[(sp++) * stride] = make_uint2(code, __float_as_uint(tn));
  else atomicOr(p.error_word, 1u);  // the stack is sized from the tree depth: unreachable
}

// One interior-node step of the ordered walk: tests the children of node
// `code`, pushes the farther hits and returns the nearest hit child (or the
// next live stack entry when no child is hit).
template <bool COUNT, int WIDTH, bool WT = false>
__device__ __forceinline__ uint32_t interior_step(const TraceParams& p, RayCtx& R, const InstanceRay& ir, uint32_t code,
                                                  float& code_tn, uint2* stack, uint32_t stride, uint32_t& sp,
                                                  uint32_t depth) {
  const float near_ = R.tmin * ir.scaling, far_ = R.far_world * ir.scaling;
  if (WIDTH == 2) {
    const float4* w = p.wide + 4 * (size_t)code;
    const float4 w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2);
    const uint2 cc = __ldg(reinterpret_cast<const uint2*>(w + 3));
    if (COUNT) R.node_visits += 2;
    float tn0, tn1;
    const bool h0 = slab<WT>(ir.o, ir.inv_d, near_, far_, w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, tn0);
    const bool h1 = slab<WT>(ir.o, ir.inv_d, near_, far_, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w, tn1);
    if (h0 && h1) {
      const bool second_first = tn1 < tn0;
      push_entry(p, stack, stride, sp, depth, second_first ? cc.x : cc.y, second_first ? tn0 : tn1);
      code_tn = second_first ? tn1 : tn0;
      return second_first ? cc.y : cc.x;
    }
    if (h0 || h1) {
      code_tn = h0 ? tn0 : tn1;
      return h0 ? cc.x : cc.y;
    }
    return pop_live(stack, stride, sp, far_, code_tn);
  } else {
    const float4* w = p.wide4 + 8 * (size_t)code;
    const float4 lx = __ldg(w), ly = __ldg(w + 1), lz = __ldg(w + 2);
    const float4 hx = __ldg(w + 3), hy = __ldg(w + 4), hz = __ldg(w + 5);
    const uint4 cc = __ldg(reinterpret_cast<const uint4*>(w + 6));
    const float inf = __int_as_float(0x7f800000);
    float t0 = inf, t1 = inf, t2 = inf, t3 = inf;
    uint32_t c0 = EMPTY_SLOT, c1 = EMPTY_SLOT, c2 = EMPTY_SLOT, c3 = EMPTY_SLOT;
    float tn;
    if (cc.x != EMPTY_SLOT && slab<WT>(ir.o, ir.inv_d, near_, far_, lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, tn)) {
      t0 = tn;
      c0 = cc.x;
    }
    if (cc.y != EMPTY_SLOT && slab<WT>(ir.o, ir.inv_d, near_, far_, lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, tn)) {
      t1 = tn;
      c1 = cc.y;
    }
    if (cc.z != EMPTY_SLOT && slab<WT>(ir.o, ir.inv_d, near_, far_, lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, tn)) {
      t2 = tn;
      c2 = cc.z;
    }
    if (cc.w != EMPTY_SLOT && slab<WT>(ir.o, ir.inv_d, near_, far_, lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, tn)) {
      t3 = tn;
      c3 = cc.w;
    }
    if (COUNT) R.node_visits += (cc.x != EMPTY_SLOT) + (cc.y != EMPTY_SLOT) + (cc.z != EMPTY_SLOT) + (cc.w != EMPTY_SLOT);
    cswap(t0, c0, t1, c1);
    cswap(t2, c2, t3, c3);
    cswap(t0, c0, t2, c2);
    cswap(t1, c1, t3, c3);
    cswap(t1, c1, t2, c2);
    if (c0 == EMPTY_SLOT) return pop_live(stack, stride, sp, far_, code_tn);
    if (c3 != EMPTY_SLOT) push_entry(p, stack, stride, sp, depth, c3, t3);
    if (c2 != EMPTY_SLOT) push_entry(p, stack, stride, sp, depth, c2, t2);
    if (c1 != EMPTY_SLOT) push_entry(p, stack, stride, sp, depth, c1, t1);
    code_tn = t0;
    return c0;
  }
}

// Ordered BLAS walk with speculative traversal: a lane that reaches a leaf
// postpones it and keeps descending until every active lane of the warp holds
// a leaf (or has finished), then the warp tests triangles together. Nodes are
// visited in near-first order with the reference's box test; the speculation
// only adds visits, never removes one, so the closest hit is unchanged.
template <bool COUNT, int WIDTH, class AH = BuiltinAnyHit, bool WT = false>
__device__ __forceinline__ bool blas_speculative(const TraceParams& p, RayCtx& R, const InstanceRay& ir,
                                                 uint32_t root_node, uint32_t gslot, uint32_t inst_slot,
                                                 bool is_opaque, bool cull_enable, bool cull_back, uint32_t prim_start,
                                                 uint2* stack, uint32_t stride, uint32_t depth,
                                                 const AH& anyhit = AH()) {
  {
    if (COUNT) R.node_visits++;
    const float4* nd = reinterpret_cast<const float4*>(p.tri_forest + root_node);
    const float4 a = __ldg(nd), b = __ldg(nd + 1);
    float tn;
    if (!slab<WT>(ir.o, ir.inv_d, R.tmin * ir.scaling, R.far_world * ir.scaling, a.x, a.y, a.z, b.x, b.y, b.z, tn))
      return false;
  }
  uint32_t code = __ldg((WIDTH == 2 ? p.geom_root_code : p.geom_root_code4) + gslot);
  float code_tn = -__int_as_float(0x7f800000);
  uint32_t leaf = EMPTY_SLOT;
  uint32_t sp = 0;
  if (code & LEAF_BIT) {
    leaf = code;
    code = EMPTY_SLOT;
  }
  while (code != EMPTY_SLOT || leaf != EMPTY_SLOT) {
    while (code != EMPTY_SLOT && !(code & LEAF_BIT)) {
      code = interior_step<COUNT, WIDTH, WT>(p, R, ir, code, code_tn, stack, stride, sp, depth);
      if (code != EMPTY_SLOT && (code & LEAF_BIT) && leaf == EMPTY_SLOT) {
        leaf = code;
        code = pop_live(stack, stride, sp, R.far_world * ir.scaling, code_tn);
      }
      // keep descending while more than spec_threshold lanes still look for a leaf
      if ((uint32_t)__popc(__ballot_sync(__activemask(), leaf == EMPTY_SLOT)) <= p.spec_threshold) break;
    }
    while (leaf != EMPTY_SLOT) {
      const uint2 lr = __ldg(p.leaves + (leaf & ~LEAF_BIT));
      if (leaf_triangles<COUNT, AH, WT>(p, R, ir, lr.x, lr.y, gslot, inst_slot, is_opaque, cull_enable, cull_back,
                                        prim_start, anyhit))
        return true;
      leaf = EMPTY_SLOT;
      // the far may have shrunk: re-check the pending node before descending into it
      if (code != EMPTY_SLOT && !(code_tn < R.far_world * ir.scaling))
        code = pop_live(stack, stride, sp, R.far_world * ir.scaling, code_tn);
      if (code != EMPTY_SLOT && (code & LEAF_BIT)) {
        leaf = code;
        code = pop_live(stack, stride, sp, R.far_world * ir.scaling, code_tn);
      }
    }
  }
  return false;
}

// Full query of one ray (traverse_cpu.rs:52-245). R must hold the ray; on
// return R.best holds the committed hit. `bad` reports an unbound TLAS index.
template <int MODE, bool COUNT, class AH = BuiltinAnyHit, bool WT = false>
__device__ __forceinline__ void traverse_ray(const TraceParams& p, RayCtx& R, uint32_t tidx, uint2* stack,
                                             uint32_t stride, bool& bad, const AH& anyhit = AH()) {
  R.inv_d = make_float3(1.0f / R.d.x, 1.0f / R.d.y, 1.0f / R.d.z);
  R.far_world = R.tmax;
  R.best.have = false;
  R.node_visits = R.tri_tests = R.tri_hits = 0;
  bad = false;
  uint32_t curr = INVALID_NEXT;
  if (tidx >= p.n_binding) {
    bad = true;
  } else {
    const uint32_t handle = __ldg(p.tlas_binding + tidx);
    if (handle >= p.n_tlas_root) bad = true;
    else curr = __ldg(p.tlas_bvh_root + handle);
  }
  bool done = false;
  // TLAS: threaded walk with the shared far (scaling 1)
  while (curr != INVALID_NEXT && !done) {
    if (COUNT) R.node_visits++;
    const float4* nd = reinterpret_cast<const float4*>(p.tlas_forest + curr);
    const float4 a = __ldg(nd), b = __ldg(nd + 1);
    const uint32_t hit_next = __float_as_uint(a.w), miss_next = __float_as_uint(b.w);
    float tn;
    if (!slab<WT>(R.o, R.inv_d, R.tmin * 1.0f, R.far_world * 1.0f, a.x, a.y, a.z, b.x, b.y, b.z, tn)) {
      curr = miss_next;
      continue;
    }
    curr = hit_next;
    if (hit_next != miss_next) continue;
    const uint2 cr = __ldg(reinterpret_cast<const uint2*>(nd + 2));
    for (uint32_t ti = cr.x; ti < cr.y && !done; ti++) {
      const float4* tb = reinterpret_cast<const float4*>(p.tlas_bounding + ti);
      const float4 ba = __ldg(tb), bb = __ldg(tb + 1);
      float tn2;
      if (!slab<WT>(R.o, R.inv_d, R.tmin, R.tmax, ba.x, ba.y, ba.z, bb.x, bb.y, bb.z, tn2)) continue;
      if ((R.cull_mask & __float_as_uint(ba.w)) == 0) continue;
      const DeviceInstance* inst = p.tlas_data + ti;
      const InstanceRay ir = to_instance(inst, R.o, R.d, R.ray_flags);
      if (ir.flags & TF_SKIP_TRIANGLES) continue;
      const uint32_t blas = __ldg(&inst->acceleration_structure_handle);
      const uint2 range = __ldg(reinterpret_cast<const uint2*>(p.blas_meta + blas));
      for (uint32_t g = range.x; g < range.y; g++) {
        const uint4 gm = __ldg(reinterpret_cast<const uint4*>(p.tri_root + g));
        bool pass, is_opaque, cull_enable, cull_back;
        geometry_cull(ir.flags, gm.w, pass, is_opaque, cull_enable, cull_back);
        if (!pass) continue;
        bool end;
        if (MODE == MODE_WIDE4)
          end = blas_speculative<COUNT, 4, AH, WT>(p, R, ir, gm.x, g, ti, is_opaque, cull_enable, cull_back, gm.z, stack,
                                               stride, p.stack_depth, anyhit);
        else if (MODE == MODE_BINARY)
          end = blas_speculative<COUNT, 2, AH, WT>(p, R, ir, gm.x, g, ti, is_opaque, cull_enable, cull_back, gm.z, stack,
                                               stride, p.stack_depth, anyhit);
        else
          end = blas_threaded<COUNT, AH, WT>(p, R, ir, gm.x, g, ti, is_opaque, cull_enable, cull_back, gm.z, anyhit);
        if (end) {
          done = true;
          break;
        }
      }
    }
  }
}

// Resumable per-lane query for dynamic-fetch schedules: the same TLAS walk,
// instance and geometry loops and speculative ordered BLAS walk as
// traverse_ray (WIDTH 2 or 4), with the state kept across calls so that a warp
// can stop, hand new rays to its idle lanes, and continue.
enum : uint32_t { WALK_IDLE = 0, WALK_TLAS = 1, WALK_INST = 2, WALK_GEOM = 3, WALK_BLAS = 4, WALK_DONE = 5 };
constexpr uint32_t kMaxWalkRounds = 1u << 24;
__device__ __forceinline__ uint32_t walk_round_cap(const TraceParams& p) {
  return p.iteration_limit ? p.iteration_limit : kMaxWalkRounds;
}

template <int WIDTH, bool WT = false>
struct LaneWalk {
  RayCtx R;
  InstanceRay ir;
  uint32_t phase, tcur, ti, ti_end, inst_slot, g, g_end, gslot, prim_start;
  bool is_opaque, cull_enable, cull_back;
  uint32_t code, leaf, sp;
  float code_tn;

  __device__ __forceinline__ void reset() {
    phase = WALK_IDLE;
    R.cull_mask = 0xFFu;
    R.best.have = false;
    ir.o = ir.d = ir.inv_d = make_float3(0.f, 0.f, 0.f);
    ir.scaling = 1.0f;
    ir.flags = 0u;
    tcur = INVALID_NEXT;
    ti = ti_end = inst_slot = g = g_end = gslot = prim_start = 0;
    is_opaque = true;
    cull_enable = cull_back = false;
    code = leaf = EMPTY_SLOT;
    sp = 0;
    code_tn = 0.0f;
  }

  __device__ __forceinline__ void start(const TraceParams& p, float4 r0, float4 r1, uint32_t tlas, uint32_t ray_flags) {
    R.o = make_float3(r0.x, r0.y, r0.z);
    R.tmin = r0.w;
    R.d = make_float3(r1.x, r1.y, r1.z);
    R.tmax = r1.w;
    R.ray_flags = ray_flags;
    R.cull_mask = 0xFFu;
    R.inv_d = make_float3(1.0f / R.d.x, 1.0f / R.d.y, 1.0f / R.d.z);
    R.far_world = R.tmax;
    R.best.have = false;
    tcur = INVALID_NEXT;
    if (tlas < p.n_binding) {
      const uint32_t handle = __ldg(p.tlas_binding + tlas);
      if (handle < p.n_tlas_root) tcur = __ldg(p.tlas_bvh_root + handle);
    }
    code = leaf = EMPTY_SLOT;
    phase = WALK_TLAS;
  }

  // TLAS / instance / geometry steps up to the next BLAS entry or the end.
  __device__ __forceinline__ void to_blas(const TraceParams& p) {
    const float inf = __int_as_float(0x7f800000);
    while (phase == WALK_TLAS || phase == WALK_INST || phase == WALK_GEOM) {
      if (phase == WALK_TLAS) {
        bool found = false;
        while (tcur != INVALID_NEXT) {
          const float4* nd = reinterpret_cast<const float4*>(p.tlas_forest + tcur);
          const float4 a = __ldg(nd), b = __ldg(nd + 1);
          const uint32_t hit_next = __float_as_uint(a.w), miss_next = __float_as_uint(b.w);
          float tn;
          if (!slab<WT>(R.o, R.inv_d, R.tmin * 1.0f, R.far_world * 1.0f, a.x, a.y, a.z, b.x, b.y, b.z, tn)) {
            tcur = miss_next;
            continue;
          }
          tcur = hit_next;
          if (hit_next != miss_next) continue;
          const uint2 cr = __ldg(reinterpret_cast<const uint2*>(nd + 2));
          ti = cr.x;
          ti_end = cr.y;
          found = true;
          break;
        }
        phase = found ? WALK_INST : WALK_DONE;
      } else if (phase == WALK_INST) {
        bool entered = false;
        while (ti < ti_end) {
          const uint32_t cur = ti++;
          const float4* tb = reinterpret_cast<const float4*>(p.tlas_bounding + cur);
          const float4 ba = __ldg(tb), bb = __ldg(tb + 1);
          float tn2;
          if (!slab<WT>(R.o, R.inv_d, R.tmin, R.tmax, ba.x, ba.y, ba.z, bb.x, bb.y, bb.z, tn2)) continue;
          if ((R.cull_mask & __float_as_uint(ba.w)) == 0) continue;
          const DeviceInstance* inst = p.tlas_data + cur;
          ir = to_instance(inst, R.o, R.d, R.ray_flags);
          if (ir.flags & TF_SKIP_TRIANGLES) continue;
          const uint32_t blas = __ldg(&inst->acceleration_structure_handle);
          const uint2 range = __ldg(reinterpret_cast<const uint2*>(p.blas_meta + blas));
          g = range.x;
          g_end = range.y;
          inst_slot = cur;
          entered = true;
          break;
        }
        phase = entered ? WALK_GEOM : WALK_TLAS;
      } else {
        bool entered = false;
        while (g < g_end) {
          const uint32_t cur = g++;
          const uint4 gm = __ldg(reinterpret_cast<const uint4*>(p.tri_root + cur));
          bool pass;
          geometry_cull(ir.flags, gm.w, pass, is_opaque, cull_enable, cull_back);
          if (!pass) continue;
          const float4* nd = reinterpret_cast<const float4*>(p.tri_forest + gm.x);
          const float4 a = __ldg(nd), b = __ldg(nd + 1);
          float tn;
          if (!slab<WT>(ir.o, ir.inv_d, R.tmin * ir.scaling, R.far_world * ir.scaling, a.x, a.y, a.z, b.x, b.y, b.z, tn))
            continue;
          code = __ldg((WIDTH == 2 ? p.geom_root_code : p.geom_root_code4) + cur);
          code_tn = -inf;
          leaf = EMPTY_SLOT;
          sp = 0;
          if (code & LEAF_BIT) {
            leaf = code;
            code = EMPTY_SLOT;
          }
          gslot = cur;
          prim_start = gm.z;
          entered = true;
          break;
        }
        phase = entered ? WALK_BLAS : WALK_INST;
      }
    }
  }

  // Advances the query: to the next BLAS entry, then rounds of traverse_ray's
  // speculative walk. Returns with phase WALK_DONE when the query ended, with
  // WALK_GEOM when this BLAS is exhausted, or still WALK_BLAS after a round in
  // which at least `threshold` lanes of the warp were outside the walk (the
  // caller then refills its idle lanes).
  __device__ __forceinline__ void advance(const TraceParams& p, uint2* stack, uint32_t stride, uint32_t threshold) {
    to_blas(p);
    if (phase != WALK_BLAS) return;
    for (uint32_t round = 0;; round++) {
      if (round >= walk_round_cap(p)) {
        atomicOr(p.error_word, 4u);
        phase = WALK_DONE;
        return;
      }
      while (code != EMPTY_SLOT && !(code & LEAF_BIT)) {
        code = interior_step<false, WIDTH, WT>(p, R, ir, code, code_tn, stack, stride, sp, p.stack_depth);
        if (code != EMPTY_SLOT && (code & LEAF_BIT) && leaf == EMPTY_SLOT) {
          leaf = code;
          code = pop_live(stack, stride, sp, R.far_world * ir.scaling, code_tn);
        }
        if ((uint32_t)__popc(__ballot_sync(__activemask(), leaf == EMPTY_SLOT)) <= p.spec_threshold) break;
      }
      while (leaf != EMPTY_SLOT) {
        const uint2 lr = __ldg(p.leaves + (leaf & ~LEAF_BIT));
        if (leaf_triangles<false, BuiltinAnyHit, WT>(p, R, ir, lr.x, lr.y, gslot, inst_slot, is_opaque, cull_enable, cull_back,
                                  prim_start)) {
          code = leaf = EMPTY_SLOT;
          phase = WALK_DONE;  // the search ends (first hit accepted)
          return;
        }
        leaf = EMPTY_SLOT;
        // the far may have shrunk: re-check the pending node before descending into it
        if (code != EMPTY_SLOT && !(code_tn < R.far_world * ir.scaling))
          code = pop_live(stack, stride, sp, R.far_world * ir.scaling, code_tn);
        if (code != EMPTY_SLOT && (code & LEAF_BIT)) {
          leaf = code;
          code = pop_live(stack, stride, sp, R.far_world * ir.scaling, code_tn);
        }
      }
      if (code == EMPTY_SLOT && leaf == EMPTY_SLOT) {
        phase = WALK_GEOM;  // next geometry / instance on the next call
        return;
      }
      if (32u - (uint32_t)__popc(__activemask()) >= threshold) return;  // let the warp refill
    }
  }
};

}  // namespace dev
}  // namespace rdn
