// Differentiable closest hit: attribute-interpolation loss and its adjoint at
// frozen visibility, sm_103a.
//
// Forward (attr_forward_kernel): per ray, closest hit (the traversal of
// traverse.cuh), value = (1-u-v)*a[i0] + u*a[i1] + v*a[i2] with the hit
// triangle's vertex attributes, loss = (value - target)^2; a miss contributes
// nothing. The per-ray value and loss are written; the loss sum is accumulated
// per block and added once per block.
//
// Adjoint (attr_adjoint_kernel): the hit is recomputed by tracing the ray again
// instead of being stored by the forward pass. With r = 2 (value - target) * g
// (g = upstream gradient of the loss sum):
//   dL/da_k = r * w_k                       (w = (1-u-v, u, v))
//   gu = r (a1 - a0), gv = r (a2 - a0), gt = 0
// The hit solves o + t d = v0 + u e1 + v e2, i.e. M (t,u,v)^T = o - v0 with
// M = [-d | e1 | e2]. Differentiating at fixed visibility gives, with
// lambda = M^{-T} (gt, gu, gv):
//   dL/do = lambda, dL/dd = t lambda,
//   dL/dv0 = -(1-u-v) lambda, dL/dv1 = -u lambda, dL/dv2 = -v lambda,
// lambda = (gt (e1 x e2) + gu (e2 x -d) + gv (-d x e1)) / ((-d) . (e1 x e2)).
// Vertex gradients are accumulated as float4 (dx, dy, dz, dattr) per vertex
// with one vector atomicAdd per triangle corner. All quantities are in the
// instance's object space (world space for identity instances).
//
// Barycentrics of the loss: the traversal finds the hit with the reference's
// f32 triangle test, whose projected barycentrics lose accuracy for rays that
// graze the triangle (relative error ~ 1e-7 / cos). Both kernels therefore
// re-solve (u, v) on the hit triangle with Cramer's rule in float-float
// arithmetic (error-free TwoSum / TwoProduct built on f32 FMA), which keeps the
// loss and its gradient accurate to ~1e-6 for rays down to a few degrees of
// grazing, with f32 arithmetic only.
#include <cuda_runtime.h>

#include <cstdint>

#include "adjoint.h"
#include "shade.cuh"
#include "traverse.cuh"

namespace rdn {
namespace {

using namespace dev;

// float-float value hi + lo
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return ff{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = a * b;
  return ff{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  const float lo = s.lo + (a.lo + b.lo);
  return two_sum(s.hi, lo);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  const float lo = p.lo + (a.hi * b.lo + a.lo * b.hi);
  return two_sum(p.hi, lo);
}
struct ff3 {
  ff x, y, z;
};
__device__ __forceinline__ ff3 ff3_sub(float3 a, float3 b) {
  return ff3{two_sum(a.x, -b.x), two_sum(a.y, -b.y), two_sum(a.z, -b.z)};
}
__device__ __forceinline__ ff3 ff3_of(float3 a) { return ff3{{a.x, 0.f}, {a.y, 0.f}, {a.z, 0.f}}; }
__device__ __forceinline__ ff3 ff3_cross(ff3 a, ff3 b) {
  return ff3{ff_add(ff_mul(a.y, b.z), ff_neg(ff_mul(a.z, b.y))),
             ff_add(ff_mul(a.z, b.x), ff_neg(ff_mul(a.x, b.z))),
             ff_add(ff_mul(a.x, b.y), ff_neg(ff_mul(a.y, b.x)))};
}
__device__ __forceinline__ ff ff3_dot(ff3 a, ff3 b) {
  return ff_add(ff_add(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_mul(a.z, b.z));
}
__device__ __forceinline__ float ff_div(ff a, ff b) { return (a.hi + a.lo) / (b.hi + b.lo); }
// a / b as a float-float value: a first quotient, its remainder formed in
// float-float, and a correction quotient.
__device__ __forceinline__ ff ff_div_ff(ff a, ff b) {
  const float q1 = a.hi / b.hi;
  const ff rem = ff_add(a, ff_neg(ff_mul(ff{q1, 0.f}, b)));
  const float q2 = (rem.hi + rem.lo) / b.hi;
  return two_sum(q1, q2);
}

struct HitGeom {
  uint32_t i0, i1, i2;
  float w0, u, v;
  ff3 b1, b2;  // e2 x (-d) and (-d) x e1 in float-float (the adjoint's lambda)
  ff3 c12;     // e1 x e2 (lambda's distance row)
  ff det;      // (-d) . (e1 x e2)
  float t_unnorm;  // hit distance in units of the unnormalised object-space direction
  ff wf, uf, vf;   // the three corner weights in float-float (w0, u, v round these)
};

// Hit triangle's vertices and barycentrics re-solved in float-float: with
// M = [-d | e1 | e2] and s = o - v0, u = det[-d, s, e2] / det M and
// v = det[-d, e1, s] / det M (Cramer), e1, e2, s formed exactly. Cramer's rule
// does not depend on the length of d, so d is the object-space direction before
// normalisation (exact for an identity instance). `tri` is the built triangle
// index, `inst` the TLAS instance slot of the hit, d_world the ray direction.
__device__ __forceinline__ HitGeom hit_vertices_at(const TraceParams& p, const uint32_t* __restrict__ indices,
                                                   const float* __restrict__ vertices, uint32_t tri, uint32_t inst,
                                                   float3 d_world, const InstanceRay& ir) {
  HitGeom h;
  h.i0 = __ldg(indices + 3 * (size_t)tri);
  h.i1 = __ldg(indices + 3 * (size_t)tri + 1);
  h.i2 = __ldg(indices + 3 * (size_t)tri + 2);
  const float3 v0 = make_float3(__ldg(vertices + 3 * (size_t)h.i0), __ldg(vertices + 3 * (size_t)h.i0 + 1),
                                __ldg(vertices + 3 * (size_t)h.i0 + 2));
  const float3 v1 = make_float3(__ldg(vertices + 3 * (size_t)h.i1), __ldg(vertices + 3 * (size_t)h.i1 + 1),
                                __ldg(vertices + 3 * (size_t)h.i1 + 2));
  const float3 v2 = make_float3(__ldg(vertices + 3 * (size_t)h.i2), __ldg(vertices + 3 * (size_t)h.i2 + 1),
                                __ldg(vertices + 3 * (size_t)h.i2 + 2));
  const ff3 E1 = ff3_sub(v1, v0), E2 = ff3_sub(v2, v0), S = ff3_sub(ir.o, v0);
  const float* m = p.tlas_data[inst].transform_inv;
  const float3 dobj = make_float3(d_world.x * __ldg(m + 0) + d_world.y * __ldg(m + 4) + d_world.z * __ldg(m + 8),
                                  d_world.x * __ldg(m + 1) + d_world.y * __ldg(m + 5) + d_world.z * __ldg(m + 9),
                                  d_world.x * __ldg(m + 2) + d_world.y * __ldg(m + 6) + d_world.z * __ldg(m + 10));
  const ff3 ND = ff3_of(make_float3(-dobj.x, -dobj.y, -dobj.z));
  const ff3 C12 = ff3_cross(E1, E2);
  const ff det = ff3_dot(ND, C12);
  const ff du = ff3_dot(ND, ff3_cross(S, E2));
  const ff dv = ff3_dot(ND, ff3_cross(E1, S));
  // distance along the unnormalised object-space direction (t = det[s, e1, e2] / det M)
  h.t_unnorm = ff_div(ff3_dot(S, C12), det);
  h.uf = ff_div_ff(du, det);
  h.vf = ff_div_ff(dv, det);
  // w0 = 1 - u - v without the cancellation near the edge v1-v2 (w0 -> 0),
  // where f32 would leave it with a large relative error
  h.wf = ff_div_ff(ff_add(det, ff_neg(ff_add(du, dv))), det);
  h.u = h.uf.hi + h.uf.lo;
  h.v = h.vf.hi + h.vf.lo;
  h.w0 = h.wf.hi + h.wf.lo;
  h.det = det;
  h.c12 = C12;
  h.b1 = ff3_cross(E2, ND);
  h.b2 = ff3_cross(ND, E1);
  return h;
}

__device__ __forceinline__ HitGeom hit_vertices(const TraceParams& p, const uint32_t* __restrict__ indices,
                                                const float* __restrict__ vertices, const RayCtx& R,
                                                const InstanceRay& ir) {
  return hit_vertices_at(p, indices, vertices, __ldg(p.redirect + R.best.k), R.best.inst, R.d, ir);
}

// lambda = M^{-T} (0, gu, gv) = (gu b1 + gv b2) / det, with the cofactors and
// determinant of the float-float solve: a ray that grazes the triangle makes
// det a small difference of large products, which f32 would lose. lambda does
// not depend on the length of d (numerator and det scale alike).
__device__ __forceinline__ float3 adjoint_lambda(const HitGeom& h, float gu, float gv) {
  const ff GU{gu, 0.f}, GV{gv, 0.f};
  return make_float3(ff_div(ff_add(ff_mul(GU, h.b1.x), ff_mul(GV, h.b2.x)), h.det),
                     ff_div(ff_add(ff_mul(GU, h.b1.y), ff_mul(GV, h.b2.y)), h.det),
                     ff_div(ff_add(ff_mul(GU, h.b1.z), ff_mul(GV, h.b2.z)), h.det));
}

// value - target with the interpolation (w0 a0 + u a1 + v a2) in float-float:
// the residual, which scales every gradient of the ray, keeps its relative
// accuracy when the interpolated value is close to the target. *value gets the
// interpolated value rounded to f32.
__device__ __forceinline__ float residual(const HitGeom& h, float a0, float a1, float a2, float target, float* value) {
  const ff v = ff_add(ff_add(ff_mul(h.wf, ff{a0, 0.f}), ff_mul(h.uf, ff{a1, 0.f})), ff_mul(h.vf, ff{a2, 0.f}));
  *value = v.hi + v.lo;
  const ff d = ff_add(v, ff{-target, 0.f});
  return d.hi + d.lo;
}

template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) attr_forward_kernel(TraceParams p, AdjointParams a) {
  RDN_TRAVERSAL_STACK(LOCAL);
  __shared__ double block_sum[4];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float loss = 0.0f;
  if (i < a.count) {
    const float4* rp = a.rays + 2 * (size_t)i;
    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
    RayCtx R;
    R.o = make_float3(r0.x, r0.y, r0.z);
    R.tmin = r0.w;
    R.d = make_float3(r1.x, r1.y, r1.z);
    R.tmax = r1.w;
    R.cull_mask = 0xFFu;
    R.ray_flags = 0u;
    bool bad;
    traverse_ray<MODE, false, BuiltinAnyHit, WT>(p, R, a.tlas_uniform, stack_ptr, stack_stride, bad);
    float value = 0.0f;
    if (R.best.have) {
      const InstanceRay ir = to_instance(p.tlas_data + R.best.inst, R.o, R.d, 0u);
      const HitGeom h = hit_vertices(p, a.indices, a.vertices, R, ir);
      const float diff = residual(h, __ldg(a.attributes + h.i0), __ldg(a.attributes + h.i1),
                                  __ldg(a.attributes + h.i2), a.targets ? __ldg(a.targets + i) : 0.0f, &value);
      loss = diff * diff;
    }
    if (a.hit_tri) a.hit_tri[i] = R.best.have ? __ldg(p.redirect + R.best.k) : INVALID_NEXT;
    if (a.hit_inst) a.hit_inst[i] = R.best.have ? R.best.inst : INVALID_NEXT;
    if (a.ray_value) a.ray_value[i] = value;
    if (a.ray_loss) a.ray_loss[i] = loss;
  }
  if (a.loss_sum) {
    double s = loss;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) block_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (uint32_t w = 0; w < (blockDim.x + 31) / 32; w++) t += block_sum[w];
      atomicAdd(a.loss_sum, t);
    }
  }
}

template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) attr_adjoint_kernel(TraceParams p, AdjointParams a) {
  RDN_TRAVERSAL_STACK(LOCAL);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.count) return;
  const float4* rp = a.rays + 2 * (size_t)i;
  const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
  RayCtx R;
  R.o = make_float3(r0.x, r0.y, r0.z);
  R.tmin = r0.w;
  R.d = make_float3(r1.x, r1.y, r1.z);
  R.tmax = r1.w;
  R.cull_mask = 0xFFu;
  R.ray_flags = 0u;
  bool bad;
  traverse_ray<MODE, false, BuiltinAnyHit, WT>(p, R, a.tlas_uniform, stack_ptr, stack_stride, bad);
  float3 go = make_float3(0.f, 0.f, 0.f), gd = go;
  if (R.best.have) {
    const InstanceRay ir = to_instance(p.tlas_data + R.best.inst, R.o, R.d, 0u);
    const HitGeom h = hit_vertices(p, a.indices, a.vertices, R, ir);
    const float a0 = __ldg(a.attributes + h.i0), a1 = __ldg(a.attributes + h.i1), a2 = __ldg(a.attributes + h.i2);
    float value;
    const float target = a.targets ? __ldg(a.targets + i) : 0.0f;
    const float r = 2.0f * residual(h, a0, a1, a2, target, &value) * a.grad_scale;
    const float gu = r * (a1 - a0), gv = r * (a2 - a0);
    const float3 lam = adjoint_lambda(h, gu, gv);
    float4* g = reinterpret_cast<float4*>(a.grad_vertices);
    atomicAdd(g + h.i0, make_float4(-h.w0 * lam.x, -h.w0 * lam.y, -h.w0 * lam.z, r * h.w0));
    atomicAdd(g + h.i1, make_float4(-h.u * lam.x, -h.u * lam.y, -h.u * lam.z, r * h.u));
    atomicAdd(g + h.i2, make_float4(-h.v * lam.x, -h.v * lam.y, -h.v * lam.z, r * h.v));
    // d(o + s d)/dd = s: s the hit's parameter along the object-space direction
    go = lam;
    gd = make_float3(h.t_unnorm * lam.x, h.t_unnorm * lam.y, h.t_unnorm * lam.z);
  }
  if (a.grad_ray_origin) {
    a.grad_ray_origin[3 * (size_t)i] = go.x;
    a.grad_ray_origin[3 * (size_t)i + 1] = go.y;
    a.grad_ray_origin[3 * (size_t)i + 2] = go.z;
  }
  if (a.grad_ray_direction) {
    a.grad_ray_direction[3 * (size_t)i] = gd.x;
    a.grad_ray_direction[3 * (size_t)i + 1] = gd.y;
    a.grad_ray_direction[3 * (size_t)i + 2] = gd.z;
  }
}

// lambda = M^{-T} (0, gu, gv) with M = [-d | e1 | e2] (object space),
// scattered to the three corners; returns lambda.
__device__ __forceinline__ float3 scatter_vertex_grads(const HitGeom& h, const InstanceRay& ir, float r, float gu,
                                                       float gv, float* grad_vertices) {
  const float3 lam = adjoint_lambda(h, gu, gv);
  float4* g = reinterpret_cast<float4*>(grad_vertices);
  atomicAdd(g + h.i0, make_float4(-h.w0 * lam.x, -h.w0 * lam.y, -h.w0 * lam.z, r * h.w0));
  atomicAdd(g + h.i1, make_float4(-h.u * lam.x, -h.u * lam.y, -h.u * lam.z, r * h.u));
  atomicAdd(g + h.i2, make_float4(-h.v * lam.x, -h.v * lam.y, -h.v * lam.z, r * h.v));
  return lam;
}

// Persistent warps over paths; ADJOINT selects the gradient pass.
template <int MODE, bool ADJOINT, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) attr_path_kernel(TraceParams p, PathAdjointParams a) {
  RDN_TRAVERSAL_STACK(LOCAL);
  __shared__ double block_sum[4];
  const uint32_t lane = threadIdx.x & 31u;
  double loss_acc = 0.0;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(a.work_counter, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= a.count) break;
    const uint32_t i = base + lane;
    if (i >= a.count) continue;
    const float4* rp = a.rays + 2 * (size_t)i;
    float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
    const uint32_t tlas = a.tlas_idx ? __ldg(a.tlas_idx + i) : a.tlas_uniform;
    bool alive = true;
    for (uint32_t k = 0; k < a.segments; k++) {
      const size_t seg = (size_t)i * a.segments + k;
      float value = 0.0f;
      uint32_t tri_out = INVALID_NEXT, inst_out = INVALID_NEXT;
      if (alive) {
        if (a.seg_rays) {
          a.seg_rays[2 * seg] = r0;
          a.seg_rays[2 * seg + 1] = r1;
        }
        RayCtx R;
        R.o = make_float3(r0.x, r0.y, r0.z);
        R.tmin = r0.w;
        R.d = make_float3(r1.x, r1.y, r1.z);
        R.tmax = r1.w;
        R.cull_mask = 0xFFu;
        R.ray_flags = 0u;
        bool bad;
        traverse_ray<MODE, false, BuiltinAnyHit, WT>(p, R, tlas, stack_ptr, stack_stride, bad);
        if (!R.best.have) {
          alive = false;
          if (!ADJOINT && a.targets) {
            const float t = __ldg(a.targets + seg);  // value 0 against the target
            loss_acc += (double)(t * t);
          }
        } else {
          const InstanceRay ir = to_instance(p.tlas_data + R.best.inst, R.o, R.d, 0u);
          const HitGeom h = hit_vertices(p, a.indices, a.vertices, R, ir);
          tri_out = __ldg(p.redirect + R.best.k);
          inst_out = R.best.inst;
          const float a0 = __ldg(a.attributes + h.i0), a1 = __ldg(a.attributes + h.i1),
                      a2 = __ldg(a.attributes + h.i2);
          const float target = a.targets ? __ldg(a.targets + seg) : 0.0f;
          const float diff = residual(h, a0, a1, a2, target, &value);
          if (ADJOINT) {
            const float r = 2.0f * diff * a.grad_scale;
            scatter_vertex_grads(h, ir, r, r * (a1 - a0), r * (a2 - a0), a.grad_vertices);
          } else {
            loss_acc += (double)(diff * diff);
          }
          if (k + 1 < a.segments) {
            uint32_t st = xxhash32(i, k, a.seed);
            const float s0 = sample_next(st);
            const float s1 = sample_next(st);
            const float3 hp = R.o + R.d * R.best.t;
            const float3 nf = facing_normal(p, R.best.k, R.best.inst, R.d);
            const float3 org = offset_ray_hit(hp, nf);
            const float3 dir = cosine_sample_in_dir(nf, s0, s1);
            r0 = make_float4(org.x, org.y, org.z, 1.1920929e-7f);
            r1 = make_float4(dir.x, dir.y, dir.z, 3.40282347e+38f);
          }
        }
      } else if (!ADJOINT && a.targets) {
        // a missed segment has value 0 against its target
        const float t = __ldg(a.targets + seg);
        loss_acc += (double)(t * t);
      }
      if (!ADJOINT && a.values) a.values[seg] = value;
      if (!ADJOINT && a.seg_tri) a.seg_tri[seg] = tri_out;
      if (!ADJOINT && a.seg_inst) a.seg_inst[seg] = inst_out;
    }
  }
  if (!ADJOINT && a.loss_sum) {
    double s = loss_acc;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) block_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (uint32_t w = 0; w < (blockDim.x + 31) / 32; w++) t += block_sum[w];
      atomicAdd(a.loss_sum, t);
    }
  }
}

// Adjoint from the forward's record (a tape): every recorded segment is
// differentiated at the triangle and instance the forward hit, with no second
// traversal. One thread per segment; misses were recorded as ~0 and add
// nothing. The forward and the adjoint therefore always agree on visibility,
// also where two triangles meet the ray at exactly the same distance.
__device__ __forceinline__ void recorded_segment(const TraceParams& p, const PathAdjointParams& a, size_t seg,
                                                 uint32_t tri) {
  const uint32_t inst = __ldg(a.seg_inst + seg);
  const float4 r0 = __ldg(a.seg_rays + 2 * seg), r1 = __ldg(a.seg_rays + 2 * seg + 1);
  const float3 o = make_float3(r0.x, r0.y, r0.z), d = make_float3(r1.x, r1.y, r1.z);
  const InstanceRay ir = to_instance(p.tlas_data + inst, o, d, 0u);
  const HitGeom h = hit_vertices_at(p, a.indices, a.vertices, tri, inst, d, ir);
  const float a0 = __ldg(a.attributes + h.i0), a1 = __ldg(a.attributes + h.i1), a2 = __ldg(a.attributes + h.i2);
  float value;
  const float target = a.targets ? __ldg(a.targets + seg) : 0.0f;
  const float r = 2.0f * residual(h, a0, a1, a2, target, &value) * a.grad_scale;
  scatter_vertex_grads(h, ir, r, r * (a1 - a0), r * (a2 - a0), a.grad_vertices);
}

// One warp per 32-segment window of the record at a time; the live segments
// (a hit was recorded) are gathered in a per-warp shared-memory queue and
// differentiated 32 at a time, so that misses do not leave lanes idle.
__global__ void __launch_bounds__(256) attr_path_recorded_kernel(TraceParams p, PathAdjointParams a) {
  __shared__ uint32_t queue[8][64];
  __shared__ uint32_t queue_tri[8][64];
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const uint32_t lanes_below = (1u << lane) - 1u;
  const size_t total = (size_t)a.count * a.segments;
  const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
  const size_t first = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  // a queued entry is (window number << 5 | lane); segment = first*32 + window*warps*32 + lane
  auto segment_of = [&](uint32_t e) { return first * 32 + (size_t)(e >> 5) * warps * 32 + (e & 31u); };
  uint32_t held = 0, window = 0;
  for (size_t w0 = first * 32; w0 < total; w0 += warps * 32, window++) {
    const size_t seg = w0 + lane;
    const uint32_t tri = seg < total ? __ldg(a.seg_tri + seg) : INVALID_NEXT;
    const uint32_t live = __ballot_sync(0xffffffffu, tri != INVALID_NEXT);
    if (tri != INVALID_NEXT) {
      const uint32_t slot = held + __popc(live & lanes_below);
      queue[wib][slot] = (window << 5) | lane;
      queue_tri[wib][slot] = tri;
    }
    held += __popc(live);
    __syncwarp();
    if (held >= 32) {
      recorded_segment(p, a, segment_of(queue[wib][lane]), queue_tri[wib][lane]);
      __syncwarp();
      held -= 32;
      if (lane < held) {
        queue[wib][lane] = queue[wib][32 + lane];
        queue_tri[wib][lane] = queue_tri[wib][32 + lane];
      }
      __syncwarp();
    }
  }
  if (lane < held) recorded_segment(p, a, segment_of(queue[wib][lane]), queue_tri[wib][lane]);
}

__global__ void __launch_bounds__(256) attr_recorded_adjoint_kernel(TraceParams p, AdjointParams a) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.count; i += gridDim.x * blockDim.x) {
    const uint32_t tri = __ldg(a.hit_tri + i);
    float3 go = make_float3(0.f, 0.f, 0.f), gd = go;
    if (tri != INVALID_NEXT) {
      const uint32_t inst = __ldg(a.hit_inst + i);
      const float4 r0 = __ldg(a.rays + 2 * (size_t)i), r1 = __ldg(a.rays + 2 * (size_t)i + 1);
      const float3 o = make_float3(r0.x, r0.y, r0.z), d = make_float3(r1.x, r1.y, r1.z);
      const InstanceRay ir = to_instance(p.tlas_data + inst, o, d, 0u);
      const HitGeom h = hit_vertices_at(p, a.indices, a.vertices, tri, inst, d, ir);
      const float a0 = __ldg(a.attributes + h.i0), a1 = __ldg(a.attributes + h.i1), a2 = __ldg(a.attributes + h.i2);
      float value;
      const float target = a.targets ? __ldg(a.targets + i) : 0.0f;
      const float r = 2.0f * residual(h, a0, a1, a2, target, &value) * a.grad_scale;
      const float3 lam = scatter_vertex_grads(h, ir, r, r * (a1 - a0), r * (a2 - a0), a.grad_vertices);
      // d(o + s d)/dd = s: s the hit's parameter along the object-space direction
      go = lam;
      gd = make_float3(h.t_unnorm * lam.x, h.t_unnorm * lam.y, h.t_unnorm * lam.z);
    }
    if (a.grad_ray_origin) {
      a.grad_ray_origin[3 * (size_t)i] = go.x;
      a.grad_ray_origin[3 * (size_t)i + 1] = go.y;
      a.grad_ray_origin[3 * (size_t)i + 2] = go.z;
    }
    if (a.grad_ray_direction) {
      a.grad_ray_direction[3 * (size_t)i] = gd.x;
      a.grad_ray_direction[3 * (size_t)i + 1] = gd.y;
      a.grad_ray_direction[3 * (size_t)i + 2] = gd.z;
    }
  }
}

// ---- differentiable hit query (rdn_hit_diff_*) ------------------------------
// Forward: per ray the closest hit's parameter t along the given direction (the
// reference's reported distance, traverse_cpu.rs:157), the barycentrics (u, v)
// and the interpolated attribute w0 a0 + u a1 + v a2, all re-solved on the hit
// triangle in float-float. Adjoint: with the caller's upstream gradients
// G = (dL/dt, dL/du, dL/dv, dL/dvalue) per ray,
//   gu = G.u + G.value (a1 - a0), gv = G.v + G.value (a2 - a0),
//   lambda = M^{-T} (G.t, gu, gv) = (G.t (e1 x e2) + gu (e2 x -d) + gv (-d x e1)) / det M,
//   dL/dv_k = -w_k lambda, dL/da_k = G.value w_k (object space, accumulated),
//   dL/do = L^T lambda, dL/dd = t L^T lambda (world space; L = the 3x3 of the
//   instance's inverse transform, which maps world to object directions).
__device__ __forceinline__ float3 to_world_covector(const DeviceInstance* inst, float3 g) {
  const float* m = inst->transform_inv;
  return make_float3(__ldg(m + 0) * g.x + __ldg(m + 1) * g.y + __ldg(m + 2) * g.z,
                     __ldg(m + 4) * g.x + __ldg(m + 5) * g.y + __ldg(m + 6) * g.z,
                     __ldg(m + 8) * g.x + __ldg(m + 9) * g.y + __ldg(m + 10) * g.z);
}

__device__ __forceinline__ void hit_diff_store(const AdjointParams& a, uint32_t i, float4 out, uint32_t tri,
                                               uint32_t inst) {
  if (a.hit_out) a.hit_out[i] = out;
  if (a.hit_tri) a.hit_tri[i] = tri;
  if (a.hit_inst) a.hit_inst[i] = inst;
}

template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) hit_diff_forward_kernel(TraceParams p, AdjointParams a) {
  RDN_TRAVERSAL_STACK(LOCAL);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.count) return;
  const float4 r0 = __ldg(a.rays + 2 * (size_t)i), r1 = __ldg(a.rays + 2 * (size_t)i + 1);
  RayCtx R;
  R.o = make_float3(r0.x, r0.y, r0.z);
  R.tmin = r0.w;
  R.d = make_float3(r1.x, r1.y, r1.z);
  R.tmax = r1.w;
  R.cull_mask = 0xFFu;
  R.ray_flags = 0u;
  bool bad;
  traverse_ray<MODE, false, BuiltinAnyHit, WT>(p, R, a.tlas_uniform, stack_ptr, stack_stride, bad);
  if (!R.best.have) {
    hit_diff_store(a, i, make_float4(R.tmax, 0.0f, 0.0f, 0.0f), INVALID_NEXT, INVALID_NEXT);
    return;
  }
  const InstanceRay ir = to_instance(p.tlas_data + R.best.inst, R.o, R.d, 0u);
  const HitGeom h = hit_vertices(p, a.indices, a.vertices, R, ir);
  float value = 0.0f;
  if (a.attributes)
    residual(h, __ldg(a.attributes + h.i0), __ldg(a.attributes + h.i1), __ldg(a.attributes + h.i2), 0.0f, &value);
  hit_diff_store(a, i, make_float4(h.t_unnorm, h.u, h.v, value), __ldg(p.redirect + R.best.k), R.best.inst);
}

// The adjoint of one ray's hit (triangle `tri` of instance `inst`).
__device__ __forceinline__ void hit_diff_scatter(const TraceParams& p, const AdjointParams& a, uint32_t i,
                                                 uint32_t tri, uint32_t inst, float3 o, float3 d, float3& go,
                                                 float3& gd) {
  const InstanceRay ir = to_instance(p.tlas_data + inst, o, d, 0u);
  const HitGeom h = hit_vertices_at(p, a.indices, a.vertices, tri, inst, d, ir);
  const float4 G = __ldg(a.grad_hit + i);
  float gu = G.y, gv = G.z;
  if (a.attributes) {
    const float a0 = __ldg(a.attributes + h.i0), a1 = __ldg(a.attributes + h.i1), a2 = __ldg(a.attributes + h.i2);
    gu = gu + G.w * (a1 - a0);
    gv = gv + G.w * (a2 - a0);
  }
  const ff GT{G.x, 0.f}, GU{gu, 0.f}, GV{gv, 0.f};
  const float3 lam = make_float3(
      ff_div(ff_add(ff_add(ff_mul(GT, h.c12.x), ff_mul(GU, h.b1.x)), ff_mul(GV, h.b2.x)), h.det),
      ff_div(ff_add(ff_add(ff_mul(GT, h.c12.y), ff_mul(GU, h.b1.y)), ff_mul(GV, h.b2.y)), h.det),
      ff_div(ff_add(ff_add(ff_mul(GT, h.c12.z), ff_mul(GU, h.b1.z)), ff_mul(GV, h.b2.z)), h.det));
  float4* g = reinterpret_cast<float4*>(a.grad_vertices);
  const float gval = a.attributes ? G.w : 0.0f;
  atomicAdd(g + h.i0, make_float4(-h.w0 * lam.x, -h.w0 * lam.y, -h.w0 * lam.z, gval * h.w0));
  atomicAdd(g + h.i1, make_float4(-h.u * lam.x, -h.u * lam.y, -h.u * lam.z, gval * h.u));
  atomicAdd(g + h.i2, make_float4(-h.v * lam.x, -h.v * lam.y, -h.v * lam.z, gval * h.v));
  go = to_world_covector(p.tlas_data + inst, lam);
  gd = make_float3(h.t_unnorm * go.x, h.t_unnorm * go.y, h.t_unnorm * go.z);
}

__device__ __forceinline__ void hit_diff_store_ray_grads(const AdjointParams& a, uint32_t i, float3 go, float3 gd) {
  if (a.grad_ray_origin) {
    a.grad_ray_origin[3 * (size_t)i] = go.x;
    a.grad_ray_origin[3 * (size_t)i + 1] = go.y;
    a.grad_ray_origin[3 * (size_t)i + 2] = go.z;
  }
  if (a.grad_ray_direction) {
    a.grad_ray_direction[3 * (size_t)i] = gd.x;
    a.grad_ray_direction[3 * (size_t)i + 1] = gd.y;
    a.grad_ray_direction[3 * (size_t)i + 2] = gd.z;
  }
}

template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) hit_diff_adjoint_kernel(TraceParams p, AdjointParams a) {
  RDN_TRAVERSAL_STACK(LOCAL);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.count) return;
  const float4 r0 = __ldg(a.rays + 2 * (size_t)i), r1 = __ldg(a.rays + 2 * (size_t)i + 1);
  RayCtx R;
  R.o = make_float3(r0.x, r0.y, r0.z);
  R.tmin = r0.w;
  R.d = make_float3(r1.x, r1.y, r1.z);
  R.tmax = r1.w;
  R.cull_mask = 0xFFu;
  R.ray_flags = 0u;
  bool bad;
  traverse_ray<MODE, false, BuiltinAnyHit, WT>(p, R, a.tlas_uniform, stack_ptr, stack_stride, bad);
  float3 go = make_float3(0.f, 0.f, 0.f), gd = go;
  if (R.best.have) hit_diff_scatter(p, a, i, __ldg(p.redirect + R.best.k), R.best.inst, R.o, R.d, go, gd);
  hit_diff_store_ray_grads(a, i, go, gd);
}

__global__ void __launch_bounds__(256) hit_diff_recorded_adjoint_kernel(TraceParams p, AdjointParams a) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.count; i += gridDim.x * blockDim.x) {
    const uint32_t tri = __ldg(a.hit_tri + i);
    float3 go = make_float3(0.f, 0.f, 0.f), gd = go;
    if (tri != INVALID_NEXT) {
      const float4 r0 = __ldg(a.rays + 2 * (size_t)i), r1 = __ldg(a.rays + 2 * (size_t)i + 1);
      hit_diff_scatter(p, a, i, tri, __ldg(a.hit_inst + i), make_float3(r0.x, r0.y, r0.z),
                       make_float3(r1.x, r1.y, r1.z), go, gd);
    }
    hit_diff_store_ray_grads(a, i, go, gd);
  }
}

inline uint32_t recorded_grid(size_t items, int sm_count) {
  const size_t need = (items + 255) / 256;
  const size_t cap = (size_t)(sm_count > 0 ? sm_count : 1) * 16;
  return (uint32_t)(need < cap ? (need ? need : 1) : cap);
}

template <int MODE, bool LOCAL, bool WT>
cudaError_t launch_attr_paths_variant(const TraceParams& p, const PathAdjointParams& a, bool adjoint, uint32_t block,
                                      int sm_count, cudaStream_t stream) {
  static std::atomic<uint64_t> done[2] = {};
  const void* fn = adjoint ? (const void*)attr_path_kernel<MODE, true, LOCAL, WT>
                           : (const void*)attr_path_kernel<MODE, false, LOCAL, WT>;
  cudaError_t e = raise_smem_limit(done[adjoint], {fn});
  if (e != cudaSuccess) return e;
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)block, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t grid = (uint32_t)(sm_count * per_sm);
  const uint32_t need = (a.count + block - 1) / block;
  if (grid > need) grid = need;
  e = cudaMemsetAsync(a.work_counter, 0, 4, stream);
  if (e != cudaSuccess) return e;
  if (adjoint) attr_path_kernel<MODE, true, LOCAL, WT><<<grid, block, smem, stream>>>(p, a);
  else attr_path_kernel<MODE, false, LOCAL, WT><<<grid, block, smem, stream>>>(p, a);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_attr_paths_mode(const TraceParams& p, const PathAdjointParams& a, bool adjoint, uint32_t block,
                                   int sm_count, cudaStream_t stream) {
  const bool local = MODE != MODE_THREADED && p.local_stack;
  if (p.watertight)
    return local ? launch_attr_paths_variant<MODE, MODE != MODE_THREADED, true>(p, a, adjoint, block, sm_count, stream)
                 : launch_attr_paths_variant<MODE, false, true>(p, a, adjoint, block, sm_count, stream);
  return local ? launch_attr_paths_variant<MODE, MODE != MODE_THREADED, false>(p, a, adjoint, block, sm_count, stream)
               : launch_attr_paths_variant<MODE, false, false>(p, a, adjoint, block, sm_count, stream);
}

template <int MODE, bool LOCAL, bool WT>
cudaError_t launch_attr_variant(const TraceParams& p, const AdjointParams& a, bool adjoint, uint32_t block,
                                cudaStream_t stream) {
  static std::atomic<uint64_t> done[2] = {};
  const cudaError_t e = raise_smem_limit(done[adjoint], {adjoint ? (const void*)attr_adjoint_kernel<MODE, LOCAL, WT>
                                                                 : (const void*)attr_forward_kernel<MODE, LOCAL, WT>});
  if (e != cudaSuccess) return e;
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  const uint32_t grid = (a.count + block - 1) / block;
  if (adjoint) attr_adjoint_kernel<MODE, LOCAL, WT><<<grid, block, smem, stream>>>(p, a);
  else attr_forward_kernel<MODE, LOCAL, WT><<<grid, block, smem, stream>>>(p, a);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_attr_mode(const TraceParams& p, const AdjointParams& a, bool adjoint, uint32_t block,
                             cudaStream_t stream) {
  const bool local = MODE != MODE_THREADED && p.local_stack;
  if (p.watertight)
    return local ? launch_attr_variant<MODE, MODE != MODE_THREADED, true>(p, a, adjoint, block, stream)
                 : launch_attr_variant<MODE, false, true>(p, a, adjoint, block, stream);
  return local ? launch_attr_variant<MODE, MODE != MODE_THREADED, false>(p, a, adjoint, block, stream)
               : launch_attr_variant<MODE, false, false>(p, a, adjoint, block, stream);
}

template <int MODE, bool LOCAL, bool WT>
cudaError_t launch_hit_diff_variant(const TraceParams& p, const AdjointParams& a, bool adjoint, uint32_t block,
                                    cudaStream_t stream) {
  static std::atomic<uint64_t> done[2] = {};
  const cudaError_t e = raise_smem_limit(done[adjoint], {adjoint ? (const void*)hit_diff_adjoint_kernel<MODE, LOCAL, WT>
                                                                 : (const void*)hit_diff_forward_kernel<MODE, LOCAL, WT>});
  if (e != cudaSuccess) return e;
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  const uint32_t grid = (a.count + block - 1) / block;
  if (adjoint) hit_diff_adjoint_kernel<MODE, LOCAL, WT><<<grid, block, smem, stream>>>(p, a);
  else hit_diff_forward_kernel<MODE, LOCAL, WT><<<grid, block, smem, stream>>>(p, a);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_hit_diff_mode(const TraceParams& p, const AdjointParams& a, bool adjoint, uint32_t block,
                                 cudaStream_t stream) {
  const bool local = MODE != MODE_THREADED && p.local_stack;
  if (p.watertight)
    return local ? launch_hit_diff_variant<MODE, MODE != MODE_THREADED, true>(p, a, adjoint, block, stream)
                 : launch_hit_diff_variant<MODE, false, true>(p, a, adjoint, block, stream);
  return local ? launch_hit_diff_variant<MODE, MODE != MODE_THREADED, false>(p, a, adjoint, block, stream)
               : launch_hit_diff_variant<MODE, false, false>(p, a, adjoint, block, stream);
}

cudaError_t launch_attr(const TraceParams& p, const AdjointParams& a, int mode, bool adjoint, uint32_t block,
                        cudaStream_t stream) {
  if (a.count == 0) return cudaSuccess;
  if (block == 0) block = 64;
  if (mode == MODE_WIDE4) return launch_attr_mode<MODE_WIDE4>(p, a, adjoint, block, stream);
  if (mode == MODE_BINARY) return launch_attr_mode<MODE_BINARY>(p, a, adjoint, block, stream);
  return launch_attr_mode<MODE_THREADED>(p, a, adjoint, block, stream);
}

}  // namespace

cudaError_t launch_attr_paths(const TraceParams& p, const PathAdjointParams& a, int mode, bool adjoint,
                              uint32_t block, int sm_count, cudaStream_t stream) {
  if (a.count == 0) return cudaSuccess;
  if (adjoint && a.from_record) {
    attr_path_recorded_kernel<<<recorded_grid((size_t)a.count * a.segments, sm_count), 256, 0, stream>>>(p, a);
    return cudaGetLastError();
  }
  if (block == 0) block = 64;
  if (mode == MODE_WIDE4) return launch_attr_paths_mode<MODE_WIDE4>(p, a, adjoint, block, sm_count, stream);
  if (mode == MODE_BINARY) return launch_attr_paths_mode<MODE_BINARY>(p, a, adjoint, block, sm_count, stream);
  return launch_attr_paths_mode<MODE_THREADED>(p, a, adjoint, block, sm_count, stream);
}

cudaError_t launch_attr_forward(const TraceParams& p, const AdjointParams& a, int mode, uint32_t block,
                                cudaStream_t stream) {
  return launch_attr(p, a, mode, false, block, stream);
}

cudaError_t launch_attr_adjoint(const TraceParams& p, const AdjointParams& a, int mode, uint32_t block,
                                int sm_count, cudaStream_t stream) {
  if (a.from_record) {
    if (a.count == 0) return cudaSuccess;
    attr_recorded_adjoint_kernel<<<recorded_grid(a.count, sm_count), 256, 0, stream>>>(p, a);
    return cudaGetLastError();
  }
  return launch_attr(p, a, mode, true, block, stream);
}

cudaError_t launch_hit_diff(const TraceParams& p, const AdjointParams& a, int mode, bool adjoint, uint32_t block,
                            int sm_count, cudaStream_t stream) {
  if (a.count == 0) return cudaSuccess;
  if (adjoint && a.from_record) {
    hit_diff_recorded_adjoint_kernel<<<recorded_grid(a.count, sm_count), 256, 0, stream>>>(p, a);
    return cudaGetLastError();
  }
  if (block == 0) block = 64;
  if (mode == MODE_WIDE4) return launch_hit_diff_mode<MODE_WIDE4>(p, a, adjoint, block, stream);
  if (mode == MODE_BINARY) return launch_hit_diff_mode<MODE_BINARY>(p, a, adjoint, block, stream);
  return launch_hit_diff_mode<MODE_THREADED>(p, a, adjoint, block, stream);
}

}  // namespace rdn
